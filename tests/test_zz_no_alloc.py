"""Allocation-free MLP prediction (rewl_mlp_predict_noalloc).

Collected last on purpose: it must give the same answers after every other
test has run in the process as it does alone in a fresh one.  The caller (this
test) owns the device input/output buffers; the entry point itself allocates
nothing and keeps its activations in a static device array.
"""
import numpy as np
import pytest


def _features(n, seed):
    rng = np.random.default_rng(seed)
    X = np.empty((n, 7), dtype=np.float32)
    X[:, 0] = rng.uniform(-2.0, 2.0, n)
    X[:, 1] = 1.0 / rng.choice([8, 16, 32, 64], n)
    X[:, 2] = 1.0
    X[:, 3] = rng.choice([0.0, 0.5], n)
    X[:, 4] = rng.uniform(0.0, 1.0, n)
    X[:, 5] = rng.uniform(-2.0, 0.0, n)
    X[:, 6] = X[:, 5] + rng.uniform(0.1, 2.0, n)
    return X


@pytest.mark.gpu
def test_noalloc_predict_matches_predict_twice_in_a_row(engine_lib):
    import torch
    from rewl_simulator_gb300.mlp import MLP
    m = MLP(hidden=256, layers=4, seed=11)
    try:
        for n in (1000, 4096):                       # ragged rows, then the maximum
            X = _features(n, seed=n)
            ref = m.predict(X)                      # the allocating entry point
            Xd = torch.from_numpy(X).cuda()
            stream = torch.cuda.current_stream()
            outs = [torch.full((n,), float("nan"), dtype=torch.float32, device="cuda") for _ in range(3)]
            # a first call outside the measurement: the driver may load kernel code lazily
            m.predict_noalloc(Xd.data_ptr(), n, 7, outs.pop().data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            for yd in outs:                         # two calls in a row on one stream
                m.predict_noalloc(Xd.data_ptr(), n, 7, yd.data_ptr(), stream.cuda_stream)
            stream.synchronize()
            # the device's free memory (driver view) is unchanged: nothing was allocated
            assert torch.cuda.mem_get_info()[0] == free0
            for yd in outs:
                got = yd.cpu().numpy()
                assert np.isfinite(got).all()
                # same kernels and the same bf16 staging: agreement to float rounding
                np.testing.assert_allclose(got, ref, rtol=0, atol=1e-6)
    finally:
        m.close()


@pytest.mark.gpu
def test_noalloc_predict_rejects_oversize_requests(engine_lib):
    import torch
    from rewl_simulator_gb300.engine import REWLError
    from rewl_simulator_gb300.mlp import MLP
    m = MLP(hidden=256, layers=2, seed=3)
    try:
        Xd = torch.zeros((4097, 7), dtype=torch.float32, device="cuda")
        yd = torch.zeros(4097, dtype=torch.float32, device="cuda")
        with pytest.raises(REWLError) as e:
            m.predict_noalloc(Xd.data_ptr(), 4097, 7, yd.data_ptr(), 0)
        assert e.value.code == 22 and "4096" in str(e.value)
        with pytest.raises(REWLError):
            m.predict_noalloc(Xd.data_ptr(), 10, 65, yd.data_ptr(), 0)
    finally:
        m.close()
    wide = MLP(hidden=320, layers=1, seed=3)
    try:
        with pytest.raises(REWLError) as e:
            wide.predict_noalloc(Xd.data_ptr(), 64, 7, yd.data_ptr(), 0)
        assert e.value.code == 22 and "256" in str(e.value)
    finally:
        wide.close()
