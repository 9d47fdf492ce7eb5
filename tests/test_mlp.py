"""Warm-start MLP: the FP64 restatement is pinned by finite differences (CPU), the GPU's BF16
tcgen05 forward/backward is checked against it and against the mma.sync kernels, GPU training
fits a smooth ln g(E)/N surface, and training is bit-reproducible for a seed."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import mlp_ref


def _random_params(hidden, layers, rng):
    layout, n = mlp_ref.make_layout(hidden, layers)
    p = np.zeros(n, dtype=np.float64)
    for l, (din, dout, wo, bo) in enumerate(layout):
        real_in = 7 if l == 0 else hidden
        real_out = 1 if l == layers else hidden
        W = np.zeros((dout, din))
        W[:real_out, :real_in] = rng.uniform(-1, 1, (real_out, real_in)) / np.sqrt(real_in)
        p[wo:wo + din * dout] = W.ravel()
        b = np.zeros(dout)
        b[:real_out] = rng.uniform(-0.1, 0.1, real_out)
        p[bo:bo + dout] = b
    return layout, p


def test_fp64_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    layout, p = _random_params(64, 2, rng)
    X = rng.normal(size=(16, 7))
    y = rng.normal(size=16)
    loss, g = mlp_ref.forward_backward(p, layout, X, y, round_bf16=False)
    idx = np.nonzero(p)[0]
    for k in rng.choice(idx, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp, _ = mlp_ref.forward_backward(pp, layout, X, y, round_bf16=False)
        lm, _ = mlp_ref.forward_backward(pm, layout, X, y, round_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_bf16_rounding_helper():
    x = np.array([1.0, 1.00390625, 1.001953125, 3.14159, -2.5e-3, 0.0])
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                  # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties go to even
    assert r[2] == 1.0
    assert r[3] == 3.140625
    assert r[5] == 0.0


@pytest.mark.gpu
def test_gpu_gradient_matches_fp64(engine_lib):
    from rewl_simulator_gb300.mlp import MLP
    rng = np.random.default_rng(1)
    m = MLP(hidden=256, layers=4, seed=5)
    layout = m.layout
    p = m.params().astype(np.float64)
    X = rng.uniform(-1, 1, (256, 7)).astype(np.float32)
    y = rng.uniform(0, 0.7, 256).astype(np.float32)
    loss = m.gradient(X, y)
    g_gpu = m.grads().astype(np.float64)
    loss_ref, g_ref = mlp_ref.forward_backward(p, layout, X.astype(np.float64), y.astype(np.float64))
    assert abs(loss - loss_ref) <= 2e-3 * abs(loss_ref) + 1e-6
    for l, (din, dout, wo, bo) in enumerate(layout):
        for off, size in ((wo, din * dout), (bo, dout)):
            a, b = g_gpu[off:off + size], g_ref[off:off + size]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert rel < 2e-2, (l, off, rel)
    yp = m.predict(X)
    np.testing.assert_allclose(yp, mlp_ref.predict(p, layout, X.astype(np.float64)), rtol=0, atol=5e-3)
    m.close()


@pytest.mark.gpu
def test_gpu_training_fits_exact_lng(engine_lib):
    from rewl_simulator_gb300.mlp import MLP, features
    Xs, ys = [], []
    for L in (8, 16, 32):
        z = np.load(GOLDEN / f"exact_ising_L{L}.npz")
        N = L * L
        Xs.append(features(z["E"], L, 1.0, 0.0, 0.0, -2.0 * N, 2.0 * N))
        ys.append(z["lng"] / N)
    X = np.concatenate(Xs)
    y = np.concatenate(ys).astype(np.float32)
    m = MLP(hidden=256, layers=4, seed=3)
    m.set_data(X, y)
    losses = m.train(600, batch=1024, lr=1e-3)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.05 * losses[:5].mean(), (losses[:5], losses[-20:])
    pred = m.predict(X)
    assert np.abs(pred - y).max() < 0.05
    m.close()


_GRAD_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from rewl_simulator_gb300.mlp import MLP
rng = np.random.default_rng(4)
m = MLP(hidden=256, layers=4, seed=9)
X = rng.uniform(-1, 1, (1024, 7)).astype(np.float32)
y = rng.uniform(0, 0.7, 1024).astype(np.float32)
loss = m.gradient(X, y)
np.savez(sys.argv[2], loss=loss, grads=m.grads(), pred=m.predict(X[:200]))
m.close()
"""


@pytest.mark.gpu
def test_gpu_tcgen05_gemm_matches_mma_sync(engine_lib, tmp_path):
    """The tcgen05 GEMMs (default) against the mma.sync ones on one forward + backward with a
    split-K weight gradient (batch 1024) and a prediction on 200 rows (a partial 128-row tile):
    same BF16 operands and FP32 accumulation, so only the summation order differs."""
    import os
    import subprocess
    import sys
    from conftest import ROOT
    out = {}
    for kind in ("tcgen05", "mma_sync"):
        env = dict(os.environ)
        env.pop("REWL_MLP_GEMM", None)
        if kind == "mma_sync":
            env["REWL_MLP_GEMM"] = "mma_sync"
        f = tmp_path / f"{kind}.npz"
        subprocess.run([sys.executable, "-c", _GRAD_SCRIPT, str(ROOT), str(f)], env=env, check=True, timeout=300)
        out[kind] = np.load(f)
    a, b = out["tcgen05"], out["mma_sync"]
    assert abs(float(a["loss"]) - float(b["loss"])) <= 1e-3 * abs(float(b["loss"]))
    ga, gb = a["grads"].astype(np.float64), b["grads"].astype(np.float64)
    assert np.linalg.norm(ga - gb) <= 1e-2 * np.linalg.norm(gb), np.linalg.norm(ga - gb) / np.linalg.norm(gb)
    np.testing.assert_allclose(a["pred"], b["pred"], rtol=0, atol=2e-3)


@pytest.mark.gpu
def test_gpu_training_is_reproducible(engine_lib):
    """The same seed and data give bit-identical parameters and losses: split-K weight gradients,
    bias column sums and the loss are summed in a fixed order (no atomics)."""
    from rewl_simulator_gb300.mlp import MLP
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, (6000, 7)).astype(np.float32)
    y = rng.uniform(0, 0.7, 6000).astype(np.float32)
    for batch in (1024, 4096):
        runs = []
        for _ in range(2):
            m = MLP(hidden=256, layers=4, seed=13)
            m.set_data(X, y)
            losses = m.train(30, batch=batch)
            runs.append((m.params(), np.asarray(losses)))
            m.close()
        assert np.array_equal(runs[0][0], runs[1][0]), batch
        assert np.array_equal(runs[0][1], runs[1][1]), batch


@pytest.mark.gpu
def test_gpu_training_resumes_across_calls(engine_lib):
    """A training call replays one captured step as a CUDA graph, with the step counter (batch
    sampling, Adam's bias corrections) kept on the device: 20 steps in one call and 7 + 13 in two
    calls give bit-identical parameters and losses, and the launch counter counts every step."""
    from rewl_simulator_gb300.mlp import MLP
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, (3000, 7)).astype(np.float32)
    y = rng.uniform(0, 0.7, 3000).astype(np.float32)
    out = []
    for split in ((20,), (7, 13)):
        m = MLP(hidden=128, layers=3, seed=5)
        m.set_data(X, y)
        n0 = m.launches()
        losses = np.concatenate([np.asarray(m.train(k, batch=1024)) for k in split])
        out.append((m.params(), losses, m.launches() - n0))
        m.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and out[0][2] % 20 == 0
    assert np.all(np.isfinite(out[0][1])) and out[0][1][-1] < out[0][1][0]
