"""The C-ABI library: exported symbols and host-side descriptor validation.

No kernel runs here; rewl_create validates a descriptor on the host before it
touches a device, so malformed batches are rejected with REWL_EINVAL anywhere,
and a valid batch on a machine without a GPU fails with REWL_EDEVICE.
"""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "rewl.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(rewl_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(engine_lib):
    lib = C.CDLL(str(engine_lib.LIBRARY_PATH))
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _create(engine_lib, **overrides):
    from rewl_simulator_gb300 import engine as E
    ins = dict(model=0, L=8, J=1.0, K=0.0, energy_min=-128.0, energy_max=132.0, bin_width=4.0,
               num_windows=2, replicas_per_window=2, window_overlap=0.75, init_mode=0, seed=1)
    bat = dict(sweeps_per_exchange=10, sweeps_per_check=20, flatness_mode=0, flatness_param=0.8,
               lnf_initial=1.0, lnf_final=1e-6, mask_mode=0, one_over_t=0, reduce_logdos=1, rng_mode=0,
               device=0, warps_per_block=0, walkers_per_warp=0)
    for k, v in overrides.items():
        (ins if k in ins else bat)[k] = v
    lib = engine_lib.load_library()
    d = E._InstanceDesc()
    for k, v in ins.items():
        setattr(d, k, v)
    d.fields = None
    arr = (E._InstanceDesc * 1)(d)
    b = E._BatchDesc()
    b.num_instances = 1
    for k, v in bat.items():
        setattr(b, k, v)
    b.instances = C.cast(arr, C.c_void_p)
    h = C.c_void_p()
    rc = lib.rewl_create(C.byref(b), C.byref(h))
    msg = lib.rewl_last_error_string().decode()
    if rc == 0:
        lib.rewl_destroy(h)
    return rc, msg


BAD = [
    dict(L=1), dict(L=200), dict(model=7), dict(num_windows=0), dict(replicas_per_window=65),
    dict(window_overlap=1.0), dict(bin_width=3.0), dict(J=0.5), dict(energy_max=-200.0),
    dict(sweeps_per_check=15), dict(sweeps_per_exchange=0), dict(lnf_initial=0.0), dict(flatness_mode=5),
    dict(mask_mode=3), dict(rng_mode=9), dict(warps_per_block=3), dict(walkers_per_warp=3), dict(init_mode=2),
    dict(persistent=2), dict(persistent=1, rng_mode=1), dict(persistent=1, walkers_per_warp=2), dict(lnf_initial=65.0),
    dict(num_windows=40, window_overlap=0.0, energy_min=-128.0, energy_max=-120.0),
]


@pytest.mark.parametrize("bad", BAD, ids=[str(b) for b in BAD])
def test_bad_descriptor_rejected_on_host(engine_lib, bad):
    rc, msg = _create(engine_lib, **bad)
    assert rc == 22, (rc, msg)
    assert msg


def test_valid_descriptor_needs_a_device(engine_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present: covered by the gpu tests")
    rc, msg = _create(engine_lib)
    assert rc == 1001, (rc, msg)
    assert "device" in msg.lower()


def test_product_path_fails_loudly_without_library(tmp_path, monkeypatch):
    from rewl_simulator_gb300 import _native
    monkeypatch.setattr(_native, "LIB", tmp_path / "missing.so")
    monkeypatch.setattr(_native, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _native.load()
