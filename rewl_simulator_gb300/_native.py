"""Build and load the native engine library (librewl_gb300.so, in-tree).

The library is compiled with nvcc for sm_103a only.  Loading never falls back
to anything else: if the library is missing or cannot be loaded, an error is
raised.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
LIB = PKG / "librewl_gb300.so"
SOURCES = [CSRC / "engine.cu", CSRC / "mlp.cu", CSRC / "thermo.cu"]
DEPS = SOURCES + [CSRC / "rng.cuh", CSRC / "models.cuh", INCLUDE / "rewl.h"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the REWL engine needs the CUDA toolkit to build")
    return cand


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the engine into rewl_simulator_gb300/librewl_gb300.so.

    Each translation unit is compiled concurrently, then linked.
    """
    if LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in DEPS)
        if LIB.stat().st_mtime >= newest:
            return LIB
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    common = [nvcc(), *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", str(INCLUDE)]
    if verbose:
        common.append("-Xptxas=-v")
    procs, objs = [], []
    for src in SOURCES:
        obj = objdir / f"{src.stem}.{os.getpid()}.o"
        objs.append(obj)
        procs.append(subprocess.Popen(common + ["-c", str(src), "-o", str(obj)]))
    rcs = [p.wait() for p in procs]
    if any(rcs):
        raise RuntimeError(f"nvcc failed for {[str(s) for s, r in zip(SOURCES, rcs) if r]}")
    tmp = LIB.with_name(f".librewl_gb300.{os.getpid()}.so")
    subprocess.run([nvcc(), *ARCH_FLAGS, "-shared", *map(str, objs), "-o", str(tmp)], check=True)
    for o in objs:
        o.unlink()
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        raise RuntimeError(f"{LIB} is missing: build it with rewl_simulator_gb300.build() "
                           "(the engine has no CPU fallback)")
    lib = C.CDLL(str(LIB))
    _declare(lib)
    _lib = lib
    return lib


def _declare(L: C.CDLL) -> None:
    vp, i32, i64, u64, sz, dp = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_size_t, C.c_void_p
    L.rewl_last_error_string.restype = C.c_char_p
    L.rewl_mlp_last_error_string.restype = C.c_char_p
    L.rewl_thermo_last_error_string.restype = C.c_char_p
    sigs = {
        "rewl_create": [vp, vp],
        "rewl_destroy": [vp],
        "rewl_num_walkers": [vp, vp],
        "rewl_walker_info": [vp, i32, vp, vp, vp],
        "rewl_window_info": [vp, i32, i32, vp, vp, vp],
        "rewl_import_dofs": [vp, i32, vp, i32],
        "rewl_import_disorder": [vp, i32, vp],
        "rewl_generate_fields": [u64, C.c_double, i32, i64, vp],
        "rewl_set_logdos": [vp, i32, i32, vp],
        "rewl_set_lnf": [vp, i32, i32, C.c_double],
        "rewl_set_uniform_stream": [vp, i32, vp, sz],
        "rewl_run_sweeps": [vp, i64],
        "rewl_exchange": [vp],
        "rewl_check_flat": [vp, vp],
        "rewl_reset_histograms": [vp, i32, i32, i32],
        "rewl_run_cycles": [vp, i64, i64, vp],
        "rewl_get_status": [vp, vp],
        "rewl_export_walker": [vp, i32, vp, vp, vp, vp, vp],
        "rewl_export_observables": [vp, i32, vp],
        "rewl_thermodynamics": [vp, vp, vp, i32, i32, i32, C.c_double, C.c_double, C.c_double, i32, i32, i32, vp, vp],
        "rewl_autotune": [vp, i32],
        "rewl_launch_shapes": [vp, vp, vp],
        "rewl_nonlinear_observables": [i32, i32, vp, i32, i32, vp, C.c_double, vp],
        "rewl_global_observables": [vp, i32, vp, vp],
        "rewl_write_microcanonical": [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, i32, i32, C.c_double, vp, vp, vp],
        "rewl_write_self_averaged": [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, i32, i32, vp, vp],
        "rewl_write_nonlinear": [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, i32, i32, vp, vp],
        "rewl_write_outputs": [vp, i32, C.c_char_p, C.c_char_p, C.c_char_p, C.c_double, C.c_double, i32],
        "rewl_export_window_observables": [vp, i32, i32, vp],
        "rewl_export_window_logdos": [vp, i32, i32, vp],
        "rewl_export_window_mask": [vp, i32, i32, vp],
        "rewl_window_state": [vp, i32, i32, vp, vp],
        "rewl_global_logdos": [vp, i32, i32, vp, vp, vp],
        "rewl_concatenate_windows": [i32, vp, vp, vp, i32, vp, C.c_double, i64, i32, i32, vp, vp, vp, vp],
        "rewl_sweep_kernel_time": [vp, vp, vp],
        "rewl_get_stream": [vp, vp],
        "rewl_snapshot_size": [vp, vp],
        "rewl_snapshot": [vp, vp, sz],
        "rewl_restore": [vp, vp, sz],
        "rewl_mlp_create": [i32, i32, i32, u64, vp],
        "rewl_mlp_destroy": [vp],
        "rewl_mlp_num_params": [vp, vp],
        "rewl_mlp_layout": [vp, vp, i32],
        "rewl_mlp_get_params": [vp, i32, vp, i64],
        "rewl_mlp_set_params": [vp, vp, i64],
        "rewl_mlp_predict": [vp, vp, i32, i32, vp],
        "rewl_mlp_gradient": [vp, vp, vp, i32, i32, vp],
        "rewl_mlp_set_data": [vp, vp, vp, i32, i32],
        "rewl_mlp_train": [vp, i32, i32, C.c_float, vp],
        "rewl_mlp_launches": [vp, vp],
        "rewl_mlp_predict_noalloc": [vp, vp, i32, i32, vp, vp],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
