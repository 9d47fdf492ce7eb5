"""ctypes bindings and build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

``build()`` compiles oracle/rewl_oracle.cpp (the C++ restatement of the
reference's REWL hot path) into oracle/_build/liboracle.so with plain g++.
``Oracle`` drives it; ``RefWalker`` drives the reference's own walker compiled
by oracle/build_ref.py (only where the reference sources are present).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

MODEL_ISING, MODEL_AT = 0, 1
SEM_REFERENCE, SEM_ENGINE = 0, 1
FLAT_MIN_OVER_MEAN, FLAT_MAX_MIN_RATIO, FLAT_ALL_VISITED = 0, 1, 2
MASK_STATIC, MASK_VISITED = 0, 1


def build(force: bool = False) -> Path:
    src = HERE / "rewl_oracle.cpp"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                    "-pthread", str(src), "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


class orc_config(C.Structure):
    _fields_ = [("model", C.c_int32), ("L", C.c_int32), ("J", C.c_double), ("K", C.c_double),
                ("escale_bits", C.c_int32), ("nwin", C.c_int32), ("R", C.c_int32),
                ("sweeps_per_exchange", C.c_int32), ("sweeps_per_check", C.c_int32),
                ("emin", C.c_double), ("emax", C.c_double), ("bw", C.c_double), ("overlap", C.c_double),
                ("lnf0", C.c_double), ("lnf_final", C.c_double), ("flat_param", C.c_double),
                ("flat_mode", C.c_int32), ("mask_mode", C.c_int32), ("one_over_t", C.c_int32),
                ("reduce_logdos", C.c_int32), ("observables", C.c_int32), ("semantics", C.c_int32),
                ("init_mode", C.c_int32), ("nthreads", C.c_int32), ("seed", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        L = _lib
        vp, u64, i64, sz, dp = C.c_void_p, C.c_uint64, C.c_int64, C.c_size_t, C.c_void_p
        L.orc_philox_word.restype = C.c_uint32
        L.orc_philox_word.argtypes = [u64, C.c_uint32, u64, C.c_uint32, C.c_uint32]
        L.orc_philox4x32_10.argtypes = [vp, vp, vp]
        L.orc_neglog_u32.restype = C.c_float
        L.orc_neglog_u32.argtypes = [C.c_uint32]
        L.orc_accept_threshold.restype = i64
        L.orc_accept_threshold.argtypes = [C.c_float]
        L.orc_mt64_uniforms.argtypes = [u64, sz, vp]
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(orc_config), vp, vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_num_walkers.restype = sz
        L.orc_num_walkers.argtypes = [vp]
        L.orc_window.argtypes = [vp, C.c_int, vp, vp, vp]
        L.orc_run_sweeps.argtypes = [vp, u64]
        L.orc_exchange.argtypes = [vp]
        for f in ("orc_flat_step", "orc_cycle", "orc_all_done"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [vp]
        L.orc_done_flags.argtypes = [vp, vp]
        L.orc_total_sweeps.restype = u64
        L.orc_total_sweeps.argtypes = [vp]
        L.orc_exchange_stats.argtypes = [vp, vp]
        L.orc_walker_state.argtypes = [vp, sz, vp]
        L.orc_walker_dofs.argtypes = [vp, sz, vp]
        L.orc_walker_tables.argtypes = [vp, sz, vp, vp, vp]
        L.orc_walker_obs.argtypes = [vp, sz, vp]
        L.orc_walker_lnf.restype = C.c_double
        L.orc_walker_lnf.argtypes = [vp, sz]
        L.orc_walker_draws.restype = u64
        L.orc_walker_draws.argtypes = [vp, sz]
        L.orc_walker_set_dofs.argtypes = [vp, sz, vp, C.c_int]
        L.orc_walker_set_lnf.argtypes = [vp, sz, C.c_double]
        L.orc_walker_set_logdos.argtypes = [vp, sz, vp]
        L.orc_walker_reset.argtypes = [vp, sz, C.c_int]
        L.orc_walker_set_rng.argtypes = [vp, sz, u64, u64]
        L.orc_window_logdos.argtypes = [vp, C.c_int, vp]
        L.orc_window_mask.restype = C.c_int
        L.orc_window_mask.argtypes = [vp, C.c_int, vp]
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def philox_word(seed: int, uid: int, ctr: int, stream: int, w3: int = 0) -> int:
    return lib().orc_philox_word(seed, uid, ctr, stream, w3)


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def neglog_u32(x: int) -> float:
    return lib().orc_neglog_u32(x)


def accept_threshold(thr: float) -> int:
    return lib().orc_accept_threshold(thr)


def mt64_uniforms(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float64)
    lib().orc_mt64_uniforms(seed, n, _p(out))
    return out


@dataclass
class Config:
    model: int = MODEL_ISING
    L: int = 4
    J: float = 1.0
    K: float = 0.5
    escale_bits: int = 0
    nwin: int = 1
    R: int = 1
    sweeps_per_exchange: int = 1000
    sweeps_per_check: int = 1000
    emin: float = -32.0
    emax: float = 36.0
    bw: float = 4.0
    overlap: float = 0.75
    lnf0: float = 1.0
    lnf_final: float = 1e-6
    flat_param: float = 0.8
    flat_mode: int = FLAT_MIN_OVER_MEAN
    mask_mode: int = MASK_STATIC
    one_over_t: int = 0
    reduce_logdos: int = 1
    observables: int = 0
    semantics: int = SEM_ENGINE
    init_mode: int = 0
    nthreads: int = 1
    seed: int = 1

    def to_c(self) -> orc_config:
        c = orc_config()
        for name, _ in orc_config._fields_:
            setattr(c, name, getattr(self, name))
        return c


class Oracle:
    """One REWL simulation in the C++ oracle."""

    def __init__(self, cfg: Config, fields: np.ndarray | None = None, init_dofs: np.ndarray | None = None):
        self.cfg = cfg
        self._c = cfg.to_c()
        self._fields = None if fields is None else np.ascontiguousarray(fields, dtype=np.float64)
        self._dofs = None if init_dofs is None else np.ascontiguousarray(init_dofs, dtype=np.float64)
        h = lib().orc_create(C.byref(self._c), None if self._fields is None else _p(self._fields),
                             None if self._dofs is None else _p(self._dofs))
        if not h:
            raise RuntimeError("oracle: a walker could not reach its window")
        self.h = h
        self.N = cfg.L * cfg.L
        self.ndof = self.N * (2 if cfg.model == MODEL_AT else 1)
        self.windows = []
        for w in range(cfg.nwin):
            mm = np.zeros(2)
            lo = np.zeros(1, dtype=np.int64)
            nb = np.zeros(1, dtype=np.uint64)
            lib().orc_window(h, w, _p(mm), _p(lo), _p(nb))
            self.windows.append((float(mm[0]), float(mm[1]), int(lo[0]), int(nb[0])))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_walkers(self) -> int:
        return self.cfg.nwin * self.cfg.R

    def run_sweeps(self, n: int):
        lib().orc_run_sweeps(self.h, n)

    def exchange(self):
        lib().orc_exchange(self.h)

    def flat_step(self) -> int:
        return lib().orc_flat_step(self.h)

    def cycle(self) -> int:
        return lib().orc_cycle(self.h)

    def all_done(self) -> bool:
        return bool(lib().orc_all_done(self.h))

    def done_flags(self) -> np.ndarray:
        out = np.zeros(self.cfg.nwin, dtype=np.int32)
        lib().orc_done_flags(self.h, _p(out))
        return out

    def total_sweeps(self) -> int:
        return lib().orc_total_sweeps(self.h)

    def exchange_stats(self):
        out = np.zeros(2, dtype=np.uint64)
        lib().orc_exchange_stats(self.h, _p(out))
        return int(out[0]), int(out[1])

    def state(self, slot: int) -> np.ndarray:
        out = np.zeros(5)
        lib().orc_walker_state(self.h, slot, _p(out))
        return out[:2] if self.cfg.model == MODEL_ISING else out

    def dofs(self, slot: int) -> np.ndarray:
        out = np.zeros(self.ndof, dtype=np.int8)
        lib().orc_walker_dofs(self.h, slot, _p(out))
        return out

    def nbins(self, slot: int) -> int:
        return self.windows[slot // self.cfg.R][3]

    def tables(self, slot: int):
        nb = self.nbins(slot)
        c = np.zeros(nb, dtype=np.uint64)
        g = np.zeros(nb)
        v = np.zeros(nb, dtype=np.uint64)
        lib().orc_walker_tables(self.h, slot, _p(c), _p(g), _p(v))
        return c, g, v

    def obs(self, slot: int) -> np.ndarray:
        corr = self.cfg.observables == 2
        k = (5 if corr else 4) if self.cfg.model == MODEL_ISING else (17 if corr else 13)
        out = np.zeros(self.nbins(slot) * k)
        lib().orc_walker_obs(self.h, slot, _p(out))
        return out.reshape(-1, k)

    def lnf(self, slot: int) -> float:
        return lib().orc_walker_lnf(self.h, slot)

    def draws(self, slot: int) -> int:
        return lib().orc_walker_draws(self.h, slot)

    def set_dofs(self, slot: int, dofs_ref_layout: np.ndarray, which: int = 0):
        d = np.ascontiguousarray(dofs_ref_layout, dtype=np.float64)
        lib().orc_walker_set_dofs(self.h, slot, _p(d), which)

    def set_lnf(self, slot: int, lnf: float):
        lib().orc_walker_set_lnf(self.h, slot, lnf)

    def set_logdos(self, slot: int, g: np.ndarray):
        g = np.ascontiguousarray(g, dtype=np.float64)
        lib().orc_walker_set_logdos(self.h, slot, _p(g))

    def reset(self, slot: int, reduce: bool = True):
        lib().orc_walker_reset(self.h, slot, int(reduce))

    def set_rng(self, slot: int, seed: int, skip: int):
        lib().orc_walker_set_rng(self.h, slot, seed, skip)

    def window_logdos(self, w: int) -> np.ndarray:
        out = np.zeros(self.windows[w][3])
        lib().orc_window_logdos(self.h, w, _p(out))
        return out

    def window_mask(self, w: int) -> np.ndarray:
        out = np.zeros(self.windows[w][3], dtype=np.uint8)
        lib().orc_window_mask(self.h, w, _p(out))
        return out.astype(bool)


class RefWalker:
    """The reference's own REWL_Walker, compiled by oracle/build_ref.py."""

    def __init__(self, so_path: Path, wmin: float, wmax: float, bw: float, nbins: int, seed: int):
        self.lib = C.CDLL(str(so_path))
        L = self.lib
        vp = C.c_void_p
        L.ref_walker_new.restype = vp
        L.ref_walker_new.argtypes = [C.c_double, C.c_double, C.c_double, C.c_size_t, C.c_uint32]
        for f in ("ref_walker_free", "ref_walker_adjust", "ref_walker_reset"):
            getattr(L, f).argtypes = [vp]
        L.ref_walker_import_dofs.argtypes = [vp, vp]
        L.ref_walker_import_disorder.argtypes = [vp, vp]
        L.ref_walker_walk.argtypes = [vp, C.c_size_t]
        L.ref_walker_set_incrementer.argtypes = [vp, C.c_double]
        L.ref_walker_flatness.restype = C.c_float
        L.ref_walker_flatness.argtypes = [vp]
        L.ref_walker_get_state.argtypes = [vp, vp]
        L.ref_walker_get_dofs.argtypes = [vp, vp]
        L.ref_walker_get_hist.argtypes = [vp, vp, vp]
        L.ref_walker_get_obs.argtypes = [vp, vp]
        L.ref_num_dof.restype = C.c_size_t
        L.ref_num_obs.restype = C.c_size_t
        L.ref_model_id.restype = C.c_int
        L.ref_uniforms.argtypes = [C.c_uint64, C.c_size_t, vp]
        L.ref_random_fields.argtypes = [C.c_uint64, C.c_double, C.c_int, C.c_size_t, vp]
        L.ref_concatenate.argtypes = [C.c_size_t, vp, vp, vp, C.c_size_t, vp, C.c_double, C.c_size_t, C.c_double,
                                      vp, vp, vp, vp]
        L.ref_glazier.argtypes = [C.c_double, C.c_double, C.c_double, C.c_size_t, C.c_size_t, C.c_double, vp, vp, vp]
        L.ref_normalize_logdos.argtypes = [C.c_double, C.c_size_t, C.c_double, C.c_size_t, vp]
        self.nbins = nbins
        self.ndof = L.ref_num_dof()
        self.nobs = L.ref_num_obs()
        self.model = L.ref_model_id()
        self.h = L.ref_walker_new(wmin, wmax, bw, nbins, seed)

    def __del__(self):
        try:
            self.lib.ref_walker_free(self.h)
        except Exception:
            pass

    def import_dofs(self, d):
        d = np.ascontiguousarray(d, dtype=np.float64)
        self.lib.ref_walker_import_dofs(self.h, _p(d))

    def import_disorder(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        self.lib.ref_walker_import_disorder(self.h, _p(f))

    def adjust(self):
        self.lib.ref_walker_adjust(self.h)

    def walk(self, n):
        self.lib.ref_walker_walk(self.h, n)

    def set_lnf(self, x):
        self.lib.ref_walker_set_incrementer(self.h, x)

    def reset(self):
        self.lib.ref_walker_reset(self.h)

    def flatness(self):
        return self.lib.ref_walker_flatness(self.h)

    def state(self):
        out = np.zeros(5)
        self.lib.ref_walker_get_state(self.h, _p(out))
        return out[:2] if self.model == 0 else out

    def dofs(self):
        out = np.zeros(self.ndof)
        self.lib.ref_walker_get_dofs(self.h, _p(out))
        return out

    def hist(self):
        c = np.zeros(self.nbins, dtype=np.uint64)
        g = np.zeros(self.nbins)
        self.lib.ref_walker_get_hist(self.h, _p(c), _p(g))
        return c, g

    def obs(self):
        out = np.zeros(self.nbins * self.nobs)
        self.lib.ref_walker_get_obs(self.h, _p(out))
        return out.reshape(self.nbins, self.nobs)

    def glazier(self, gmin, gmax, bw, nwin, rpw, overlap):
        mins = np.zeros(nwin)
        maxs = np.zeros(nwin)
        nb = np.zeros(nwin, dtype=np.uint64)
        self.lib.ref_glazier(gmin, gmax, bw, nwin, rpw, overlap, _p(mins), _p(maxs), _p(nb))
        return mins, maxs, nb
