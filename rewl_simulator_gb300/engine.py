"""Python mirror of the REWL engine's C ABI (include/rewl.h).

``Engine`` wraps one ``rewl_engine``: a batch of REWL instances advanced together
on one GPU.  Method names follow the reference's simulation interface where one
exists (REWL_simulation::simulate, REWL_Walker::wang_landau_walk, the
Hamiltonian's import_DoFs / import_disorder, rewl_histograms::export_logdos).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _native

REWL_OK = 0
REWL_EINVAL = 22
REWL_ENOMEM = 12
REWL_ETIMEDOUT = 110
REWL_EDEVICE = 1001
REWL_EBOUNDS = 1002
REWL_ESTATE = 1003

MODEL_ISING2D = 0
MODEL_ASHKIN_TELLER2D = 1
FLAT_MIN_OVER_MEAN = 0
FLAT_MAX_MIN_RATIO = 1
FLAT_ALL_VISITED = 2
MASK_STATIC = 0
MASK_VISITED = 1
RNG_PHILOX = 0
RNG_REPLAY = 1
DISORDER_UNIFORM = 0        # REWL_DISORDER_*: the reference's disorder_distribution
DISORDER_GAUSSIAN = 1
MATCH_DERIVATIVE = 0        # REWL_MATCH_*: where concatenate_windows splices neighbouring windows
MATCH_REFERENCE = 1


class REWLError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class _InstanceDesc(C.Structure):
    _fields_ = [("model", C.c_int32), ("L", C.c_int32), ("J", C.c_double), ("K", C.c_double),
                ("fields", C.c_void_p), ("energy_min", C.c_double), ("energy_max", C.c_double),
                ("bin_width", C.c_double), ("num_windows", C.c_int32), ("replicas_per_window", C.c_int32),
                ("window_overlap", C.c_double), ("init_mode", C.c_int32), ("reserved", C.c_int32),
                ("seed", C.c_uint64)]


class _BatchDesc(C.Structure):
    _fields_ = [("num_instances", C.c_int32), ("sweeps_per_exchange", C.c_int32),
                ("sweeps_per_check", C.c_int32), ("flatness_mode", C.c_int32), ("flatness_param", C.c_double),
                ("lnf_initial", C.c_double), ("lnf_final", C.c_double), ("mask_mode", C.c_int32),
                ("one_over_t", C.c_int32), ("reduce_logdos", C.c_int32), ("rng_mode", C.c_int32),
                ("device", C.c_int32), ("warps_per_block", C.c_int32), ("walkers_per_warp", C.c_int32),
                ("observables", C.c_int32), ("graphs", C.c_int32), ("autotune", C.c_int32),
                ("persistent", C.c_int32),
                ("instances", C.c_void_p)]


class _Status(C.Structure):
    _fields_ = [("sweeps", C.c_int64), ("cycles", C.c_int64), ("flat_events", C.c_int64),
                ("windows_done", C.c_int64), ("windows_total", C.c_int64),
                ("exchanges_attempted", C.c_int64), ("exchanges_accepted", C.c_int64),
                ("attempted_flips", C.c_int64), ("kernel_launches", C.c_int64), ("all_done", C.c_int32),
                ("device_error", C.c_int32)]


@dataclass
class Instance:
    """One REWL problem: model, lattice, couplings, energy windows, seed."""
    model: int = MODEL_ISING2D
    L: int = 16
    J: float = 1.0
    K: float = 0.0
    fields: Optional[np.ndarray] = None
    energy_min: float = -512.0
    energy_max: float = 516.0
    bin_width: float = 4.0
    num_windows: int = 4
    replicas_per_window: int = 1
    window_overlap: float = 0.75
    init_mode: int = 0
    seed: int = 1

    @property
    def N(self) -> int:
        return self.L * self.L

    @property
    def ndof(self) -> int:
        return self.N * (2 if self.model == MODEL_ASHKIN_TELLER2D else 1)


@dataclass
class Batch:
    instances: Sequence[Instance] = field(default_factory=list)
    sweeps_per_exchange: int = 1000
    sweeps_per_check: int = 1000
    flatness_mode: int = FLAT_MIN_OVER_MEAN
    flatness_param: float = 0.8
    lnf_initial: float = 1.0
    lnf_final: float = 1e-6
    mask_mode: int = MASK_STATIC
    one_over_t: int = 0
    reduce_logdos: int = 1
    rng_mode: int = RNG_PHILOX
    device: int = 0
    warps_per_block: int = 0
    walkers_per_warp: int = 0
    observables: int = 0            # 1: per-bin moments; 2: also the G(q_min) correlators
    graphs: int = 0                 # 1: replay each check interval as one captured CUDA graph
    autotune: int = 0               # 1: time the launch groups' kernel shapes before the first cycle
    persistent: int = 0             # 1: all launch groups in one persistent work-stealing launch per phase


@dataclass
class Status:
    sweeps: int
    cycles: int
    flat_events: int
    windows_done: int
    windows_total: int
    exchanges_attempted: int
    exchanges_accepted: int
    attempted_flips: int
    kernel_launches: int
    all_done: bool
    device_error: int


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def instance_key(seed: int) -> int:
    """The Philox key the engine derives from an instance's seed: SplitMix64's output function
    (Steele, Lea, Flood, OOPSLA 2014).  Walker u of the instance is keyed (key_lo ^ u, key_hi)."""
    m = (1 << 64) - 1
    z = (int(seed) + 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


def generate_fields(seed: int, strength: float, num_sites: int, distribution: int = DISORDER_GAUSSIAN) -> np.ndarray:
    """Random fields drawn as the reference's Disorder::generate_random_field draws them
    (src/Hamiltonians/Disorder/random_fields.hpp:41-75), from `seed` instead of the clock:
    Gaussian with standard deviation `strength`, or uniform on [-2 strength, 2 strength].
    Host only; the result goes to Instance.fields (which rounds it to multiples of 2^-20)."""
    lib = _native.load()
    out = np.zeros(int(num_sites), dtype=np.float64)
    rc = lib.rewl_generate_fields(int(seed), float(strength), int(distribution), int(num_sites), _p(out))
    if rc != 0:
        raise REWLError(rc, lib.rewl_last_error_string().decode())
    return out


def concatenate_windows(windows, states_per_site: float, system_size: int, half_spectrum: bool = False,
                        match: int = MATCH_DERIVATIVE):
    """Concatenate per-window tables and normalise, as the reference's post-processing does
    (concatenate_tables with multiple overlap, then normalize_logDoS); host only.
    windows: sequence of (E, lng) or (E, lng, obs) with ascending energies, valid levels only, and
    obs of shape (rows, K) averaged over each overlap as the reference averages observables.
    match=MATCH_REFERENCE reproduces the reference's compiled splice rule bit for bit.
    Returns (E, lng) or (E, lng, obs)."""
    lib = _native.load()
    Es = [np.ascontiguousarray(w[0], dtype=np.float64) for w in windows]
    Gs = [np.ascontiguousarray(w[1], dtype=np.float64) for w in windows]
    with_obs = all(len(w) > 2 for w in windows)
    Os = [np.ascontiguousarray(w[2], dtype=np.float64).reshape(len(w[0]), -1) for w in windows] if with_obs else []
    K = Os[0].shape[1] if with_obs else 0
    sizes = np.array([len(e) for e in Es], dtype=np.int32)
    E, G = np.concatenate(Es), np.concatenate(Gs)
    O = np.concatenate(Os) if with_obs else np.zeros(0)
    cap = C.c_int32(int(sizes.sum()))
    oe, og, oo = np.zeros(cap.value), np.zeros(cap.value), np.zeros(cap.value * K)
    rc = lib.rewl_concatenate_windows(len(Es), _p(sizes), _p(E), _p(G), K, _p(O) if K else None, float(states_per_site),
                                      int(system_size), int(bool(half_spectrum)), int(match), _p(oe), _p(og),
                                      _p(oo) if K else None, C.byref(cap))
    if rc != 0:
        raise REWLError(rc, lib.rewl_last_error_string().decode())
    n = cap.value
    if with_obs:
        return oe[:n].copy(), og[:n].copy(), oo[:n * K].reshape(n, K).copy()
    return oe[:n].copy(), og[:n].copy()


def obs_columns(model: int, observables: int) -> int:
    """Columns of an exported observables row: the averages and the count.  Ising |m|, m^2, m^4
    (+ G(q_min)); Ashkin-Teller 12 moments (+ a G(q_min) after each group of three)."""
    corr = observables == 2
    return (5 if corr else 4) if model == MODEL_ISING2D else (17 if corr else 13)


class Engine:
    """A batch of REWL instances on one GPU (wraps rewl_create / rewl_destroy)."""

    def __init__(self, batch: Batch):
        self.lib = _native.load()
        self.batch = batch
        n = len(batch.instances)
        self._inst = (_InstanceDesc * n)()
        self._fields = []
        for k, ins in enumerate(batch.instances):
            d = self._inst[k]
            d.model, d.L, d.J, d.K = ins.model, ins.L, ins.J, ins.K
            if ins.fields is not None:
                f = np.ascontiguousarray(ins.fields, dtype=np.float64)
                if f.shape != (ins.N,):
                    raise ValueError("fields must have L*L entries")
                self._fields.append(f)
                d.fields = f.ctypes.data
            else:
                d.fields = None
            d.energy_min, d.energy_max, d.bin_width = ins.energy_min, ins.energy_max, ins.bin_width
            d.num_windows, d.replicas_per_window, d.window_overlap = ins.num_windows, ins.replicas_per_window, ins.window_overlap
            d.init_mode, d.seed = ins.init_mode, ins.seed
        b = _BatchDesc()
        b.num_instances = n
        for name in ("sweeps_per_exchange", "sweeps_per_check", "flatness_mode", "flatness_param", "lnf_initial",
                     "lnf_final", "mask_mode", "one_over_t", "reduce_logdos", "rng_mode", "device",
                     "warps_per_block", "walkers_per_warp", "observables", "graphs", "autotune", "persistent"):
            setattr(b, name, getattr(batch, name))
        b.instances = C.cast(self._inst, C.c_void_p)
        self._desc = b
        h = C.c_void_p()
        self._check(self.lib.rewl_create(C.byref(b), C.byref(h)))
        self.h = h
        nw = C.c_int32()
        self._check(self.lib.rewl_num_walkers(self.h, C.byref(nw)))
        self.num_walkers = nw.value
        self.windows = []
        for k, ins in enumerate(batch.instances):
            ws = []
            for w in range(ins.num_windows):
                lo, hi, nb = C.c_double(), C.c_double(), C.c_int32()
                self._check(self.lib.rewl_window_info(self.h, k, w, C.byref(lo), C.byref(hi), C.byref(nb)))
                ws.append((lo.value, hi.value, nb.value))
            self.windows.append(ws)
        self._walker_inst = []
        for s in range(self.num_walkers):
            i, w, r = C.c_int32(), C.c_int32(), C.c_int32()
            self._check(self.lib.rewl_walker_info(self.h, s, C.byref(i), C.byref(w), C.byref(r)))
            self._walker_inst.append((i.value, w.value, r.value))

    # -- plumbing ---------------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc != REWL_OK:
            raise REWLError(rc, self.lib.rewl_last_error_string().decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.rewl_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def walker_info(self, walker: int):
        return self._walker_inst[walker]

    def walker_id(self, instance: int, window: int, replica: int) -> int:
        for s, t in enumerate(self._walker_inst):
            if t == (instance, window, replica):
                return s
        raise KeyError((instance, window, replica))

    # -- imports ------------------------------------------------------------------
    def import_dofs(self, walker: int, dofs: np.ndarray, flavour: int = 0) -> None:
        d = np.ascontiguousarray(dofs, dtype=np.int8)
        self._check(self.lib.rewl_import_dofs(self.h, walker, _p(d), flavour))

    def import_disorder(self, instance: int, fields: np.ndarray) -> None:
        f = np.ascontiguousarray(fields, dtype=np.float64)
        self._check(self.lib.rewl_import_disorder(self.h, instance, _p(f)))

    def set_logdos(self, instance: int, window: int, logdos: np.ndarray) -> None:
        g = np.ascontiguousarray(logdos, dtype=np.float64)
        self._check(self.lib.rewl_set_logdos(self.h, instance, window, _p(g)))

    def set_lnf(self, instance: int, window: int, lnf: float) -> None:
        self._check(self.lib.rewl_set_lnf(self.h, instance, window, lnf))

    def set_uniform_stream(self, walker: int, uniforms: np.ndarray) -> None:
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        self._check(self.lib.rewl_set_uniform_stream(self.h, walker, _p(u), u.size))

    # -- running ------------------------------------------------------------------
    def wang_landau_walk(self, num_sweeps: int) -> None:
        self._check(self.lib.rewl_run_sweeps(self.h, num_sweeps))

    run_sweeps = wang_landau_walk

    def replica_exchange_update(self) -> None:
        self._check(self.lib.rewl_exchange(self.h))

    def check_flat(self) -> int:
        n = C.c_int32()
        self._check(self.lib.rewl_check_flat(self.h, C.byref(n)))
        return n.value

    def reset_histograms(self, instance: int, window: int, reduce_logdos: bool = True) -> None:
        self._check(self.lib.rewl_reset_histograms(self.h, instance, window, int(reduce_logdos)))

    def run_cycles(self, num_cycles: int, timeout_ms: int = 0) -> Status:
        st = _Status()
        self._check(self.lib.rewl_run_cycles(self.h, num_cycles, timeout_ms, C.byref(st)))
        return self._status(st)

    def simulate(self, max_cycles: int = 1 << 40, timeout_ms: int = 0) -> Status:
        """Run until every window is done (REWL_simulation::simulate)."""
        return self.run_cycles(max_cycles, timeout_ms)

    def autotune(self, sweeps: int = 0) -> None:
        """Time each launch group's kernel shapes and keep the fastest (state unchanged)."""
        self._check(self.lib.rewl_autotune(self.h, sweeps))

    def launch_shapes(self) -> np.ndarray:
        """Rows of [model, bin-tracking kernel, walkers per warp, warps per block] per launch group."""
        n = C.c_int32(0)
        self._check(self.lib.rewl_launch_shapes(self.h, None, C.byref(n)))
        out = np.zeros((n.value, 4), dtype=np.int32)
        self._check(self.lib.rewl_launch_shapes(self.h, _p(out), C.byref(n)))
        return out

    def status(self) -> Status:
        st = _Status()
        self._check(self.lib.rewl_get_status(self.h, C.byref(st)))
        return self._status(st)

    @staticmethod
    def _status(st: _Status) -> Status:
        return Status(st.sweeps, st.cycles, st.flat_events, st.windows_done, st.windows_total,
                      st.exchanges_attempted, st.exchanges_accepted, st.attempted_flips, st.kernel_launches,
                      bool(st.all_done), st.device_error)

    # -- exports ------------------------------------------------------------------
    def export_walker(self, walker: int):
        inst, w, _ = self._walker_inst[walker]
        ins = self.batch.instances[inst]
        nb = self.windows[inst][w][2]
        dofs = np.zeros(ins.ndof, dtype=np.int8)
        state = np.zeros(5)
        counts = np.zeros(nb, dtype=np.uint64)
        logdos = np.zeros(nb)
        visits = np.zeros(nb, dtype=np.uint64)
        self._check(self.lib.rewl_export_walker(self.h, walker, _p(dofs), _p(state), _p(counts), _p(logdos), _p(visits)))
        if ins.model == MODEL_ISING2D:
            state = state[:2]
        return dict(dofs=dofs, state=state, counts=counts, logdos=logdos, visits=visits)

    def _obs_cols(self, instance: int) -> int:
        return obs_columns(self.batch.instances[instance].model, self.batch.observables)

    def export_observables(self, walker: int) -> np.ndarray:
        """Per-bin observable averages of a walker, rows of [K averages, count] (observables=1 or 2)."""
        inst, w, _ = self._walker_inst[walker]
        out = np.zeros((self.windows[inst][w][2], self._obs_cols(inst)))
        self._check(self.lib.rewl_export_observables(self.h, walker, _p(out)))
        return out

    def window_observables(self, instance: int, window: int) -> np.ndarray:
        """Count-weighted average of the window's replicas' observables, same layout."""
        out = np.zeros((self.windows[instance][window][2], self._obs_cols(instance)))
        self._check(self.lib.rewl_export_window_observables(self.h, instance, window, _p(out)))
        return out

    def window_logdos(self, instance: int, window: int) -> np.ndarray:
        out = np.zeros(self.windows[instance][window][2])
        self._check(self.lib.rewl_export_window_logdos(self.h, instance, window, _p(out)))
        return out

    def window_mask(self, instance: int, window: int) -> np.ndarray:
        out = np.zeros(self.windows[instance][window][2], dtype=np.uint8)
        self._check(self.lib.rewl_export_window_mask(self.h, instance, window, _p(out)))
        return out.astype(bool)

    def window_state(self, instance: int, window: int):
        lnf, done = C.c_double(), C.c_int32()
        self._check(self.lib.rewl_window_state(self.h, instance, window, C.byref(lnf), C.byref(done)))
        return lnf.value, bool(done.value)

    def global_logdos(self, instance: int, half_spectrum: bool = False):
        """Concatenated, normalised ln g(E) of an instance: (energies, ln g)."""
        cap = sum(w[2] for w in self.windows[instance])
        e = np.zeros(cap)
        g = np.zeros(cap)
        n = C.c_int32(cap)
        self._check(self.lib.rewl_global_logdos(self.h, instance, int(half_spectrum), _p(e), _p(g), C.byref(n)))
        return e[:n.value].copy(), g[:n.value].copy()

    def sweep_kernel_time(self):
        """(milliseconds, launches) of the sweep kernels since the last call."""
        ms, n = C.c_double(), C.c_int64()
        self._check(self.lib.rewl_sweep_kernel_time(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def snapshot_size(self) -> int:
        n = C.c_size_t()
        self._check(self.lib.rewl_snapshot_size(self.h, C.byref(n)))
        return n.value

    def snapshot_into(self, ptr: int, nbytes: int) -> None:
        """Copy the full device state into host memory at `ptr` (checkpoint)."""
        self._check(self.lib.rewl_snapshot(self.h, C.c_void_p(ptr), nbytes))

    def restore_from(self, ptr: int, nbytes: int) -> None:
        """Load a state written by snapshot_into (resume)."""
        self._check(self.lib.rewl_restore(self.h, C.c_void_p(ptr), nbytes))

    def snapshot(self) -> np.ndarray:
        buf = np.zeros(self.snapshot_size(), dtype=np.uint8)
        self.snapshot_into(buf.ctypes.data, buf.nbytes)
        return buf

    def restore(self, buf: np.ndarray) -> None:
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self.restore_from(buf.ctypes.data, buf.nbytes)

    def stream_handle(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.rewl_get_stream(self.h, C.byref(s)))
        return s.value or 0
