"""MLP warm start for REWL windows, with a plain-WL fallback for stalled windows.

warm_start() fills every window of an instance with the prediction
N * [s0(E/N) + f(E/N, 1/L, J, K, sigma_h, lo/N, hi/N)] (made window-relative, as
the reference's REDUCE_LOGDOS keeps it) and sets ln f to a small value.  s0 is an
optional baseline: the converged ln g/N of the largest training lattice,
interpolated in E/N.  With it the network only learns the finite-size residual,
whose amplitude is ~100x smaller than ln g/N itself, so the BF16 network's ~1e-3
relative precision costs ~1e-5 in ln g/N instead of ~1e-3 (which times N = 4096
would be several nats).  run() drives check intervals with a burn-in (histograms
cleared while the walkers correct the warm start's error) and returns a window
that stalls in its warm-started stage to plain Wang-Landau.  training_rows()
turns a converged plain run into (features, ln g/N) rows for the next, larger
system.
"""
from __future__ import annotations

import numpy as np

from .engine import Engine, MODEL_ISING2D
from .mlp import MLP, features


def window_energies(engine: Engine, instance: int, window: int) -> np.ndarray:
    lo, hi, nb = engine.windows[instance][window]
    bw = engine.batch.instances[instance].bin_width
    return lo + bw * np.arange(nb)


class Baseline:
    """s0(e): ln g/N of a converged lattice as a monotone piecewise-cubic function of e = E/N."""

    def __init__(self, e: np.ndarray, s: np.ndarray):
        order = np.argsort(e)
        self.e = np.asarray(e, dtype=np.float64)[order]
        self.s = np.asarray(s, dtype=np.float64)[order]
        try:
            from scipy.interpolate import PchipInterpolator
            self._f = PchipInterpolator(self.e, self.s, extrapolate=True)
        except ImportError:                      # linear interpolation is the fallback
            self._f = lambda x: np.interp(x, self.e, self.s)

    @classmethod
    def from_engine(cls, engine: Engine, instance: int) -> "Baseline":
        ins = engine.batch.instances[instance]
        half = ins.model != MODEL_ISING2D and ins.energy_max <= 0.0
        E, lng = engine.global_logdos(instance, half_spectrum=half)
        N = ins.L * ins.L
        return cls(E / N, lng / N)

    def __call__(self, e: np.ndarray) -> np.ndarray:
        return np.asarray(self._f(np.asarray(e, dtype=np.float64)), dtype=np.float64)


def predict_lng(mlp: MLP, E: np.ndarray, L: int, J: float, K: float, sigma_h: float, lo: float, hi: float,
                base: Baseline | None = None) -> np.ndarray:
    """ln g(E) predicted for an L x L instance (baseline + residual network, times N)."""
    N = L * L
    y = mlp.predict(features(E, L, J, K, sigma_h, lo, hi)).astype(np.float64)
    if base is not None:
        y = y + base(np.asarray(E, dtype=np.float64) / N)
    return y * N


def warm_start(engine: Engine, mlp: MLP, instance: int, sigma_h: float = 0.0, lnf0: float = 1e-4,
               base: Baseline | None = None) -> None:
    ins = engine.batch.instances[instance]
    N = ins.L * ins.L
    rows, spans, Es = [], [], []
    for w, (lo, hi, nb) in enumerate(engine.windows[instance]):
        E = window_energies(engine, instance, w)
        rows.append(features(E, ins.L, ins.J, ins.K, sigma_h, lo, hi))
        spans.append(nb)
        Es.append(E)
    pred = mlp.predict(np.concatenate(rows)).astype(np.float64)
    if base is not None:
        pred = pred + base(np.concatenate(Es) / N)
    pred = pred * N
    k = 0
    for w, nb in enumerate(spans):
        g = pred[k:k + nb]
        k += nb
        engine.set_logdos(instance, w, g - g[0])
        engine.set_lnf(instance, w, lnf0)


def run(engine: Engine, max_cycles: int, stall_checks: int = 0, on_cycle=None, burn_in: int = 0):
    """Run check intervals until done, with the warm start's burn-in and stall fallback.

    burn_in: for the first `burn_in` check intervals, clear every window's histogram
    (keeping ln g) after the interval, so that the transient in which the walkers
    correct the warm start's error does not count toward the first flatness test.
    stall_checks: a window still in its first (warm-started) ln f stage after this
    many intervals without a flat event goes back to plain Wang-Landau (ln g = 0,
    ln f = 1, histograms cleared).  Later stages are plain WL and are left alone.
    on_cycle(engine, status) may return True to stop early.
    Returns (status, number of fallbacks).
    """
    first_stage = {}
    if stall_checks > 0:
        for i, ins in enumerate(engine.batch.instances):
            for w in range(ins.num_windows):
                first_stage[(i, w)] = [engine.window_state(i, w)[0], 0]    # ln f0, intervals so far
    fallbacks = 0
    st = engine.status()
    for cycle in range(max_cycles):
        st = engine.run_cycles(1)
        if on_cycle is not None and on_cycle(engine, st):
            break
        if st.all_done:
            break
        if cycle < burn_in:
            for i, ins in enumerate(engine.batch.instances):
                for w in range(ins.num_windows):
                    engine.reset_histograms(i, w, False)
        for key in list(first_stage):
            lnf, done = engine.window_state(*key)
            if lnf != first_stage[key][0] or done:
                del first_stage[key]                    # first flat event: plain WL from here on
                continue
            first_stage[key][1] += 1
            if first_stage[key][1] >= stall_checks:
                i, w = key
                nb = engine.windows[i][w][2]
                engine.set_logdos(i, w, np.zeros(nb))
                engine.set_lnf(i, w, 1.0)
                engine.reset_histograms(i, w, False)
                del first_stage[key]
                fallbacks += 1
    return st, fallbacks


def training_rows(engine: Engine, instance: int, sigma_h: float = 0.0, base: Baseline | None = None):
    """(features, ln g/N) rows from an engine whose windows have converged; with `base`
    the targets are the residual ln g/N - s0(E/N)."""
    ins = engine.batch.instances[instance]
    N = ins.L * ins.L
    half = ins.model != MODEL_ISING2D and ins.energy_max <= 0.0
    E, lng = engine.global_logdos(instance, half_spectrum=half)
    table = dict(zip(np.round(E, 9), lng))
    Xs, ys = [], []
    for w, (lo, hi, nb) in enumerate(engine.windows[instance]):
        Ew = window_energies(engine, instance, w)
        mask = engine.window_mask(instance, w)
        keep = [e for e, m in zip(Ew, mask) if m and round(e, 9) in table]
        if not keep:
            continue
        keep = np.array(keep)
        Xs.append(features(keep, ins.L, ins.J, ins.K, sigma_h, lo, hi))
        y = np.array([table[round(e, 9)] for e in keep]) / N
        if base is not None:
            y = y - base(keep / N)
        ys.append(y)
    return np.concatenate(Xs), np.concatenate(ys).astype(np.float32)
