"""MLP warm start for REWL windows, with a plain-WL fallback for stalled windows.

warm_start() fills every window of an instance with the network's prediction
N * f(E/N, 1/L, J, K, sigma_h, lo/N, hi/N) (made window-relative, as the
reference's REDUCE_LOGDOS keeps it) and sets ln f to a small value.  run() drives
check intervals and returns a window to plain Wang-Landau (ln g = 0, ln f = 1,
histograms cleared) when it has gone `stall_checks` intervals without a flat
event.  training_rows() turns a converged plain run into (features, ln g/N)
rows for the next, larger system.
"""
from __future__ import annotations

import numpy as np

from .engine import Engine, MODEL_ISING2D
from .mlp import MLP, features


def window_energies(engine: Engine, instance: int, window: int) -> np.ndarray:
    lo, hi, nb = engine.windows[instance][window]
    bw = engine.batch.instances[instance].bin_width
    return lo + bw * np.arange(nb)


def warm_start(engine: Engine, mlp: MLP, instance: int, sigma_h: float = 0.0, lnf0: float = 1e-4) -> None:
    ins = engine.batch.instances[instance]
    N = ins.L * ins.L
    rows, spans = [], []
    for w, (lo, hi, nb) in enumerate(engine.windows[instance]):
        rows.append(features(window_energies(engine, instance, w), ins.L, ins.J, ins.K, sigma_h, lo, hi))
        spans.append(nb)
    pred = mlp.predict(np.concatenate(rows)).astype(np.float64) * N
    k = 0
    for w, nb in enumerate(spans):
        g = pred[k:k + nb]
        k += nb
        engine.set_logdos(instance, w, g - g[0])
        engine.set_lnf(instance, w, lnf0)


def run(engine: Engine, max_cycles: int, stall_checks: int = 0, on_cycle=None):
    """Run check intervals until done; optionally fall back to plain WL per stalled window.

    on_cycle(engine, status) may return True to stop early.
    """
    last_lnf = {}
    since = {}
    fallbacks = 0
    st = engine.status()
    for _ in range(max_cycles):
        st = engine.run_cycles(1)
        if on_cycle is not None and on_cycle(engine, st):
            break
        if st.all_done:
            break
        if stall_checks > 0:
            for i, ins in enumerate(engine.batch.instances):
                for w in range(ins.num_windows):
                    lnf, done = engine.window_state(i, w)
                    key = (i, w)
                    if last_lnf.get(key) != lnf:
                        last_lnf[key] = lnf
                        since[key] = 0
                        continue
                    since[key] += 1
                    if since[key] >= stall_checks and not done:
                        nb = engine.windows[i][w][2]
                        engine.set_logdos(i, w, np.zeros(nb))
                        engine.set_lnf(i, w, 1.0)
                        engine.reset_histograms(i, w, False)
                        since[key] = 0
                        last_lnf[key] = 1.0
                        fallbacks += 1
    return st, fallbacks


def training_rows(engine: Engine, instance: int, sigma_h: float = 0.0):
    """(features, ln g/N) rows from an engine whose windows have converged."""
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
        ys.append(np.array([table[round(e, 9)] for e in keep]) / N)
    return np.concatenate(Xs), np.concatenate(ys).astype(np.float32)
