"""Walkers stay inside their windows whatever their logDoS holds.

The bin-tracking Ising sweep rejects proposals outside the window through guard
bins that hold INT64_MAX, so no value of g at the current bin can let a walker
step out of its window's table.  A window whose logDoS grows past 2^62 grid
units without a flat event (a replica trapped away from part of its range, so
the window never goes flat) is reported as REWL_ESTATE at the next flatness
check instead of being left to overflow int64.
"""
import numpy as np
import pytest

from rewl_simulator_gb300.engine import REWL_ESTATE

UNITS = 2.0 ** 40                 # logDoS grid: 2^-40 nats


@pytest.mark.gpu
def test_walkers_stay_in_window_with_logdos_beyond_2_62_units(engine_lib):
    rg = engine_lib
    L, N = 16, 256
    ins = rg.Instance(model=rg.MODEL_ISING2D, L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                      num_windows=16, replicas_per_window=2, seed=21)
    b = rg.Batch(instances=[ins], sweeps_per_exchange=500, sweeps_per_check=1000, lnf_initial=1.0, lnf_final=1e-6)
    with rg.Engine(b) as eng:
        wins = eng.windows[0]
        for w, (lo, hi, nb) in enumerate(wins):
            eng.set_logdos(0, w, np.full(nb, 1e6))
            eng.set_lnf(0, w, 64.0)                       # 64 nats per visit: g climbs fast
        walkers = [(eng.walker_id(0, w, r), w) for w in range(len(wins)) for r in range(2)]
        top = 0.0
        for _ in range(14):
            eng.run_sweeps(1000)                          # raises on a device error word
            for wk, w in walkers:
                out = eng.export_walker(wk)
                lo, hi, nb = wins[w]
                E = float(out["state"][0])
                assert lo <= E < hi, (wk, w, E, lo, hi)
                top = max(top, float(out["logdos"].max()))
            if top > 4.5e6:
                break
        assert top * UNITS > 2.0 ** 62 + 2.0 ** 58, top   # past the old guard value 2^62
        with pytest.raises(rg.REWLError) as err:
            eng.check_flat()
        assert err.value.code == REWL_ESTATE
