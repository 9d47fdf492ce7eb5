"""Walkers stay inside their windows whatever their logDoS holds, and no logDoS entry can
overflow int64.

The bin-tracking Ising sweep rejects proposals outside the window through guard bins that
hold INT64_MAX, so no value of g at the current bin can let a walker step out of its window's
table.  Every kernel that adds to g checks the values it wrote against 2^62 grid units
(6.7e7 nats) and, once one passes, the engine stops with REWL_ESTATE: every later kernel
returns without work.  Sweep launches are split so that one launch adds at most
2^62 - 2^58 units to a bin (here ln f = 64 nats at L = 32: at most 960 sweeps per launch), so
the largest value ever stored stays below 2^63.
"""
import numpy as np
import pytest

from rewl_simulator_gb300.engine import REWL_ESTATE

UNITS = 2.0 ** 36                 # logDoS grid: 2^-36 nats
LIMIT = 2.0 ** 62 / UNITS         # 6.71e7 nats
INT64_TOP = 2.0 ** 63 / UNITS     # 1.34e8 nats
START = 2.0 ** 24                 # nats: the largest logDoS rewl_set_logdos takes (2^60 units)


@pytest.mark.gpu
def test_logdos_past_the_limit_stops_the_engine_before_int64_overflow(engine_lib):
    rg = engine_lib
    L, N = 32, 1024
    ins = rg.Instance(model=rg.MODEL_ISING2D, L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                      num_windows=64, replicas_per_window=2, seed=21)
    b = rg.Batch(instances=[ins], sweeps_per_exchange=500, sweeps_per_check=1000, lnf_initial=1.0, lnf_final=1e-6)
    with rg.Engine(b) as eng:
        wins = eng.windows[0]
        for w, (lo, hi, nb) in enumerate(wins):
            eng.set_logdos(0, w, np.full(nb, START))
            eng.set_lnf(0, w, 64.0)                       # 64 nats per visit: g climbs fast
        walkers = [(eng.walker_id(0, w, r), w) for w in range(len(wins)) for r in range(2)]

        def check_walkers():
            top = 0.0
            for wk, w in walkers:
                out = eng.export_walker(wk)
                lo, hi, nb = wins[w]
                E = float(out["state"][0])
                assert lo <= E < hi, (wk, w, E, lo, hi)
                g = out["logdos"]
                assert np.isfinite(g).all() and g.min() >= START - 1e-6    # only grows: no wrap
                top = max(top, float(g.max()))
            return top

        stopped = None
        for k in range(40):
            try:
                eng.run_sweeps(3000)
            except rg.REWLError as err:
                stopped = err
                break
            assert check_walkers() < LIMIT
        assert stopped is not None and stopped.code == REWL_ESTATE, stopped
        top = check_walkers()
        assert LIMIT <= top < INT64_TOP, top                # past the limit, far from overflow
        # the engine has stopped: later calls report it and change nothing
        before = eng.export_walker(0)["logdos"].copy()
        with pytest.raises(rg.REWLError) as again:
            eng.run_sweeps(10)
        assert again.value.code == REWL_ESTATE
        np.testing.assert_array_equal(eng.export_walker(0)["logdos"], before)


@pytest.mark.gpu
def test_large_lnf_splits_launches_without_changing_results(engine_lib, oracle_lib):
    """ln f = 64 nats on L = 64 allows at most (2^62 - 2^58) / (64 x 2^36) / 4096 = 240 sweeps per
    launch: an exchange interval of 500 sweeps becomes three launches, bit for bit the oracle's
    run."""
    rg, po = engine_lib, oracle_lib
    L, N = 64, 4096
    ins = rg.Instance(model=0, L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0, num_windows=4,
                      replicas_per_window=2, seed=5)
    b = rg.Batch(instances=[ins], sweeps_per_exchange=500, sweeps_per_check=1000, lnf_initial=64.0, lnf_final=1e-6)
    cfg = po.Config(model=0, L=L, nwin=4, R=2, sweeps_per_exchange=500, sweeps_per_check=1000, emin=-2.0 * N,
                    emax=2.0 * N + 4, bw=4.0, lnf0=64.0, lnf_final=1e-6, semantics=po.SEM_ENGINE, seed=5)
    orc = po.Oracle(cfg)
    with rg.Engine(b) as eng:
        st0 = eng.status()
        eng.run_cycles(1)
        orc.cycle()
        st = eng.status()
        # 2 exchange intervals x 3 launches + 2 exchanges + 1 flatness step
        assert st.kernel_launches - st0.kernel_launches == 9, st.kernel_launches - st0.kernel_launches
        for s in range(8):
            out = eng.export_walker(s)
            c, g, v = orc.tables(s)
            np.testing.assert_array_equal(out["counts"], c)
            np.testing.assert_array_equal(out["logdos"], g)
            np.testing.assert_array_equal(out["dofs"], orc.dofs(s))
    orc.close()
