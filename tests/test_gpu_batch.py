"""Uneven batches: instances of different models, sizes and bin widths in one engine.

Every random stream of an instance (initial spins, sweeps, exchange pairing and
acceptance) is keyed by that instance's own seed and instance-relative walker
index, and exchange, flatness and ln f act within an instance.  So an instance
run inside a mixed batch must follow exactly the trajectory of the same instance
run alone: here each one is compared bit for bit with its own CPU oracle after
every check interval.
"""
import numpy as np
import pytest

SE, SC, LNF_FINAL = 20, 40, 1e-7

# name, model, L, K, sigma_h, emin, emax, bw, nwin, R, seed
INSTANCES = [
    ("ising_L8", 0, 8, 0.0, 0.0, -128.0, 132.0, 4.0, 3, 2, 11),
    ("ising_L12_bw8", 0, 12, 0.0, 0.0, -288.0, 296.0, 8.0, 4, 2, 3),      # general sweep kernel
    ("at_L4_rf", 1, 4, 0.5, 0.5, -(2.5) * 2 * 16, 0.0, 0.05, 2, 2, 7),
    ("ising_L16", 0, 16, 0.0, 0.0, -512.0, 516.0, 4.0, 4, 3, 17),
]


@pytest.mark.gpu
@pytest.mark.parametrize("graphs,autotune,persistent", [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 0, 1), (1, 1, 1)],
                         ids=["eager", "graphs", "graphs_autotuned", "persistent", "persistent_graphs"])
def test_mixed_batch_instances_match_their_oracles(engine_lib, oracle_lib, graphs, autotune, persistent):
    """The launch groups (two bin-tracking shapes, the general Ising kernel, Ashkin-Teller) run
    concurrently on their own streams; with graphs each check interval replays as one captured
    graph; the autotuner times the groups' shapes first.  With `persistent` every group's walkers
    are tasks of one work-stealing launch (the bin width 8 instance on the global-table form).
    None of it may change a trajectory."""
    rg, po = engine_lib, oracle_lib
    inss, orcs = [], []
    for name, model, L, K, sig, emin, emax, bw, nwin, R, seed in INSTANCES:
        N = L * L
        fields = None
        if sig > 0:
            fields = np.round(np.random.default_rng(seed).normal(0, sig, N) * 2**20) / 2**20
        inss.append(rg.Instance(model=model, L=L, K=K, fields=fields, energy_min=emin, energy_max=emax, bin_width=bw,
                                num_windows=nwin, replicas_per_window=R, window_overlap=0.75, init_mode=0, seed=seed))
        cfg = po.Config(model=model, L=L, K=K, escale_bits=0 if model == 0 else 20, nwin=nwin, R=R,
                        sweeps_per_exchange=SE, sweeps_per_check=SC, emin=emin, emax=emax, bw=bw, overlap=0.75,
                        lnf0=1.0, lnf_final=LNF_FINAL, flat_param=0.8, mask_mode=po.MASK_VISITED,
                        semantics=po.SEM_ENGINE, seed=seed)
        orcs.append(po.Oracle(cfg, fields=fields))
    b = rg.Batch(instances=inss, sweeps_per_exchange=SE, sweeps_per_check=SC, flatness_param=0.8,
                 lnf_initial=1.0, lnf_final=LNF_FINAL, mask_mode=rg.MASK_VISITED, graphs=graphs, autotune=autotune,
                 persistent=persistent)
    eng = rg.Engine(b)
    try:
        def compare(tag):
            for i, (spec, orc) in enumerate(zip(INSTANCES, orcs)):
                nwin, R = spec[8], spec[9]
                for w in range(nwin):
                    for r in range(R):
                        out = eng.export_walker(eng.walker_id(i, w, r))
                        s = w * R + r
                        c, g, v = orc.tables(s)
                        msg = f"{tag} {spec[0]} window {w} replica {r}"
                        np.testing.assert_array_equal(out["dofs"], orc.dofs(s), err_msg=msg + " dofs")
                        np.testing.assert_array_equal(out["state"], orc.state(s), err_msg=msg + " state")
                        np.testing.assert_array_equal(out["counts"], c, err_msg=msg + " counts")
                        np.testing.assert_array_equal(out["logdos"], g, err_msg=msg + " logdos")
                    lnf, done = eng.window_state(i, w)
                    assert lnf == orc.lnf(w * R), f"{tag} {spec[0]} window {w} lnf"
                    assert done == bool(orc.done_flags()[w]), f"{tag} {spec[0]} window {w} done"

        compare("init")
        for k in range(4):
            eng.run_cycles(1)
            for orc in orcs:
                orc.cycle()
            compare(f"cycle {k}")
        st = eng.status()
        assert st.exchanges_attempted == sum(o.exchange_stats()[0] for o in orcs)
        assert st.exchanges_accepted == sum(o.exchange_stats()[1] for o in orcs)
    finally:
        eng.close()
        for o in orcs:
            o.close()


@pytest.mark.gpu
def test_autotune_leaves_the_state_unchanged(engine_lib):
    """rewl_autotune runs trial sweeps on the live state and restores it: every walker's tables,
    configuration and the engine's counters are as before, and the shapes it keeps are admissible."""
    rg = engine_lib
    inss = [rg.Instance(model=0, L=16, energy_min=-512.0, energy_max=516.0, bin_width=4.0, num_windows=4,
                        replicas_per_window=4, seed=3),
            rg.Instance(model=0, L=8, energy_min=-128.0, energy_max=132.0, bin_width=4.0, num_windows=3,
                        replicas_per_window=2, seed=4)]
    b = rg.Batch(instances=inss, sweeps_per_exchange=20, sweeps_per_check=40, lnf_final=1e-6)
    with rg.Engine(b) as eng:
        eng.run_cycles(2)
        before = [eng.export_walker(s) for s in range(eng.num_walkers)]
        st0 = eng.status()
        eng.autotune(sweeps=5)
        after = [eng.export_walker(s) for s in range(eng.num_walkers)]
        st1 = eng.status()
        for x, y in zip(before, after):
            for k in x:
                np.testing.assert_array_equal(x[k], y[k])
        assert (st0.sweeps, st0.attempted_flips, st0.cycles, st0.exchanges_attempted) == \
               (st1.sweeps, st1.attempted_flips, st1.cycles, st1.exchanges_attempted)
        shapes = eng.launch_shapes()
        assert len(shapes) == 2
        for model, bins, g, wpb in shapes:
            assert g in (1, 2, 4) and wpb in (1, 2, 4, 8)


@pytest.mark.gpu
def test_graph_replay_with_manual_steps_and_restore(engine_lib):
    """Graph replay interleaved with hand-run sweeps and exchanges (the next interval then runs
    eagerly), a snapshot, more cycles, and a restore of the snapshot followed by the same cycles:
    a graph engine and an eager engine end in identical states."""
    rg = engine_lib
    ins = [rg.Instance(model=0, L=8, energy_min=-128.0, energy_max=132.0, bin_width=4.0, num_windows=3,
                       replicas_per_window=2, seed=21),
           rg.Instance(model=1, L=4, K=0.5, energy_min=-80.0, energy_max=0.0, bin_width=0.05, num_windows=2,
                       replicas_per_window=2, seed=22,
                       fields=np.round(np.random.default_rng(22).normal(0, 0.5, 16) * 2**20) / 2**20)]

    def run(graphs):
        b = rg.Batch(instances=ins, sweeps_per_exchange=10, sweeps_per_check=30, lnf_final=1e-6,
                     mask_mode=rg.MASK_VISITED, graphs=graphs)
        with rg.Engine(b) as eng:
            eng.run_cycles(2)
            eng.wang_landau_walk(7)
            eng.replica_exchange_update()
            eng.run_cycles(2)
            snap = eng.snapshot()
            eng.run_cycles(3)
            first = [eng.export_walker(s) for s in range(eng.num_walkers)]
            eng.restore(snap)
            eng.run_cycles(3)
            again = [eng.export_walker(s) for s in range(eng.num_walkers)]
            st = eng.status()
        return first, again, st

    g_first, g_again, g_st = run(1)
    e_first, e_again, e_st = run(0)
    for a, b, c, d in zip(g_first, e_first, g_again, e_again):
        for k in a:
            np.testing.assert_array_equal(a[k], b[k])     # graph == eager
            np.testing.assert_array_equal(a[k], c[k])     # restore + the same cycles == first pass
            np.testing.assert_array_equal(c[k], d[k])
    assert (g_st.sweeps, g_st.exchanges_attempted, g_st.exchanges_accepted, g_st.flat_events) == \
           (e_st.sweeps, e_st.exchanges_attempted, e_st.exchanges_accepted, e_st.flat_events)
