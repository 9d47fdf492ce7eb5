"""GPU engine (through the C ABI) against the reference and the CPU oracle.

* Replay parity: fed the reference walker's own uniform stream, the CUDA sweep
  kernels must reproduce the reference's lattices, energies, magnetisations,
  histograms and logDoS bit for bit (golden fixtures from the reference's
  REWL_Walker, tests/golden/make_golden.py).
* Engine-semantics parity: with Philox streams, a multi-window, multi-replica
  REWL run on the GPU (sweeps, replica exchange, flatness, averaging, ln f) must
  match the CPU oracle bit for bit after every check interval.
"""
import numpy as np
import pytest

from conftest import GOLDEN

REPLAY = sorted(p.name for p in GOLDEN.glob("replay_*.npz"))


def _assert_obs_close(got, ref, corr, msg="", rtol=1e-12):
    """Moments to FP64 rounding of the running means; the G(q_min) columns (every fourth with
    correlators) to the rounding of a transform summed in another order: the reference adds
    it site by site, the kernels from row and column sums."""
    g = np.zeros(got.shape[1], bool)
    if corr:
        g[3::4] = True
    np.testing.assert_allclose(got[:, ~g], ref[:, ~g], rtol=rtol, atol=1e-15, err_msg=msg)
    np.testing.assert_allclose(got[:, g], ref[:, g], rtol=1e-10, atol=1e-14, err_msg=msg + " G(q_min)")


def _engine_layout(dofs_ref: np.ndarray, model: int) -> np.ndarray:
    if model == 0:
        return dofs_ref.astype(np.int8)
    return np.concatenate([dofs_ref[0::2], dofs_ref[1::2]]).astype(np.int8)


@pytest.mark.gpu
@pytest.mark.parametrize("name", REPLAY)
def test_replay_matches_reference(engine_lib, oracle_lib, name):
    rg, po = engine_lib, oracle_lib
    z = np.load(GOLDEN / name)
    corr = name.startswith("replay_corr_")     # the reference's CORRELATION_LENGTHS build
    model = int(z["model"])
    fields = z["fields"] if z["fields"].size else None
    ins = rg.Instance(model=model, L=int(z["L"]), J=1.0, K=float(z["K"]) if model else 0.0, fields=fields,
                      energy_min=float(z["wmin"]), energy_max=float(z["wmax"]), bin_width=float(z["bw"]),
                      num_windows=1, replicas_per_window=1, init_mode=1, seed=1)
    b = rg.Batch(instances=[ins], rng_mode=rg.RNG_REPLAY, lnf_initial=float(z["lnf1"]), lnf_final=1e-9,
                 observables=2 if corr else 1)
    with rg.Engine(b) as eng:
        which = int(z["state0"][4]) if model else 0
        eng.import_dofs(0, _engine_layout(z["dofs0"], model), which)
        skip = int(z["adjust_draws"])
        need = int(z["draws2"]) + 64
        u = po.mt64_uniforms(int(z["seed"]), need)[skip:]
        eng.set_uniform_stream(0, u)
        st0 = eng.export_walker(0)
        np.testing.assert_array_equal(st0["state"], z["state0"])
        for stage in (1, 2):
            if stage == 2:
                eng.reset_histograms(0, 0, True)
                eng.set_lnf(0, 0, float(z["lnf2"]))
            eng.run_sweeps(int(z[f"sweeps{stage}"]))
            out = eng.export_walker(0)
            np.testing.assert_array_equal(out["counts"], z[f"counts{stage}"])
            np.testing.assert_array_equal(out["logdos"], z[f"logdos{stage}"])
            np.testing.assert_array_equal(out["state"], z[f"state{stage}"])
            np.testing.assert_array_equal(out["dofs"], _engine_layout(z[f"dofs{stage}"], model))
            # per-bin observables: the reference's running means, to FP64 rounding
            obs, ref = eng.export_observables(0), z[f"obs{stage}"]
            np.testing.assert_array_equal(obs[:, -1], ref[:, -1])
            _assert_obs_close(obs[:, :-1], ref[:, :-1], corr, f"stage {stage}")


def _pair(rg, po, model, L, emin, emax, bw, nwin, R, se, sc, seed, K=0.5, fields=None, flat=0.8,
          mask=0, lnf0=1.0, overlap=0.75, flat_mode=0, walkers_per_warp=0, observables=0, one_over_t=0,
          lnf_final=1e-7, nthreads=1):
    ins = rg.Instance(model=model, L=L, J=1.0, K=K if model else 0.0, fields=fields, energy_min=emin,
                      energy_max=emax, bin_width=bw, num_windows=nwin, replicas_per_window=R,
                      window_overlap=overlap, init_mode=0, seed=seed)
    b = rg.Batch(instances=[ins], sweeps_per_exchange=se, sweeps_per_check=sc, flatness_mode=flat_mode,
                 flatness_param=flat, lnf_initial=lnf0, lnf_final=lnf_final, mask_mode=mask,
                 walkers_per_warp=walkers_per_warp, observables=observables, one_over_t=one_over_t)
    eng = rg.Engine(b)
    cfg = po.Config(model=model, L=L, K=K, escale_bits=0 if model == 0 else 20, nwin=nwin, R=R,
                    sweeps_per_exchange=se, sweeps_per_check=sc, emin=emin, emax=emax, bw=bw, overlap=overlap,
                    lnf0=lnf0, lnf_final=lnf_final, flat_param=flat, flat_mode=flat_mode, mask_mode=mask,
                    semantics=po.SEM_ENGINE, seed=seed, observables=observables, one_over_t=one_over_t,
                    nthreads=nthreads)
    orc = po.Oracle(cfg, fields=fields)
    return eng, orc


def _compare(eng, orc, tag):
    for s in range(orc.num_walkers):
        out = eng.export_walker(s)
        c, g, v = orc.tables(s)
        np.testing.assert_array_equal(out["dofs"], orc.dofs(s), err_msg=f"{tag} walker {s} dofs")
        np.testing.assert_array_equal(out["state"], orc.state(s), err_msg=f"{tag} walker {s} state")
        np.testing.assert_array_equal(out["counts"], c, err_msg=f"{tag} walker {s} counts")
        np.testing.assert_array_equal(out["visits"], v, err_msg=f"{tag} walker {s} visits")
        np.testing.assert_array_equal(out["logdos"], g, err_msg=f"{tag} walker {s} logdos")
    for w in range(orc.cfg.nwin):
        lnf, done = eng.window_state(0, w)
        assert lnf == orc.lnf(w * orc.cfg.R), f"{tag} window {w} lnf"
        assert done == bool(orc.done_flags()[w]), f"{tag} window {w} done"


CASES = [
    # model, L, emin, emax, bw, nwin, R, se, sc, seed, cycles
    ("ising_L8_3x2", 0, 8, -128.0, 132.0, 4.0, 3, 2, 50, 100, 11, 6),
    ("ising_L16_4x3", 0, 16, -512.0, 516.0, 4.0, 4, 3, 20, 40, 17, 5),
    ("ising_L32_64w_top", 0, 32, -2048.0, 2052.0, 4.0, 64, 1, 4, 8, 23, 2),
    ("ising_L6_2x3", 0, 6, -72.0, 76.0, 4.0, 2, 3, 20, 40, 5, 8),
    ("ising_L12_4x2_bw8", 0, 12, -288.0, 296.0, 8.0, 4, 2, 10, 20, 3, 5),
    ("ising_L40_3x2", 0, 40, -3200.0, -2000.0, 4.0, 3, 2, 4, 8, 9, 3),
    ("ising_L64_2x2", 0, 64, -8192.0, -7000.0, 4.0, 2, 2, 2, 4, 2, 2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("walkers_per_warp", [0, 1, 2, 4])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_engine_matches_oracle_ising(engine_lib, oracle_lib, case, walkers_per_warp):
    _, model, L, emin, emax, bw, nwin, R, se, sc, seed, cycles = case
    eng, orc = _pair(engine_lib, oracle_lib, model, L, emin, emax, bw, nwin, R, se, sc, seed,
                     walkers_per_warp=walkers_per_warp)
    try:
        _compare(eng, orc, "init")
        for k in range(cycles):
            eng.run_cycles(1)
            orc.cycle()
            _compare(eng, orc, f"cycle {k}")
        st = eng.status()
        att, acc = orc.exchange_stats()
        assert (st.exchanges_attempted, st.exchanges_accepted) == (att, acc)
        if L <= 12:
            assert st.exchanges_accepted > 0
    finally:
        eng.close()
        orc.close()


AT_CASES = [
    # name, L, K, sigma_h, bw, nwin, R, se, sc, seed, cycles, mask
    ("at_L4_rf", 4, 0.5, 0.5, 0.05, 2, 2, 20, 40, 7, 4, 1),
    ("at_L6_clean_bw025", 6, 0.25, 0.0, 0.25, 3, 2, 10, 20, 3, 4, 1),
    ("at_L8_rf_bw05", 8, 0.5, 0.3, 0.5, 2, 2, 5, 10, 13, 3, 1),
    # odd rows: the chunk is a whole row of 5 / 7 sites (row wrap inside an odd chunk)
    ("at_L5_rf", 5, 0.5, 0.5, 0.05, 2, 2, 20, 40, 5, 4, 1),
    ("at_L7_clean_bw025", 7, 0.25, 0.0, 0.25, 2, 2, 10, 20, 9, 3, 1),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", AT_CASES, ids=[c[0] for c in AT_CASES])
def test_engine_matches_oracle_at(engine_lib, oracle_lib, case):
    _, L, K, sig, bw, nwin, R, se, sc, seed, cycles, mask = case
    N = L * L
    emin = -(2.0 + K) * 2 * N
    rng = np.random.default_rng(seed)
    fields = np.round(rng.normal(0, sig, N) * 2**20) / 2**20 if sig > 0 else None
    eng, orc = _pair(engine_lib, oracle_lib, 1, L, emin, 0.0, bw, nwin, R, se, sc, seed, K=K, fields=fields,
                     mask=mask)
    try:
        _compare(eng, orc, "init")
        for k in range(cycles):
            eng.run_cycles(1)
            orc.cycle()
            _compare(eng, orc, f"cycle {k}")
    finally:
        eng.close()
        orc.close()


@pytest.mark.gpu
def test_ising_L8_converges_to_exact(engine_lib, oracle_lib):
    """A whole run to ln f < 1e-5 (halving): the concatenated ln g equals the one the oracle's run
    of the same seed gives, to rounding, and lies within 0.1 of the exact density of states.  The
    halving schedule's error floor at this size spans 0.03-0.16 over seeds (oracle runs of seeds
    20-29); this seed's is 0.033."""
    rg, po = engine_lib, oracle_lib
    z = np.load(GOLDEN / "exact_ising_L8.npz")
    seed = 25
    ins = rg.Instance(model=0, L=8, energy_min=-128.0, energy_max=132.0, bin_width=4.0, num_windows=2,
                      replicas_per_window=4, seed=seed)
    b = rg.Batch(instances=[ins], sweeps_per_exchange=100, sweeps_per_check=200, lnf_final=1e-5)
    orc = po.Oracle(po.Config(model=0, L=8, nwin=2, R=4, sweeps_per_exchange=100, sweeps_per_check=200,
                              emin=-128.0, emax=132.0, bw=4.0, lnf_final=1e-5, semantics=po.SEM_ENGINE, seed=seed))
    while not orc.all_done():
        orc.cycle()
    wins = []
    for w in range(2):
        lo, _, _, nb = orc.windows[w]
        m = orc.window_mask(w)
        wins.append(((lo + 4.0 * np.arange(nb))[m], orc.window_logdos(w)[m]))
    orc.close()
    E_ref, g_ref = rg.concatenate_windows(wins, 2.0, 64)
    with rg.Engine(b) as eng:
        st = eng.simulate(max_cycles=200000, timeout_ms=300000)
        assert st.all_done
        E, g = eng.global_logdos(0)
        np.testing.assert_array_equal(E, z["E"])
        np.testing.assert_array_equal(E, E_ref)
        np.testing.assert_allclose(g, g_ref, rtol=0, atol=1e-9)
        err = np.abs(g - z["lng"]).max()
        assert err < 0.1, err


OBS_CASES = [
    # name, model, L, emin, emax, bw, nwin, R, se, sc, seed, cycles, walkers_per_warp, sigma_h, mask, observables
    ("ising_L8_bins", 0, 8, -128.0, 132.0, 4.0, 3, 2, 50, 100, 11, 3, 0, 0.0, 0, 1),
    ("ising_L16_bins_2perwarp", 0, 16, -512.0, 516.0, 4.0, 4, 3, 20, 40, 17, 3, 2, 0.0, 0, 1),
    ("ising_L12_bw8_general", 0, 12, -288.0, 296.0, 8.0, 4, 2, 10, 20, 3, 3, 0, 0.0, 0, 1),
    ("at_L4_rf", 1, 4, -(2.5) * 2 * 16, 0.0, 0.05, 2, 2, 20, 40, 7, 3, 0, 0.5, 1, 1),
    # with the G(q_min) correlators: the bin-tracking kernel (chunk = row, chunks within a row, two
    # walkers per warp), the general Ising kernel (bin width 8) and the Ashkin-Teller kernel;
    # exchanges add transforms through the exchange touch
    ("ising_L8_corr", 0, 8, -128.0, 132.0, 4.0, 3, 2, 50, 100, 11, 4, 0, 0.0, 0, 2),
    ("ising_L16_corr", 0, 16, -512.0, 516.0, 4.0, 4, 3, 20, 40, 17, 3, 0, 0.0, 0, 2),
    ("ising_L64_corr_chunks", 0, 64, -8192.0, -7000.0, 4.0, 2, 2, 4, 8, 29, 2, 0, 0.0, 0, 2),
    ("ising_L16_corr_2perwarp", 0, 16, -512.0, 516.0, 4.0, 4, 3, 20, 40, 17, 3, 2, 0.0, 0, 2),
    ("ising_L12_bw8_corr_general", 0, 12, -288.0, 296.0, 8.0, 4, 2, 10, 20, 3, 3, 0, 0.0, 0, 2),
    ("at_L4_rf_corr", 1, 4, -(2.5) * 2 * 16, 0.0, 0.05, 2, 2, 20, 40, 7, 3, 0, 0.5, 1, 2),
    ("at_L8_rf_corr", 1, 8, -(2.5) * 2 * 64, -40.0, 0.05, 2, 2, 10, 20, 9, 3, 0, 0.5, 1, 2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", OBS_CASES, ids=[c[0] for c in OBS_CASES])
def test_engine_observables_match_oracle(engine_lib, oracle_lib, case):
    """Per-bin observables of every walker, and their count-weighted window average, against
    the oracle's running means after every check interval (all three sweep kernels)."""
    _run_observables_case(engine_lib, oracle_lib, case)


TABLE_CASES = [
    ("ising_L8_tables", 0, 8, -128.0, 132.0, 4.0, 3, 2, 50, 100, 11, 3, 0, 0.0, 0, 1),
    ("ising_L16_tables_corr", 0, 16, -512.0, 516.0, 4.0, 4, 3, 20, 40, 17, 3, 0, 0.0, 0, 2),
    ("ising_L12_bw8_tables_corr", 0, 12, -288.0, 296.0, 8.0, 4, 2, 10, 20, 3, 3, 0, 0.0, 0, 2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", TABLE_CASES, ids=[c[0] for c in TABLE_CASES])
def test_ising_on_the_global_table_kernel(engine_lib, oracle_lib, monkeypatch, case):
    """The model-generic global-table kernel (k_sweep_tables) instantiated for Ising -- the
    kernel an Ising window too large for shared memory runs on -- against the oracle."""
    monkeypatch.setenv("REWL_SWEEP_VARIANT", "4")
    _run_observables_case(engine_lib, oracle_lib, case)


def _run_observables_case(engine_lib, oracle_lib, case):
    _, model, L, emin, emax, bw, nwin, R, se, sc, seed, cycles, wpw, sig, mask, obs_mode = case
    fields = None
    if sig > 0:
        fields = np.round(np.random.default_rng(seed).normal(0, sig, L * L) * 2**20) / 2**20
    eng, orc = _pair(engine_lib, oracle_lib, model, L, emin, emax, bw, nwin, R, se, sc, seed, fields=fields,
                     mask=mask, walkers_per_warp=wpw, observables=obs_mode)
    try:
        for k in range(cycles):
            eng.run_cycles(1)
            orc.cycle()
            _compare(eng, orc, f"cycle {k}")
            for w in range(nwin):
                ws = []
                for r in range(R):
                    s = w * R + r
                    got, ref = eng.export_observables(s), orc.obs(s)
                    np.testing.assert_array_equal(got[:, -1], ref[:, -1], err_msg=f"cycle {k} walker {s} counts")
                    _assert_obs_close(got[:, :-1], ref[:, :-1], obs_mode == 2, f"cycle {k} walker {s}")
                    ws.append(ref)
                cnt = sum(o[:, -1] for o in ws)
                avg = sum(o[:, :-1] * o[:, -1:] for o in ws) / np.maximum(cnt, 1)[:, None]
                got = eng.window_observables(0, w)
                np.testing.assert_array_equal(got[:, -1], cnt)
                _assert_obs_close(got[:, :-1], avg, obs_mode == 2, f"cycle {k} window {w}", rtol=1e-11)
    finally:
        eng.close()
        orc.close()


@pytest.mark.gpu
def test_ising_window_too_large_for_shared_memory(engine_lib, oracle_lib):
    """An Ising window of 36,865 bins (L = 96, one window over the whole spectrum at bin width 1)
    does not fit in shared memory: the engine runs it on the global-table kernel, bit for bit
    with the oracle."""
    rg, po = engine_lib, oracle_lib
    L, N = 96, 96 * 96
    eng, orc = _pair(rg, po, 0, L, -2.0 * N, 2.0 * N + 4, 1.0, 1, 2, 5, 10, 41)
    try:
        shapes = eng.launch_shapes()
        assert len(shapes) == 1 and shapes[0][1] == 0          # not the bin-tracking kernel
        for k in range(2):
            eng.run_cycles(1)
            orc.cycle()
            _compare(eng, orc, f"cycle {k}")
    finally:
        eng.close()
        orc.close()


def _one_over_t_engaged(orc) -> bool:
    """Once the 1/t rule takes over, ln f = 1/t is no longer a power of two (halving from 1 keeps
    it one)."""
    for w in range(orc.cfg.nwin):
        e = np.log2(orc.lnf(w * orc.cfg.R))
        if abs(e - round(e)) > 1e-9:
            return True
    return False


FLAT_CASES = [
    # name, model, L, emin, emax, bw, nwin, R, se, sc, seed, cycles, K, sigma_h, flat_mode, flat_param,
    #   mask, one_over_t, walkers_per_warp, flat events at least, 1/t engaged
    # count-weighted averaging over eight replicas (the benchmark layouts' R), both walker packings
    ("ising_L8_3x8", 0, 8, -128.0, 132.0, 4.0, 3, 8, 50, 100, 11, 12, 0.0, 0.0, 0, 0.8, 0, 0, 0, 3, False),
    ("ising_L8_3x8_2perwarp", 0, 8, -128.0, 132.0, 4.0, 3, 8, 50, 100, 11, 12, 0.0, 0.0, 0, 0.8, 0, 0, 2, 3, False),
    ("ising_L16_4x8", 0, 16, -512.0, 516.0, 4.0, 4, 8, 100, 200, 17, 10, 0.0, 0.0, 0, 0.8, 0, 0, 0, 2, False),
    # more than 32 replicas per window (the exchange's acceptance words then start at counter 64)
    ("ising_L6_2x40", 0, 6, -72.0, 76.0, 4.0, 2, 40, 50, 100, 11, 20, 0.0, 0.0, 0, 0.8, 0, 0, 0, 5, False),
    # the reference's classic rule (max - min) / min <= 0.3 (rewl_histograms.hpp:131-152)
    ("ising_L8_max_min_ratio", 0, 8, -128.0, 132.0, 4.0, 3, 2, 50, 100, 11, 20, 0.0, 0.0, 1, 0.3, 0, 0, 0, 7, False),
    # the reference's default build: 1/t with the all-visited rule (rewl_histograms.hpp:115-130,
    # rewl_simulation.hpp:557-567); 1/t engages at the 21st interval
    ("ising_L8_all_visited_1overt", 0, 8, -128.0, 132.0, 4.0, 3, 2, 50, 100, 11, 40, 0.0, 0.0, 2, 0.0, 0, 1, 0, 30, True),
    # 1/t under min >= 0.5 mean: engages after about 150 intervals
    ("ising_L6_min_over_mean_1overt", 0, 6, -72.0, 76.0, 4.0, 2, 2, 10, 20, 7, 220, 0.0, 0.0, 0, 0.5, 0, 1, 0, 20, True),
    # Ashkin-Teller at bin width 0.05 with the visited-bin mask (clean couplings reach every fifth
    # bin only), four replicas averaged
    ("at_L6_clean_K025_bw005_visited", 1, 6, -(2.25) * 2 * 36, 0.0, 0.05, 3, 4, 50, 100, 3, 30, 0.25, 0.0, 0, 0.8, 1, 0, 0, 10, False),
    ("at_L4_clean_K05_bw005_visited", 1, 4, -(2.5) * 2 * 16, 0.0, 0.05, 2, 4, 50, 100, 7, 30, 0.5, 0.0, 0, 0.8, 1, 0, 0, 10, False),
    # Baxter fields, resets and averaging of the Ashkin-Teller tables
    ("at_L6_fields_bw1_visited", 1, 6, -(2.5) * 2 * 36, 0.0, 1.0, 3, 4, 50, 100, 3, 30, 0.5, 0.5, 0, 0.8, 1, 0, 0, 8, False),
    ("at_L4_clean_all_visited_1overt", 1, 4, -80.0, 0.0, 0.05, 2, 4, 20, 40, 7, 30, 0.5, 0.0, 2, 0.0, 1, 1, 0, 30, True),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", FLAT_CASES, ids=[c[0] for c in FLAT_CASES])
def test_engine_matches_oracle_through_flat_events(engine_lib, oracle_lib, case):
    """Runs that reach many flat events, so that the flatness vote, the count-weighted average
    over the replicas, the histogram reset with REDUCE_LOGDOS, the visited-bin mask, the ln f
    halving and the switch to the 1/t schedule all run on the GPU, bit for bit against the
    oracle after every check interval (rewl_simulation.hpp:361-470,541-600;
    rewl_histograms.hpp:83-152)."""
    (_, model, L, emin, emax, bw, nwin, R, se, sc, seed, cycles, K, sig, flat_mode, flat_param, mask, oot, wpw,
     min_events, want_oot) = case
    fields = None
    if sig > 0:
        fields = np.round(np.random.default_rng(seed).normal(0, sig, L * L) * 2**20) / 2**20
    eng, orc = _pair(engine_lib, oracle_lib, model, L, emin, emax, bw, nwin, R, se, sc, seed, K=K, fields=fields,
                     flat=flat_param, mask=mask, flat_mode=flat_mode, walkers_per_warp=wpw, one_over_t=oot,
                     lnf_final=1e-12)
    try:
        _compare(eng, orc, "init")
        events = 0
        for k in range(cycles):
            eng.run_cycles(1)
            events += orc.cycle()
            if cycles <= 60 or k % 10 == 9 or k == cycles - 1:
                _compare(eng, orc, f"cycle {k}")
        st = eng.status()
        assert st.flat_events == events
        assert events >= min_events, events
        assert _one_over_t_engaged(orc) == want_oot
        for w in range(nwin):
            np.testing.assert_array_equal(eng.window_mask(0, w), orc.window_mask(w), err_msg=f"window {w} mask")
    finally:
        eng.close()
        orc.close()


def _layout_fields(L, seed):
    return np.round(np.random.default_rng(seed).normal(0.0, 0.5, L * L) * 2**20) / 2**20


LAYOUTS = [
    # name, model, L, K, emin, emax, bw, nwin, R, se, sc, mask, cycles
    # batched Ising L = 32: 16 windows x 8 walkers, exchange every 500 sweeps, check every 1000
    ("ising_L32_16x8", 0, 32, 0.0, -2048.0, 2052.0, 4.0, 16, 8, 500, 1000, 0, 2),
    # one realisation of Ashkin-Teller L = 32, K = 0.5, Baxter fields sigma 0.5, bins of 0.05
    # (37,237 per window): 8 windows x 4 walkers
    ("at_L32_K05_h05_8x4", 1, 32, 0.5, -5120.0, 0.0, 0.05, 8, 4, 100, 200, 1, 2),
    # Ising L = 64 over the whole spectrum: 64 windows x 8 walkers
    ("ising_L64_64x8", 0, 64, 0.0, -8192.0, 8196.0, 4.0, 64, 8, 500, 1000, 0, 1),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", LAYOUTS, ids=[c[0] for c in LAYOUTS])
def test_benchmark_layouts_match_oracle(engine_lib, oracle_lib, case):
    """The benchmark configurations themselves, one or two check intervals of their own sweep
    and exchange intervals, bit for bit against the oracle (run on all host cores).  The Ising
    layouts go flat many times already at ln f = 1."""
    import os
    _, model, L, K, emin, emax, bw, nwin, R, se, sc, mask, cycles = case
    fields = _layout_fields(L, 100) if model == 1 else None
    eng, orc = _pair(engine_lib, oracle_lib, model, L, emin, emax, bw, nwin, R, se, sc, 1001, K=K,
                     fields=fields, mask=mask, lnf_final=1e-8, nthreads=os.cpu_count() or 1)
    try:
        _compare(eng, orc, "init")
        events = 0
        for k in range(cycles):
            eng.run_cycles(1)
            events += orc.cycle()
            _compare(eng, orc, f"cycle {k}")
        assert eng.status().flat_events == events
        att, acc = orc.exchange_stats()
        st = eng.status()
        assert (st.exchanges_attempted, st.exchanges_accepted) == (att, acc)
    finally:
        eng.close()
        orc.close()


@pytest.mark.gpu
def test_nearby_seeds_give_unrelated_walker_streams(engine_lib, oracle_lib):
    """Instances seeded 2 and 3 in one batch: before the seed was mixed into the Philox key, the
    walker keys (seed ^ walker) of the two coincided, swapped, and the runs were identical.  Each
    must match its own oracle, and the two must differ."""
    rg, po = engine_lib, oracle_lib
    inss = [rg.Instance(model=0, L=4, energy_min=-32.0, energy_max=36.0, bin_width=4.0, num_windows=1,
                        replicas_per_window=2, seed=sd) for sd in (2, 3)]
    b = rg.Batch(instances=inss, sweeps_per_exchange=20, sweeps_per_check=40, lnf_final=1e-7)
    with rg.Engine(b) as eng:
        orcs = [po.Oracle(po.Config(model=0, L=4, nwin=1, R=2, sweeps_per_exchange=20, sweeps_per_check=40,
                                    emin=-32.0, emax=36.0, bw=4.0, lnf_final=1e-7, semantics=po.SEM_ENGINE,
                                    seed=sd)) for sd in (2, 3)]
        for _ in range(3):
            eng.run_cycles(1)
            for o in orcs:
                o.cycle()
        tabs = []
        for i, o in enumerate(orcs):
            for r in range(2):
                out = eng.export_walker(eng.walker_id(i, 0, r))
                c, g, _ = o.tables(r)
                np.testing.assert_array_equal(out["counts"], c)
                np.testing.assert_array_equal(out["logdos"], g)
                np.testing.assert_array_equal(out["dofs"], o.dofs(r))
                tabs.append(out["counts"])
        assert not np.array_equal(tabs[0], tabs[3]) and not np.array_equal(tabs[1], tabs[2])
        for o in orcs:
            o.close()


LEAN_CASES = [c for c in CASES if c[0] in ("ising_L8_3x2", "ising_L16_4x3", "ising_L64_2x2")]


@pytest.mark.gpu
@pytest.mark.parametrize("walkers_per_warp", [2, 4])
@pytest.mark.parametrize("case", LEAN_CASES, ids=[c[0] for c in LEAN_CASES])
def test_lean_chain_matches_oracle(engine_lib, oracle_lib, monkeypatch, case, walkers_per_warp):
    """The bin-tracking kernel's lean chain (the next proposal read after each step's write, no
    candidate prefetch), which the engine takes for warps of several walkers from 5 warps per SM
    on, forced on for small cases: bit for bit against the oracle."""
    monkeypatch.setenv("REWL_BINS_LEAN", "1")
    test_engine_matches_oracle_ising(engine_lib, oracle_lib, case, walkers_per_warp)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in FLAT_CASES if c[0].endswith("2perwarp")], ids=lambda c: c[0])
def test_lean_chain_through_flat_events(engine_lib, oracle_lib, monkeypatch, case):
    monkeypatch.setenv("REWL_BINS_LEAN", "1")
    test_engine_matches_oracle_through_flat_events(engine_lib, oracle_lib, case)


@pytest.mark.gpu
def test_benchmark_layout_32_walkers_per_window(engine_lib, oracle_lib):
    """Ising L = 64, 64 windows x 32 walkers (2048 walkers, two per warp: the lean chain by
    occupancy), one check interval of its own sweep and exchange intervals, against the oracle."""
    test_benchmark_layouts_match_oracle(engine_lib, oracle_lib,
                                        ("ising_L64_64x32", 0, 64, 0.0, -8192.0, 8196.0, 4.0, 64, 32, 500, 1000, 0, 1))
