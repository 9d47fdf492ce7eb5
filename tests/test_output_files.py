"""Output files in the reference's text formats.

tests/golden/writers/ holds files written by the reference's own writers
(write_microcanonical_observables, write_observables_to_file,
write_nonlinear_obs_to_file; tests/golden/make_golden.py writers).  The library's
writers, given the same arrays, must produce the same bytes.  On the GPU, the
end-to-end post-processing of an engine is checked against its parts.
"""
import numpy as np
import pytest

from conftest import GOLDEN

HEADER = "# Model: 2D Ising, L = 16\n# REWL: 4 windows, 75 % overlap\n"
NAMES = ["Magnetization", "Magnetization2", "Magnetization4", "Counts per Bin"]
THERMAL = ["Free Energy", "Energy", "Energy2", "Entropy", "Specific Heat"] + NAMES


def test_writers_match_the_reference_byte_for_byte(engine_lib, tmp_path):
    from rewl_simulator_gb300 import output
    z = np.load(GOLDEN / "thermo_ising.npz")
    T, out = z["temperatures"], z["out"]
    files = [output.write_table("microcanonical", tmp_path, "golden", HEADER, NAMES, z["E"], z["obs"], z["lng"], 256.0),
             output.write_table("self_averaged", tmp_path, "golden", HEADER, THERMAL, T, out),
             output.write_table("nonlinear", tmp_path, "golden", HEADER, ["Susceptibility", "Binder Cumulant"], T,
                                out[:, 5:7])]
    for f in files:
        assert f.read_bytes() == (GOLDEN / "writers" / f.name).read_bytes(), f.name


@pytest.mark.gpu
def test_write_outputs_end_to_end(engine_lib, tmp_path):
    rg = engine_lib
    from rewl_simulator_gb300 import output, thermo
    ins = rg.Instance(model=0, L=8, energy_min=-128.0, energy_max=132.0, bin_width=4.0, num_windows=3,
                      replicas_per_window=2, seed=5)
    b = rg.Batch(instances=[ins], sweeps_per_exchange=100, sweeps_per_check=200, lnf_final=1e-4, observables=1)
    with rg.Engine(b) as eng:
        eng.simulate(max_cycles=2000)
        files = output.write_outputs(eng, 0, tmp_path, "ising_L8", header="# test\n", num_T=500)
        assert [f.name.split("-")[0] for f in files] == ["microcanonical_observables", "self_averaged_observables",
                                                        "nonlinear_observables"]
        E, lng = eng.global_logdos(0)
        obs = output.global_observables(eng, 0)
    micro = np.loadtxt(files[0], delimiter=",", comments="#")
    np.testing.assert_allclose(micro[:, 0], E / 64, rtol=1e-14)
    np.testing.assert_allclose(micro[:, 1], lng / 64, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(micro[:, 2:], obs, rtol=1e-14)
    # counts on the concatenated axis are the visits summed over a window's replicas, then averaged
    # over the windows holding the energy; every level of a converged run was visited
    assert np.all(micro[:, -1] > 0)
    T, rows = thermo.thermodynamics(E, lng, 64, obs=obs, counts_col=3, num_T=500)
    sa = np.loadtxt(files[1], delimiter=",", comments="#")
    np.testing.assert_allclose(sa[:, 0], T, rtol=1e-14)
    np.testing.assert_allclose(sa[:, 1:], rows, rtol=1e-13, atol=1e-300)
    nl = np.loadtxt(files[2], delimiter=",", comments="#")
    np.testing.assert_allclose(nl[:, 1:], thermo.nonlinear(0, T, rows, 64), rtol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("model", [0, 1])
def test_write_outputs_with_correlators(engine_lib, tmp_path, model):
    """observables = 2, the reference's default CORRELATION_LENGTHS build: the microcanonical and
    self-averaged files carry the G(q_min) columns named as the reference names them, and the
    nonlinear file the correlation lengths over L."""
    rg = engine_lib
    from rewl_simulator_gb300 import output, thermo
    if model == 0:
        ins = rg.Instance(model=0, L=8, energy_min=-128.0, energy_max=132.0, bin_width=4.0, num_windows=3,
                          replicas_per_window=2, seed=5)
        N, K = 64, 4
    else:
        h = np.round(np.random.default_rng(3).normal(0, 0.5, 16) * 2**20) / 2**20
        # one window: at L = 4 the visited bins of two windows need not overlap
        ins = rg.Instance(model=1, L=4, K=0.5, fields=h, energy_min=-80.0, energy_max=0.0, bin_width=0.05,
                          num_windows=1, replicas_per_window=2, seed=5)
        N, K = 16, 16
    # with random fields many bins are unreachable: flatness over the visited bins
    b = rg.Batch(instances=[ins], sweeps_per_exchange=50, sweeps_per_check=100, lnf_final=1e-3, observables=2,
                 mask_mode=0 if model == 0 else rg.MASK_VISITED)
    with rg.Engine(b) as eng:
        eng.simulate(max_cycles=400)
        files = output.write_outputs(eng, 0, tmp_path, "corr", header="# test\n", num_T=300)
        E, lng = eng.global_logdos(0, half_spectrum=model == 1)
        obs = output.global_observables(eng, 0)
    assert obs.shape[1] == K + 1
    micro_text = files[0].read_text()
    assert ("G(qmin)" in micro_text) if model == 0 else all(
        f"{x} G(qmin)" in micro_text for x in ("Sigma", "Tau", "Phi", "Baxter"))
    micro = np.loadtxt(files[0], delimiter=",", comments="#")
    np.testing.assert_allclose(micro[:, 2:], obs, rtol=1e-14)
    g_cols = [3] if model == 0 else [3, 7, 11, 15]
    assert np.all(obs[:, g_cols] >= 0) and np.any(obs[:, g_cols] > 0)
    if model == 1:
        # tau's correlator is computed from sigma, as the reference does; phi's is the sum
        np.testing.assert_array_equal(obs[:, 7], obs[:, 3])
        np.testing.assert_allclose(obs[:, 11], 2 * obs[:, 3], rtol=1e-15)
    T, rows = thermo.thermodynamics(E, lng, N, obs=obs, counts_col=K, num_T=300)
    nl = np.loadtxt(files[2], delimiter=",", comments="#")
    assert nl.shape[1] == 1 + (3 if model == 0 else 12)
    np.testing.assert_allclose(nl[:, 1:], thermo.nonlinear(model, T, rows, N, correlators=True), rtol=1e-13)
    assert "Correlation Length over L" in files[2].read_text()
