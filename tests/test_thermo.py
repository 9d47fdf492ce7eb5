"""Canonical thermodynamics (FP64 log-sum-exp over temperatures).

The golden fixtures are the reference's own Thermodynamics::calculate_thermodynamics
(src/Thermodynamics/thermodynamics.hpp, compiled by oracle/build_ref.py,
tests/golden/make_golden.py thermo), with and without the trapezoidal rule.  The FP64
restatement in oracle/thermo_ref.py is pinned against them; the GPU kernel is checked
against them too.  Tolerances: 1e-12 relative, except the specific heat
C = N (U2 - U^2) / T^2, whose cancellation at low T is judged against N U2 / T^2.
"""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import build_ref, thermo_ref

CASES = ["thermo_ising", "thermo_at", "thermo_ising_plain", "thermo_at_plain"]


def _check(T, out, z, rtol=1e-12):
    N = float(z["N"])
    ref = z["out"]
    np.testing.assert_array_equal(T, z["temperatures"])
    cols = [k for k in range(ref.shape[1]) if k != 4]
    np.testing.assert_allclose(out[:, cols], ref[:, cols], rtol=rtol, atol=0)
    scale = N * np.abs(ref[:, 2]) / T ** 2
    assert np.all(np.abs(out[:, 4] - ref[:, 4]) <= 1e-11 * scale + rtol * np.abs(ref[:, 4]))


def _args(z):
    return (z["E"], z["lng"], z["obs"], float(z["N"]), float(z["Tmin"]), float(z["Tmax"]), int(z["nT"]),
            int(z["counts_col"]), bool(z["trapezoid"]))


@pytest.mark.parametrize("name", CASES)
def test_restatement_matches_reference_fixtures(name):
    z = np.load(GOLDEN / f"{name}.npz")
    T, out = thermo_ref.thermodynamics(*_args(z))
    _check(T, out, z)


@pytest.mark.skipif(not build_ref.reference_available(), reason="reference sources not present")
def test_restatement_matches_live_reference_harness():
    import ctypes as C
    lib = C.CDLL(str(build_ref.build_thermo(trapezoid=True)))
    lib.ref_thermo.argtypes = [C.c_int, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_double,
                               C.c_double, C.c_size_t, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(3)
    E = np.sort(rng.uniform(-200, 50, 300))
    lng = 30 * np.sin(E / 70.0) + 0.001 * E ** 2
    obs = np.ascontiguousarray(np.stack([rng.uniform(0, 1, 300) for _ in range(3)] + [rng.integers(1, 9, 300)], 1)
                               .astype(np.float64))
    nT = 700
    out, T = np.zeros((nT, 9)), np.zeros(nT)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.ref_thermo(0, 300, p(E), p(lng), p(obs), 64, 0.05, 20.05, nT, p(out), p(T))
    T2, mine = thermo_ref.thermodynamics(E, lng, obs, 64.0, 0.05, 20.05, nT, 3, True)
    _check(T2, mine, {"N": 64, "out": out, "temperatures": T})


def test_nonlinear_observables_host(engine_lib):
    from rewl_simulator_gb300 import thermo
    for name in ("thermo_ising", "thermo_at"):
        z = np.load(GOLDEN / f"{name}.npz")
        model = int(z["model"])
        got = thermo.nonlinear(model, z["temperatures"], z["out"], int(z["N"]))
        ref = thermo_ref.nonlinear(model, z["out"], z["temperatures"], float(z["N"]))
        np.testing.assert_allclose(got, ref, rtol=1e-14, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_thermodynamics_matches_reference(engine_lib, name):
    from rewl_simulator_gb300 import thermo
    z = np.load(GOLDEN / f"{name}.npz")
    T, out = thermo.thermodynamics(z["E"], z["lng"], int(z["N"]), obs=z["obs"], counts_col=int(z["counts_col"]),
                                   Tmin=float(z["Tmin"]), Tmax=float(z["Tmax"]), num_T=int(z["nT"]),
                                   trapezoid=bool(z["trapezoid"]))
    _check(T, out, z)


@pytest.mark.gpu
def test_gpu_thermodynamics_reference_ladder_on_exact_L64(engine_lib):
    """The reference's own run shape: 50,000 temperatures over the exact L = 64 ln g."""
    from rewl_simulator_gb300 import thermo
    zz = np.load(GOLDEN / "exact_ising_L64.npz")
    ok = np.isfinite(zz["lng"])
    E, lng = zz["E"][ok].astype(np.float64), zz["lng"][ok]
    T, out = thermo.thermodynamics(E, lng, 4096)
    pick = np.arange(0, 50000, 997)
    T2, ref = thermo_ref.thermodynamics(E, lng, None, 4096.0, 0.01, 50.01, 50000)
    _check(T[pick], out[pick], {"N": 4096, "out": ref[pick], "temperatures": T2[pick]})
    # the specific-heat peak sits near the critical temperature 2 / ln(1 + sqrt 2) = 2.269
    assert abs(T[np.argmax(out[:, 4])] - 2.269) < 0.05


def test_cumulants_pinned_to_reference():
    """The restatement's susceptibility, Binder cumulants and correlation length over L against
    the reference's order_parameter_cumulants.hpp (tests/golden/cumulants.npz), including the
    DBL_MAX / L of a vanishing G and the NaN of G above <m^2>."""
    z = np.load(GOLDEN / "cumulants.npz")
    N = int(z["N"])
    got = np.stack([thermo_ref.susceptibility(z["m2"], z["m"], z["T"], float(N)),
                    thermo_ref.binder(z["m4"], z["m2"]), thermo_ref.binder_two_component(z["m4"], z["m2"]),
                    thermo_ref.correlation_length_over_L(z["m2"], z["G"], N)], axis=1)
    np.testing.assert_array_equal(got, z["out"])


def _rows_with_correlators(model, nT, seed):
    rng = np.random.default_rng(seed)
    groups = 1 if model == 0 else 4
    cols = []
    for _ in range(groups):
        m = rng.uniform(0.05, 0.95, nT)
        m2 = m * m + rng.uniform(0.0, 0.05, nT)
        cols += [m, m2, m2 * m2 + rng.uniform(0.0, 0.05, nT), m2 * rng.uniform(0.01, 0.9, nT)]
    thermal = rng.uniform(-2, 2, (nT, 5))
    counts = rng.integers(1, 100, (nT, 1)).astype(np.float64)
    return np.ascontiguousarray(np.concatenate([thermal, np.stack(cols, 1), counts], axis=1))


def test_nonlinear_observables_with_correlators_host(engine_lib):
    """The C ABI's correlation lengths (observables = 2 layout) against the restatement."""
    from rewl_simulator_gb300 import thermo
    for model in (0, 1):
        rows = _rows_with_correlators(model, 300, 5 + model)
        rows[0, 5 + 3] = 0.0                      # a vanishing G: DBL_MAX / L
        T = np.linspace(0.1, 5.0, 300)
        got = thermo.nonlinear(model, T, rows, 256, correlators=True)
        ref = thermo_ref.nonlinear(model, rows, T, 256.0, correlators=True)
        assert got.shape == (300, 3 if model == 0 else 12)
        np.testing.assert_allclose(got, ref, rtol=1e-14, atol=0)
