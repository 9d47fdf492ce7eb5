"""Window concatenation + normalisation (rewl_concatenate_windows, host only) against the
reference's own concatenate_tables (multiple overlap) and normalize_logDoS, run by the reference
harness on the same tables, observables averaged over the overlaps included
(tests/golden/concatenate.npz, written by tests/golden/make_golden.py concatenate).

The reference's splice search takes abs() of a double difference of derivatives in a translation
unit where that resolves to the C library's int abs(int), so the difference is truncated to an
integer.  REWL_MATCH_REFERENCE reproduces that bit for bit; REWL_MATCH_DERIVATIVE (the engine's
rule) minimises the true difference and is checked against a restatement here."""
import math

import numpy as np
import pytest

from conftest import GOLDEN


_Z = np.load(GOLDEN / "concatenate.npz")
NAMES = sorted({k.split(".")[0] for k in _Z.files})


def _case(name):
    c = {k.split(".", 1)[1]: _Z[k] for k in _Z.files if k.startswith(name + ".")}
    spp, N, half, K = c["meta"]
    c.update(states_per_site=float(spp), system_size=int(N), half_spectrum=bool(half), num_obs=int(K))
    return c


def _windows(c, with_obs=False):
    out, k, K = [], 0, c["num_obs"]
    for n in c["sizes"]:
        w = (c["energies"][k:k + n], c["logdos"][k:k + n])
        out.append(w + (c["obs"][k * K:(k + n) * K].reshape(n, K),) if with_obs else w)
        k += n
    return out


def _deriv(i, f, a):
    n = len(f)
    if i == 0:
        return (f[1] - f[0]) / (a[1] - a[0])
    if i == n - 1:
        return (f[i] - f[i - 1]) / (a[i] - a[i - 1])
    if i in (1, n - 2):
        return (f[i + 1] - f[i - 1]) / (2. * (a[i] - a[i - 1]))
    return (-f[i + 2] + 8. * f[i + 1] - 8. * f[i - 1] + f[i - 2]) / (12. * (a[i] - a[i - 1]))


def _restated(windows, spp, N, half, truncate):
    """concatenate_tables (multiple overlap) + normalize_logDoS, step for step."""
    fe, fg = list(windows[0][0]), list(windows[0][1])
    gap = (lambda d: float(abs(int(d)))) if truncate else abs
    for er, gr in windows[1:]:
        ls = max(k for k in range(len(fe)) if fe[k] == er[0])
        best, cl = gap(_deriv(ls, fg, fe) - _deriv(0, gr, er)), ls
        for i in range(1, len(fe) - ls):
            v = gap(_deriv(ls + i, fg, fe) - _deriv(i, gr, er))
            if v + 0.5 < best + 0.5:
                best, cl = v, ls + i
        shift = fg[cl] - gr[cl - ls]
        for k in range(cl + 1, len(fe)):
            fg[k] = gr[k - ls] + shift
        for k in range(len(fe) - ls, len(er)):
            fe.append(er[k])
            fg.append(gr[k] + shift)
    mx = 0.0
    for v in fg:
        mx = mx if mx > v else v
    s = 0.0
    for v in fg:
        s += math.exp(-(mx - v))
    s = math.log(s) + mx
    sh = N * math.log(spp) - s - math.log(2.) * (1.0 if half else 0.0)
    return np.array(fe), np.array([v + sh for v in fg])


@pytest.mark.parametrize("case", NAMES)
def test_reference_rule_is_bit_identical_to_the_reference(engine_lib, case):
    rg = engine_lib
    c = _case(case)
    E, G, O = rg.concatenate_windows(_windows(c, True), c["states_per_site"], c["system_size"], c["half_spectrum"],
                                     rg.MATCH_REFERENCE)
    assert np.array_equal(E, c["out_energies"])
    assert np.array_equal(G.view(np.uint64), c["out_logdos"].view(np.uint64))
    assert np.array_equal(O.ravel().view(np.uint64), c["out_obs"].view(np.uint64))
    # the restatement of the reference's rule agrees, so the one of the engine's rule is trusted
    rE, rG = _restated(_windows(c), c["states_per_site"], c["system_size"], c["half_spectrum"], True)
    assert np.array_equal(rE, c["out_energies"]) and np.allclose(rG, c["out_logdos"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", NAMES)
def test_derivative_rule_matches_its_restatement(engine_lib, case):
    rg = engine_lib
    c = _case(case)
    E, G = rg.concatenate_windows(_windows(c), c["states_per_site"], c["system_size"], c["half_spectrum"])
    rE, rG = _restated(_windows(c), c["states_per_site"], c["system_size"], c["half_spectrum"], False)
    assert np.array_equal(E, rE) and np.allclose(G, rG, rtol=0, atol=1e-12)


def test_the_two_rules_differ_on_noisy_windows(engine_lib):
    rg = engine_lib
    c = _case("ising_L16_3win")
    _, a = rg.concatenate_windows(_windows(c), 2.0, 256, False, rg.MATCH_REFERENCE)
    _, b = rg.concatenate_windows(_windows(c), 2.0, 256, False, rg.MATCH_DERIVATIVE)
    assert np.abs(a - b).max() > 0.01


def test_windows_that_do_not_overlap_are_refused(engine_lib):
    rg = engine_lib
    w = [(np.array([0.0, 4.0, 8.0]), np.zeros(3)), (np.array([12.0, 16.0, 20.0]), np.zeros(3))]
    with pytest.raises(rg.REWLError):
        rg.concatenate_windows(w, 2.0, 16)


def test_arguments_are_checked(engine_lib):
    import ctypes as C
    rg = engine_lib
    lib = rg.load_library()
    E = np.array([0.0, 4.0, 8.0, 4.0, 8.0, 12.0])
    G = np.array([0.0, 1.0, 2.0, 0.0, 1.0, 2.0])
    sizes = np.array([3, 3], dtype=np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    out_e, out_g = np.zeros(8), np.zeros(8)
    n = C.c_int32(2)                                    # too small: the needed size comes back
    assert lib.rewl_concatenate_windows(2, p(sizes), p(E), p(G), 0, None, 2.0, 16, 0, 0, p(out_e), p(out_g), None,
                                        C.byref(n)) != 0 and n.value == 4
    n = C.c_int32(8)
    assert lib.rewl_concatenate_windows(2, p(sizes), p(E), p(G), 0, None, 2.0, 16, 0, 0, p(out_e), p(out_g), None,
                                        C.byref(n)) == 0 and n.value == 4
    assert np.array_equal(out_e[:4], [0.0, 4.0, 8.0, 12.0])
    for bad in (dict(match=7), dict(num_obs=2), dict(sizes=np.array([1, 3], dtype=np.int32))):
        n = C.c_int32(8)
        s = bad.get("sizes", sizes)
        assert lib.rewl_concatenate_windows(2, p(s), p(E), p(G), bad.get("num_obs", 0), None, 2.0, 16, 0,
                                            bad.get("match", 0), p(out_e), p(out_g), None, C.byref(n)) != 0, bad
