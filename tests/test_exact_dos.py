"""Exact 2D Ising density of states (Beale) pinned by brute force and identities."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import beale


def test_beale_matches_brute_force_L4():
    bf = beale.brute_force_dos(4)
    g = beale.exact_dos(4)
    N = 16
    for k, v in enumerate(g):
        assert v == bf.get(-2 * N + 4 * k, 0)


@pytest.mark.parametrize("L", [4, 6, 8, 16])
def test_beale_identities(L):
    g = beale.exact_dos(L)
    N = L * L
    assert sum(g) == 2 ** N
    assert g[0] == 2 and g[1] == 0 and g[2] == 2 * N and g[3] == 4 * N
    if L >= 5:
        assert g[4] == N * N + 9 * N
    else:
        assert g[4] == N * N + 9 * N + 24
    assert g == g[::-1]
    assert all(v > 0 for v in g[2:-2])


@pytest.mark.parametrize("L", [4, 6, 8, 16, 24, 32, 64])
def test_exact_fixture_consistent(L):
    z = np.load(GOLDEN / f"exact_ising_L{L}.npz")
    E, lng = z["E"], z["lng"]
    N = L * L
    assert E[0] == -2 * N and E[-1] == 2 * N and len(E) == N - 1
    m = lng.max()
    assert abs(m + np.log(np.exp(lng - m).sum()) - N * np.log(2.0)) < 1e-9 * N
    np.testing.assert_allclose(lng, lng[::-1], rtol=0, atol=1e-9)
    assert abs(lng[0] - np.log(2.0)) < 1e-12
    if L <= 24:
        E2, lng2 = beale.exact_lng(L)
        np.testing.assert_array_equal(E, E2)
        np.testing.assert_allclose(lng, lng2, rtol=0, atol=1e-12)


def test_brute_force_L5_identities():
    """L = 5 (2^25 states, odd: no E -> -E symmetry): the low-energy counts that the identities
    for L >= 5 state, checked by enumeration."""
    bf = beale.brute_force_dos(5)
    N = 25
    assert sum(bf.values()) == 2 ** N
    assert bf[-2 * N] == 2 and -2 * N + 4 not in bf
    assert bf[-2 * N + 8] == 2 * N and bf[-2 * N + 12] == 4 * N and bf[-2 * N + 16] == N * N + 9 * N
