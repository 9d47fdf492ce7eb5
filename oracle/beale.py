"""Exact density of states of the 2D Ising model on an L x L torus (even L).

TEST INFRASTRUCTURE ONLY.  Restates Beale's method (P. D. Beale, "Exact
distribution of energies in the two-dimensional Ising model", PRL 76, 78
(1996)): Kaufman's finite-lattice partition function

    Z = 1/2 (2 sinh 2K)^(N/2) [Z1 + Z2 + Z3 + Z4]
    Z1 = prod_{r=0}^{L-1} 2 cosh(L g_{2r+1}/2),  Z2 = same with sinh,
    Z3 = prod_{r=0}^{L-1} 2 cosh(L g_{2r}/2),    Z4 = same with sinh,
    cosh g_l = cosh 2K coth 2K - cos(pi l / L),  g_0 = 2K + ln tanh K,

is expanded exactly as a polynomial in t = e^{2K}.  Pairing l with 2L - l
turns the products into products of 2 +- 2 T_L(cosh g_l) (T_L the Chebyshev
polynomial), which after multiplying by D^L, D = 2t(t^2 - 1), are polynomials
in t.  The two self-paired factors g_0 and g_L give
    (2cosh)(2cosh), (2sinh)(2sinh) = t^L + t^-L +- [((t-1)/(t+1))^L + ((t+1)/(t-1))^L].
Collecting powers:

    2^(N/2+1) t^N Z = prod_odd P+_l + prod_odd P-_l
                      + 2^L V+ prod_even P+_l + 2^L V- prod_even P-_l
    P+-_l = 2 D^L T_L(c_l) +- 2 D^L,   V+- = (t^2-1)^L (t^2L + 1) +- t^L [(t-1)^2L + (t+1)^2L]

and t^N Z = sum_E g(E) t^(N - E/2).  The coefficients are integers, computed
here modulo primes p = 1 (mod 2L) (where cos(pi l/L) = (z^l + z^-l)/2 with z a
primitive 2L-th root of unity exists in GF(p)) and recombined by the Chinese
remainder theorem.  Checked against brute-force enumeration at L = 4 and the
identities sum g = 2^N, g(-2N) = 2, g(-2N+4) = 0, g(-2N+8) = 2N, symmetry.
"""
from __future__ import annotations

import math

import numpy as np


def _primes_1_mod(m: int, count: int, below: int = 1 << 25):
    out = []
    k = (below - 1) // m
    while len(out) < count:
        p = k * m + 1
        k -= 1
        if p < 3:
            raise ValueError("ran out of primes")
        if _is_prime(p):
            out.append(p)
    return out


def _is_prime(n: int) -> bool:
    if n < 2:
        return False
    for q in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        if n % q == 0:
            return n == q
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in (2, 3, 5, 7, 11, 13, 17):
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def _root_of_unity(order: int, p: int) -> int:
    fac = []
    m, q = p - 1, 2
    while q * q <= m:
        if m % q == 0:
            fac.append(q)
            while m % q == 0:
                m //= q
        q += 1
    if m > 1:
        fac.append(m)
    for g in range(2, p):
        if all(pow(g, (p - 1) // f, p) != 1 for f in fac):
            return pow(g, (p - 1) // order, p)
    raise ValueError("no generator")


def _mul(a: np.ndarray, b: np.ndarray, p: int) -> np.ndarray:
    return np.convolve(a, b) % p


def _poly_pow(a: np.ndarray, e: int, p: int) -> np.ndarray:
    r = np.array([1], dtype=np.int64)
    while e:
        if e & 1:
            r = _mul(r, a, p)
        a = _mul(a, a, p)
        e >>= 1
    return r


def _add(a: np.ndarray, b: np.ndarray, p: int) -> np.ndarray:
    n = max(len(a), len(b))
    r = np.zeros(n, dtype=np.int64)
    r[:len(a)] += a
    r[:len(b)] += b
    return r % p


def _scale(a: np.ndarray, s: int, p: int) -> np.ndarray:
    return (a * (s % p)) % p


def _residue(L: int, p: int) -> np.ndarray:
    """g(E_k) mod p for k = 0..N, E_k = -2N + 4k."""
    N = L * L
    z = _root_of_unity(2 * L, p)
    inv2 = pow(2, p - 2, p)
    # polynomials are coefficient arrays in increasing powers of t
    D = np.array([0, p - 2, 0, 2], dtype=np.int64)               # 2t^3 - 2t
    D2 = _mul(D, D, p)
    DL = _poly_pow(D, L, p)

    def P_pm(l: int):
        c = (pow(z, l, p) + pow(z, 2 * L - l, p)) * inv2 % p     # cos(pi l / L)
        # (t^2+1)^2 - c D = t^4 - 2c t^3 + 2 t^2 + 2c t + 1
        Pl = np.array([1, 2 * c % p, 2, (p - 2 * c % p) % p, 1], dtype=np.int64)
        q_prev = np.array([1], dtype=np.int64)
        q = Pl.copy()
        for _ in range(1, L):
            q_next = _add(_scale(_mul(Pl, q, p), 2, p), _scale(_mul(D2, q_prev, p), p - 1, p), p)
            q_prev, q = q, q_next
        twoQ = _scale(q, 2, p)
        twoD = _scale(DL, 2, p)
        return _add(twoQ, twoD, p), _add(twoQ, _scale(twoD, p - 1, p), p)

    prod = {"op": np.array([1], dtype=np.int64), "om": np.array([1], dtype=np.int64),
            "ep": np.array([1], dtype=np.int64), "em": np.array([1], dtype=np.int64)}
    for l in range(1, L, 2):
        pp, pm = P_pm(l)
        prod["op"] = _mul(prod["op"], pp, p)
        prod["om"] = _mul(prod["om"], pm, p)
    for l in range(2, L - 1, 2):
        pp, pm = P_pm(l)
        prod["ep"] = _mul(prod["ep"], pp, p)
        prod["em"] = _mul(prod["em"], pm, p)
    t2m1L = _poly_pow(np.array([p - 1, 0, 1], dtype=np.int64), L, p)        # (t^2 - 1)^L
    t2L1 = np.zeros(2 * L + 1, dtype=np.int64)
    t2L1[0] = 1
    t2L1[2 * L] = 1
    A = _mul(t2m1L, t2L1, p)
    B = _add(_poly_pow(np.array([p - 1, 1], dtype=np.int64), 2 * L, p),
             _poly_pow(np.array([1, 1], dtype=np.int64), 2 * L, p), p)
    B = np.concatenate([np.zeros(L, dtype=np.int64), B])                    # t^L * (...)
    Vp = _add(A, B, p)
    Vm = _add(A, _scale(B, p - 1, p), p)
    twoL = pow(2, L, p)
    total = _add(prod["op"], prod["om"], p)
    total = _add(total, _scale(_mul(Vp, prod["ep"], p), twoL, p), p)
    total = _add(total, _scale(_mul(Vm, prod["em"], p), twoL, p), p)
    full = np.zeros(2 * N + 1, dtype=np.int64)
    full[:min(len(total), 2 * N + 1)] = total[:2 * N + 1]
    if len(total) > 2 * N + 1 and np.any(total[2 * N + 1:] % p):
        raise ArithmeticError("degree overflow")
    norm = pow(pow(2, N // 2 + 1, p), p - 2, p)
    full = full * norm % p
    # coefficient of t^(N - E/2) = t^(2N - 2k) for E = -2N + 4k
    k = np.arange(N + 1)
    return full[2 * N - 2 * k]


def exact_dos(L: int) -> list[int]:
    """Exact g(E) for E = -2N + 4k, k = 0..N (python ints), L even >= 2."""
    if L % 2 or L < 2:
        raise ValueError("even L only")
    N = L * L
    bits_needed = N + 2
    primes = _primes_1_mod(2 * L, bits_needed // 24 + 3)
    residues = [_residue(L, p).astype(object) for p in primes]
    M = 1
    acc = [0] * (N + 1)
    for p, r in zip(primes, residues):
        # incremental CRT
        inv = pow(M % p, p - 2, p)
        for i in range(N + 1):
            a = acc[i]
            t = ((int(r[i]) - a) % p) * inv % p
            acc[i] = a + M * t
        M *= p
    return acc


def exact_lng(L: int) -> tuple[np.ndarray, np.ndarray]:
    """(energies, ln g) over the reachable levels (g > 0)."""
    g = exact_dos(L)
    N = L * L
    E, lng = [], []
    for k, v in enumerate(g):
        if v > 0:
            E.append(-2 * N + 4 * k)
            lng.append(_ln_big(v))
    return np.array(E, dtype=np.int64), np.array(lng)


def _ln_big(v: int) -> float:
    b = v.bit_length()
    if b <= 1000:
        return math.log(v)
    sh = b - 900
    return math.log(v >> sh) + sh * math.log(2.0)


def brute_force_dos(L: int) -> dict[int, int]:
    """Enumerate all 2^(L*L) configurations (L <= 5), 2^20 at a time: configuration x has spin
    i = +1 where bit i is set, and E = sum over the 2N bonds of (+1 if the two bits differ, else -1)."""
    N = L * L
    bonds = [(y * L + x, y * L + (x + 1) % L) for y in range(L) for x in range(L)] + \
            [(y * L + x, ((y + 1) % L) * L + x) for y in range(L) for x in range(L)]
    hist: dict[int, int] = {}
    chunk = 1 << min(N, 20)
    for base in range(0, 1 << N, chunk):
        idx = np.arange(base, base + chunk, dtype=np.int64)
        diff = np.zeros(chunk, dtype=np.int64)
        for i, j in bonds:
            diff += ((idx >> i) ^ (idx >> j)) & 1
        vals, counts = np.unique(2 * diff - len(bonds), return_counts=True)
        for v, c in zip(vals.tolist(), counts.tolist()):
            hist[v] = hist.get(v, 0) + c
    return hist
