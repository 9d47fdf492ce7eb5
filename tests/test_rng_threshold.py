"""Random streams and the integer acceptance threshold of the engine semantics."""
import math
import struct

import numpy as np
import pytest


def test_philox_known_answers(oracle_lib):
    # Known-answer vectors of Philox4x32-10 (Salmon et al., SC'11, Random123 kat_vectors)
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        got = oracle_lib.philox4x32_10(ctr, key)
        assert [int(x) for x in got] == want


def test_neglog_accuracy(oracle_lib):
    rng = np.random.default_rng(0)
    xs = list(rng.integers(0, 2**32, 20000, dtype=np.uint64)) + [0, 1, 2, 3, 2**31, 2**32 - 1, 2**32 - 2]
    for x in xs:
        x = int(x)
        u = (2 * (x >> 1) + 1) / 2.0**32
        want = -math.log(u)
        got = oracle_lib.neglog_u32(x)
        assert got > 0
        assert abs(got - want) <= 4e-7 * max(1.0, want), (x, got, want)


def f32(x: float) -> float:
    return struct.unpack("f", struct.pack("f", x))[0]


def _float_lt(d: int, thr: float) -> bool:
    """float(d * 2^-36) < thr with IEEE round-to-nearest-even (numpy float32)."""
    return bool(np.float32(np.float64(d) * 2.0**-36) < np.float32(thr))


def test_accept_threshold_exact(oracle_lib):
    rng = np.random.default_rng(1)
    thrs = [oracle_lib.neglog_u32(int(x)) for x in rng.integers(0, 2**32, 300, dtype=np.uint64)]
    thrs += [1.0, 2.0, 0.5, 2.0**-20, 2.0**-30, 22.0, f32(0.1), f32(1.0 / 3.0)]
    for thr in thrs:
        T = oracle_lib.accept_threshold(thr)
        assert T >= 1
        # boundary: d = T-1 accepted, d = T rejected; and a few around
        for d in (T - 3, T - 2, T - 1, T, T + 1, T + 2):
            if d < 1:
                continue
            assert (d < T) == _float_lt(d, thr), (thr, T, d)
        for d in rng.integers(1, max(2, 4 * T), 50):
            assert (int(d) < T) == _float_lt(int(d), thr), (thr, T, int(d))


def _splitmix64_finaliser(seed: int) -> int:
    """SplitMix64's output function (Steele, Lea, Flood, OOPSLA 2014), the instance-key mix."""
    m = (1 << 64) - 1
    z = (seed + 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


def test_nearby_seeds_give_distinct_walker_keys():
    """Walker keys are (key_lo ^ walker, key_hi) with key = mix(seed).  Without the mix, seeds
    that differ in bits below the walker count handed their walkers each other's keys; with it,
    no two walkers of a thousand consecutive seeds x 64 walkers share a key."""
    keys = set()
    for seed in range(1000):
        k = _splitmix64_finaliser(seed)
        for w in range(64):
            keys.add(((k & 0xFFFFFFFF) ^ w, k >> 32))
    assert len(keys) == 1000 * 64
    assert _splitmix64_finaliser(0) == 0xE220A8397B1DCDAF       # SplitMix64's first output from state 0


def test_seeds_two_and_three_no_longer_run_identically(oracle_lib):
    po = oracle_lib
    runs = []
    for seed in (2, 3):
        cfg = po.Config(model=po.MODEL_ISING, L=4, nwin=1, R=2, sweeps_per_exchange=20, sweeps_per_check=40,
                        emin=-32.0, emax=36.0, bw=4.0, semantics=po.SEM_ENGINE, seed=seed)
        orc = po.Oracle(cfg)
        for _ in range(3):
            orc.cycle()
        runs.append([orc.tables(s)[0].copy() for s in range(2)])
        orc.close()
    assert not np.array_equal(runs[0][0], runs[1][1]) and not np.array_equal(runs[0][1], runs[1][0])
    assert not np.array_equal(runs[0][0], runs[1][0])


def test_engine_and_oracle_share_the_logdos_unit():
    """The engine (rng.cuh) and the oracle restate the logDoS unit separately: they must agree,
    and the tests above check the boundary at that unit."""
    import re
    from conftest import ROOT
    rng = (ROOT / "rewl_simulator_gb300" / "csrc" / "rng.cuh").read_text()
    orc = (ROOT / "oracle" / "rewl_oracle.cpp").read_text()
    bits = int(re.search(r"kLogdosBits = (\d+);", rng).group(1))
    scale = float(re.search(r"kLogdosScale = ([0-9.]+);", rng).group(1))
    qbits = int(re.search(r"QBITS = (\d+);", orc).group(1))
    qscale = float(re.search(r"QSCALE = ([0-9.]+);", orc).group(1))
    assert bits == qbits == 36 and scale == qscale == 2.0 ** bits
    assert f"const int sh = s + {bits};" in orc
