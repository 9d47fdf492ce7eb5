"""Ashkin-Teller ln g within the walker-to-walker spread of the reference's algorithm (CPU).

The oracle runs the REWL path in the reference's semantics (its walker, mt19937_64 stream and
float acceptance test, pinned bit for bit to the reference by the replay fixtures) and in the
engine's (Philox, integer logDoS; the GPU matches it bit for bit).  Eight independent reference
runs of one Ashkin-Teller instance (L = 4, K = 0.5, Baxter fields sigma 0.5, 1/t down to
ln f < 1e-5) give the run-to-run spread; each engine run must lie as close to the reference mean
as a reference run held out from it does, and the engine mean must agree with the reference mean
to within the spread."""
import numpy as np
import pytest

L, K = 4, 0.5
N = L * L


def _run(po, sem, seed, fields):
    cfg = po.Config(model=po.MODEL_AT, L=L, K=K, escale_bits=20, nwin=1, R=2, sweeps_per_exchange=100,
                    sweeps_per_check=400, emin=-(2 + K) * 2 * N, emax=0.0, bw=0.25, lnf_final=1e-5, one_over_t=1,
                    mask_mode=po.MASK_VISITED, semantics=sem, seed=seed)
    orc = po.Oracle(cfg, fields=fields)
    for _ in range(20000):
        orc.cycle()
        if orc.all_done():
            break
    done = orc.all_done()
    g, m = orc.window_logdos(0), orc.window_mask(0).astype(bool)
    orc.close()
    assert done
    x = g[m]
    mx = x.max()
    return x - (mx + np.log(np.exp(x - mx).sum())) + N * np.log(4.0) - np.log(2.0), m    # half spectrum


def test_engine_semantics_within_the_reference_spread(oracle_lib):
    po = oracle_lib
    h = np.round(np.random.default_rng(77).normal(0.0, 0.5, N) * 2**20) / 2**20
    refs, mask = [], None
    for seed in range(1, 9):
        lng, m = _run(po, po.SEM_REFERENCE, seed, h)
        assert mask is None or np.array_equal(m, mask)
        mask = m
        refs.append(lng)
    R = np.array(refs)
    # a held-out reference run's RMS distance from the mean of the other seven
    d_ref = [np.sqrt(np.mean((R[k] - np.delete(R, k, 0).mean(0)) ** 2)) for k in range(len(R))]
    mu = R.mean(0)
    engs = []
    for seed in (1 << 20, 2 << 20, 3 << 20, 4 << 20):         # seeds 2^20 apart: distinct walker keys
        lng, m = _run(po, po.SEM_ENGINE, seed, h)
        assert np.array_equal(m, mask)
        engs.append(lng)
        assert np.sqrt(np.mean((lng - mu) ** 2)) <= 1.5 * max(d_ref), (np.sqrt(np.mean((lng - mu) ** 2)), d_ref)
    # no systematic offset: the engine mean sits within the spread of one run
    assert np.sqrt(np.mean((np.mean(engs, 0) - mu) ** 2)) <= np.median(d_ref)
