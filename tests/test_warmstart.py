"""Warm-start host logic (rewl_simulator_gb300/warmstart.py) on CPU, against a fake engine:
the burn-in, the plain-WL fallback of a window stalled in its warm-started stage, and the
window-relative injection of the prediction."""
from dataclasses import dataclass, field

import numpy as np
import pytest

from rewl_simulator_gb300 import warmstart as ws


@dataclass
class _Ins:
    num_windows: int
    L: int = 8
    J: float = 1.0
    K: float = 0.0
    bin_width: float = 4.0
    model: int = 0
    energy_max: float = 260.0


@dataclass
class _Batch:
    instances: list = field(default_factory=list)


class _Status:
    def __init__(self, done):
        self.all_done = done


class FakeEngine:
    """Windows whose ln f halves at the intervals listed in `flat_at` (never if absent)."""

    def __init__(self, nwin, flat_at, lnf0=1e-4):
        self.batch = _Batch([_Ins(nwin)])
        self.windows = [[(-128.0 + 40.0 * w, -128.0 + 40.0 * w + 80.0, 20) for w in range(nwin)]]
        self.lnf = {w: lnf0 for w in range(nwin)}
        self.flat_at = flat_at
        self.cycle = 0
        self.calls = []

    def status(self):
        return _Status(False)

    def run_cycles(self, n):
        self.cycle += n
        for w, at in self.flat_at.items():
            if self.cycle == at:
                self.lnf[w] /= 2
        return _Status(False)

    def window_state(self, i, w):
        return self.lnf[w], False

    def reset_histograms(self, i, w, reduce):
        self.calls.append(("reset", self.cycle, w, reduce))

    def set_logdos(self, i, w, g):
        self.calls.append(("logdos", self.cycle, w, np.asarray(g).copy()))

    def set_lnf(self, i, w, lnf):
        self.calls.append(("lnf", self.cycle, w, lnf))
        self.lnf[w] = lnf


def test_burn_in_clears_every_window_keeping_logdos():
    eng = FakeEngine(3, {})
    ws.run(eng, max_cycles=5, burn_in=2)
    resets = [c for c in eng.calls if c[0] == "reset"]
    assert [(c[1], c[2]) for c in resets] == [(1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2)]
    assert all(c[3] is False for c in resets)          # histograms only, ln g kept


def test_stalled_warm_window_falls_back_to_plain_wl():
    # window 0 goes flat at interval 2; window 1 never does in its warm-started stage
    eng = FakeEngine(2, {0: 2})
    st, fallbacks = ws.run(eng, max_cycles=12, stall_checks=4)
    assert fallbacks == 1
    touched = [c for c in eng.calls if c[0] in ("logdos", "lnf")]
    assert [c[2] for c in touched] == [1, 1]           # only the stalled window
    logdos = next(c for c in touched if c[0] == "logdos")
    assert logdos[1] == 4 and np.array_equal(logdos[3], np.zeros(20))
    assert next(c for c in touched if c[0] == "lnf")[3] == 1.0
    assert any(c[0] == "reset" and c[2] == 1 and c[1] == 4 for c in eng.calls)


def test_a_window_past_its_first_stage_is_left_alone():
    eng = FakeEngine(1, {0: 1})
    _, fallbacks = ws.run(eng, max_cycles=20, stall_checks=3)
    assert fallbacks == 0
    assert not [c for c in eng.calls if c[0] in ("logdos", "lnf")]


class FakeMLP:
    def predict(self, X):
        return (0.1 * X[:, 0] + 0.01).astype(np.float32)


def test_warm_start_injects_window_relative_prediction():
    eng = FakeEngine(2, {})
    base = ws.Baseline(np.array([-2.0, 0.0, 2.0]), np.array([0.0, 0.5, 0.0]))
    ws.warm_start(eng, FakeMLP(), 0, lnf0=3e-4, base=base)
    N = 64
    for w in range(2):
        lo, hi, nb = eng.windows[0][w]
        E = lo + 4.0 * np.arange(nb)
        from rewl_simulator_gb300.mlp import features
        f = features(E, 8, 1.0, 0.0, 0.0, lo, hi)
        pred = (FakeMLP().predict(f).astype(np.float64) + base(E / N)) * N
        got = next(c[3] for c in eng.calls if c[0] == "logdos" and c[2] == w)
        np.testing.assert_allclose(got, pred - pred[0], rtol=1e-12, atol=1e-12)
        assert got[0] == 0.0
    assert [c[3] for c in eng.calls if c[0] == "lnf"] == [3e-4, 3e-4]


# --------------------------------------------------------------------------- GPU
def _ising(rg, L, nwin, R, lnf0, seed, one_over_t=1):
    N = L * L
    ins = rg.Instance(model=rg.MODEL_ISING2D, L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                      num_windows=nwin, replicas_per_window=R, window_overlap=0.75, seed=seed, init_mode=1)
    return rg.Batch(instances=[ins], sweeps_per_exchange=100, sweeps_per_check=200, flatness_param=0.8,
                    lnf_initial=lnf0, lnf_final=1e-8, one_over_t=one_over_t)


def _exact(L):
    from conftest import GOLDEN
    z = np.load(GOLDEN / f"exact_ising_L{L}.npz")
    return dict(zip(z["E"].astype(np.int64).tolist(), z["lng"]))


def _exact_rows(eng, exact, L, base):
    """(features, residual ln g/N) over the engine's windows, the targets taken from the exact ln g."""
    from rewl_simulator_gb300.mlp import features
    N = L * L
    Xs, ys = [], []
    for w, (lo, hi, nb) in enumerate(eng.windows[0]):
        E = ws.window_energies(eng, 0, w)[eng.window_mask(0, w)]
        E = np.array([e for e in E if int(round(e)) in exact])
        Xs.append(features(E, L, 1.0, 0.0, 0.0, lo, hi))
        ys.append(np.array([exact[int(round(e))] for e in E]) / N - base(E / N))
    return np.concatenate(Xs), np.concatenate(ys).astype(np.float32)


def _max_err(eng, exact):
    E, g = eng.global_logdos(0)
    return float(np.max(np.abs([g[i] - exact[int(round(E[i]))] for i in range(len(E))])))


@pytest.mark.gpu
def test_gpu_warm_start_gain_over_plain_wang_landau(engine_lib):
    """2D Ising L=32, 16 windows x 2 walkers.  A network trained on the exact ln g of L = 8 and 16
    (residual over the L=16 ln g/N) predicts the L=32 windows: its error at injection is compared
    with the zero start of plain Wang-Landau, and plain WL (ln f0 = 1) is run until it is as
    accurate as the prediction was before a single flip; the warm-started run (ln f0 = 1e-4,
    burn-in) must keep its accuracy over the intervals before its stall fallback could act."""
    rg = engine_lib
    from rewl_simulator_gb300.mlp import MLP
    e16 = _exact(16)
    base = ws.Baseline(np.array(list(e16)) / 256.0, np.array(list(e16.values())) / 256.0)
    rows = []
    for L, nwin in ((8, 4), (8, 8), (16, 8), (16, 16)):
        with rg.Engine(_ising(rg, L, nwin, 1, 1.0, 1)) as eng:
            rows.append(_exact_rows(eng, _exact(L), L, base))
    X = np.concatenate([r[0] for r in rows])
    y = np.concatenate([r[1] for r in rows])
    mlp = MLP(hidden=256, layers=4, seed=7)
    mlp.set_data(X, y)
    losses = mlp.train(3000, batch=1024, lr=1e-3)
    assert np.isfinite(losses).all()

    exact = _exact(32)
    cap = 400
    with rg.Engine(_ising(rg, 32, 16, 2, 1.0, 11)) as plain:
        err_zero = _max_err(plain, exact)
        with rg.Engine(_ising(rg, 32, 16, 2, 1e-4, 11)) as warm:
            ws.warm_start(warm, mlp, 0, lnf0=1e-4, base=base)
            err_warm0 = _max_err(warm, exact)
            assert err_warm0 < 0.05 * err_zero, (err_warm0, err_zero)

            need, flips = None, 0
            for k in range(1, cap + 1):
                st = plain.run_cycles(1)
                if _max_err(plain, exact) <= err_warm0:
                    need, flips = k, st.attempted_flips
                    break
            # plain WL spends many check intervals (6.6 M flips each) to get where the network
            # starts: 124 on a GB300 with these seeds
            assert need is None or need >= 20, (need, err_warm0)

            errs = []

            def track(e, s):
                errs.append(_max_err(e, exact))
                return False

            # before any window could fall back to plain WL (which zeroes its ln g), the small
            # ln f keeps the network's estimate: the error stays near its value at injection
            stall = 80
            ws.run(warm, min(need or cap, stall - 1), stall_checks=stall, burn_in=8, on_cycle=track)
            assert max(errs) <= 2.0 * err_warm0 + 0.5, (err_warm0, errs[:5], max(errs))
            assert errs[-1] < err_warm0, (err_warm0, errs[-1])          # and improves on it (12.7 -> 6.1 on a GB300)
    mlp.close()
    print(f"\nwarm start L=32: max|dlng| {err_warm0:.3f} at injection (zero start {err_zero:.1f}); "
          f"plain WL needs {need} intervals ({flips} flips) to reach it; warm run after {len(errs)}: {errs[-1]:.3f}")


@pytest.mark.gpu
def test_gpu_warm_start_ashkin_teller(engine_lib):
    """The warm start on Ashkin-Teller (half spectrum, Baxter-field feature): five L=6 realisations
    (K=0.5, h ~ N(0, 0.5^2)) run plain WL in one engine; a network trained on four of them
    predicts the fifth, whose own plain-WL ln g judges it.  The prediction's shape error (ln g is
    defined up to a constant) must be a small fraction of the zero start's."""
    rg = engine_lib
    from rewl_simulator_gb300.mlp import MLP
    L, K, sh = 6, 0.5, 0.5
    N = L * L
    inss = [rg.Instance(model=rg.MODEL_ASHKIN_TELLER2D, L=L, K=K,
                        fields=np.round(np.random.default_rng(200 + k).normal(0.0, sh, N) * 2**20) / 2**20,
                        energy_min=-(2.0 + K) * 2 * N, energy_max=0.0, bin_width=0.25, num_windows=4,
                        replicas_per_window=2, window_overlap=0.75, seed=31 + k) for k in range(5)]
    batch = rg.Batch(instances=inss, sweeps_per_exchange=500, sweeps_per_check=2000, flatness_param=0.8,
                     lnf_initial=1.0, lnf_final=1e-5, mask_mode=rg.MASK_VISITED)
    with rg.Engine(batch) as eng:
        eng.simulate(max_cycles=600)
        rows = [ws.training_rows(eng, i, sigma_h=sh) for i in range(4)]
        E, lng = eng.global_logdos(4, half_spectrum=True)
        wins = [(lo, hi, ws.window_energies(eng, 4, w)) for w, (lo, hi, nb) in enumerate(eng.windows[4])]
    X = np.concatenate([r[0] for r in rows])
    y = np.concatenate([r[1] for r in rows])
    mlp = MLP(hidden=256, layers=4, seed=11)
    mlp.set_data(X, y)
    losses = mlp.train(3000, batch=1024, lr=1e-3)
    assert np.isfinite(losses).all()
    pred = {}
    for lo, hi, Ew in wins:
        for e, v in zip(Ew, ws.predict_lng(mlp, Ew, L, 1.0, K, sh, lo, hi)):
            pred.setdefault(round(float(e), 9), v)
    mlp.close()
    d = np.array([pred[round(float(e), 9)] for e in E]) - lng
    err_warm = float(np.max(np.abs(d - d.mean())))
    err_zero = float(np.max(np.abs(lng - lng.mean())))
    print(f"\nAshkin-Teller L=6 warm start: shape error {err_warm:.3f} nats against {err_zero:.2f} for the zero start "
          f"({len(E)} levels)")
    assert err_warm < 0.15 * err_zero, (err_warm, err_zero)


def test_baseline_interpolates_monotone_pieces_and_sorts():
    e = np.array([0.5, -1.0, 0.0, -2.0])
    s = np.array([0.6, 0.4, 0.69, 0.0])
    b = ws.Baseline(e, s)
    np.testing.assert_allclose(b(np.array([-2.0, -1.0, 0.0, 0.5])), [0.0, 0.4, 0.69, 0.6], atol=1e-12)
    x = np.linspace(-2.0, 0.0, 41)
    assert np.all(np.diff(b(x)) >= -1e-12)                 # monotone data stays monotone (no overshoot)


class RowsEngine(FakeEngine):
    """A converged fake: ln g(E) = 0.01 E^2 on Ising levels, every other bin masked out."""

    def global_logdos(self, i, half_spectrum=False):
        E = np.arange(-128.0, 132.0, 4.0)
        return E, 0.01 * E ** 2

    def window_mask(self, i, w):
        m = np.ones(self.windows[i][w][2], dtype=bool)
        m[1::2] = False
        return m


def test_training_rows_take_masked_levels_and_subtract_the_baseline():
    from rewl_simulator_gb300.mlp import features
    eng = RowsEngine(2, {})
    base = ws.Baseline(np.array([-2.0, 0.0, 2.0]), np.array([0.0, 0.1, 0.0]))
    X, y = ws.training_rows(eng, 0, base=base)
    n_expected = sum((nb + 1) // 2 for _, _, nb in eng.windows[0])
    assert X.shape == (n_expected, 7) and y.shape == (n_expected,)
    lo, hi, nb = eng.windows[0][0]
    E = lo + 4.0 * np.arange(0, nb, 2)
    np.testing.assert_allclose(X[:len(E)], features(E, 8, 1.0, 0.0, 0.0, lo, hi), rtol=1e-6)
    np.testing.assert_allclose(y[:len(E)], 0.01 * E ** 2 / 64 - base(E / 64), rtol=1e-5, atol=1e-6)
