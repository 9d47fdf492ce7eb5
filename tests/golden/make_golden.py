"""Generate the golden fixtures in tests/golden/ (run in a container that has the
reference sources; the fixtures are committed so the tests need no reference).

    REWL_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py            # everything
    REWL_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py replay     # one group

Groups
  replay   -- the reference's own REWL_Walker (oracle/build_ref.py harness):
              initial configuration after adjust_state_to_range, then K1 sweeps
              at ln f = 1, then reset_histogram (REDUCE_LOGDOS) and K2 sweeps at
              ln f = 1/2.  Records lattices, states, histograms, logDoS and
              per-bin observables (src/REWL/wang_landau.hpp:51-120,
              src/REWL/rewl_walker.hpp:79-158).
  replay_corr -- the same on a subset of the cases with the reference's
              CORRELATION_LENGTHS build (its CMake default): the observables carry
              G(q_min) columns (src/Hamiltonians/Correlations/fourier_correlator.hpp).
  glazier  -- glazier::construct_windows windows (src/REWL/glazier.hpp:305-351).
  rng      -- the first uniforms of random_number_generator<double>
              (src/util/random_number_generators.hpp:14-31) for a few seeds.
  normalize-- normalize_logDoS (src/util/array_shift.hpp:15-43).
  exact    -- exact 2D Ising ln g(E) (oracle/beale.py) for L = 4..64.
  thermo   -- the reference's Thermodynamics::calculate_thermodynamics
              (src/Thermodynamics/thermodynamics.hpp:158-297, oracle/ref_thermo.cpp)
              on the exact L = 16 Ising ln g with synthetic observables, and on a
              synthetic Ashkin-Teller-like spectrum with 12 moments, with and without
              the trapezoidal rule.
  cumulants-- the reference's susceptibility, Binder cumulants and correlation length
              (src/Thermodynamics/order_parameter_cumulants.hpp:17-59) on random averages.
  writers  -- the reference's three output writers (oracle/ref_writers.cpp) on
              the thermo_ising inputs: tests/golden/writers/*.txt.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import beale, build_ref, pyoracle  # noqa: E402

OUT = Path(__file__).resolve().parent

ISING_CASES = [
    # name, L, wmin, wmax, bw, seed, K1, K2
    ("ising_L4_full", 4, -32, 36, 4, 101, 300, 300),
    ("ising_L8_low", 8, -128, -20, 4, 12345, 100, 100),
    ("ising_L16_c1w1", 16, -368, 224, 4, 7, 60, 60),
    ("ising_L16_bw8", 16, -296, 200, 8, 5, 60, 60),
    ("ising_L32_c2w3", 32, -1404, -536, 4, 3, 20, 20),
]
AT_CASES = [
    # name, L, K, sigma_h, window lo (bins of 0.05 above E_allup), nbins, seed, K1, K2
    ("at_L4_rf", 4, 0.5, 0.5, 400, 900, 3, 40, 40),
    ("at_L8_rf", 8, 0.5, 0.5, 3000, 4000, 11, 25, 25),
    ("at_L6_clean_K025", 6, 0.25, 0.0, 1000, 2000, 2, 30, 30),
]


def quantised_fields(rng, n, sigma):
    return np.round(rng.normal(0.0, sigma, n) * 2.0**20) / 2.0**20


def _stage(ref, orc):
    c, g = ref.hist()
    return dict(dofs=ref.dofs().astype(np.int8), state=ref.state(), counts=c, logdos=g, obs=ref.obs(),
                draws=np.array(orc.draws(0), dtype=np.uint64))


def _replay_case(model, name, L, K, wmin, wmax, bw, nb, seed, k1, k2, fields=None, corr=False):
    if model == "ising":
        so = build_ref.build("ising", L, bw, corr=corr)
    else:
        so = build_ref.build("at", L, bw, K=K, fields=fields is not None, corr=corr)
    ref = pyoracle.RefWalker(so, wmin, wmax, bw, nb, seed)
    rng = np.random.default_rng(seed)
    if fields is not None:
        ref.import_disorder(fields)
    d0 = rng.choice([-1.0, 1.0], size=ref.ndof)
    ref.import_dofs(d0)
    ref.adjust()
    st0, dofs0 = ref.state().copy(), ref.dofs().copy()
    # the port follows along so that the number of uniforms consumed is known
    cfg = pyoracle.Config(model=pyoracle.MODEL_ISING if model == "ising" else pyoracle.MODEL_AT, L=L, K=K,
                          escale_bits=0 if model == "ising" else 20, nwin=1, R=1, emin=wmin, emax=wmax, bw=bw,
                          semantics=pyoracle.SEM_REFERENCE, observables=2 if corr else 1)
    orc = pyoracle.Oracle(cfg, fields=fields, init_dofs=dofs0)
    orc.set_dofs(0, dofs0, int(st0[4]) if model != "ising" else 0)
    orc.set_rng(0, seed, 1)
    ref.walk(k1)
    orc.run_sweeps(k1)
    s1 = _stage(ref, orc)
    ref.reset()
    ref.set_lnf(0.5)
    orc.reset(0, True)
    orc.set_lnf(0, 0.5)
    ref.walk(k2)
    orc.run_sweeps(k2)
    s2 = _stage(ref, orc)
    c2, g2, _ = orc.tables(0)
    assert np.array_equal(c2, s2["counts"]) and np.array_equal(g2, s2["logdos"]), name
    data = dict(model=np.array(0 if model == "ising" else 1), L=np.array(L), K=np.array(K), bw=np.array(bw),
                wmin=np.array(float(wmin)), wmax=np.array(float(wmax)), nbins=np.array(nb), seed=np.array(seed),
                sweeps1=np.array(k1), sweeps2=np.array(k2), lnf1=np.array(1.0), lnf2=np.array(0.5),
                fields=np.zeros(0) if fields is None else fields,
                init_dofs_raw=d0.astype(np.int8), dofs0=dofs0.astype(np.int8), state0=st0,
                adjust_draws=np.array(1))
    for k, v in s1.items():
        data[f"{k}1"] = v
    for k, v in s2.items():
        data[f"{k}2"] = v
    if corr:
        # the port's correlators follow the reference's summation order: equal bit for bit
        o2 = orc.obs(0)
        assert np.array_equal(o2, s2["obs"]), (name, np.abs(o2 - s2["obs"]).max())
    np.savez_compressed(OUT / (f"replay_corr_{name}.npz" if corr else f"replay_{name}.npz"), **data)
    print("wrote", name, "state", s2["state"], "draws", s1["draws"], s2["draws"])


def gen_replay(corr=False, only=None):
    for name, L, wmin, wmax, bw, seed, k1, k2 in ISING_CASES:
        if only and name not in only:
            continue
        nb = int(round((wmax - wmin) / bw))
        _replay_case("ising", name, L, 0.0, wmin, wmax, bw, nb, seed, k1, k2, corr=corr)
    for name, L, K, sig, wlo, nb, seed, k1, k2 in AT_CASES:
        if only and name not in only:
            continue
        N = L * L
        emin = -(2.0 + K) * 2 * N
        wmin, wmax = emin + wlo / 20.0, emin + (wlo + nb) / 20.0
        rng = np.random.default_rng(seed + 1000)
        fields = quantised_fields(rng, N, sig) if sig > 0 else None
        _replay_case("at", name, L, K, wmin, wmax, 0.05, nb, seed, k1, k2, fields=fields, corr=corr)


# the reference's CORRELATION_LENGTHS build (its CMake default): observables with G(q_min) columns
CORR_CASES = ("ising_L4_full", "ising_L8_low", "ising_L16_c1w1", "at_L4_rf", "at_L8_rf")


# long runs so that bins see several transforms (counts past 1000, 2000, ...)
CORR_LONG_ISING = [("ising_L4_long", 4, -32, 36, 4, 101, 2000, 2000)]
CORR_LONG_AT = [("at_L4_rf_long", 4, 0.5, 0.5, 400, 900, 5, 1500, 1500)]


def gen_replay_corr():
    gen_replay(corr=True, only=CORR_CASES)
    for name, L, wmin, wmax, bw, seed, k1, k2 in CORR_LONG_ISING:
        _replay_case("ising", name, L, 0.0, wmin, wmax, bw, int(round((wmax - wmin) / bw)), seed, k1, k2, corr=True)
    for name, L, K, sig, wlo, nb, seed, k1, k2 in CORR_LONG_AT:
        N = L * L
        emin = -(2.0 + K) * 2 * N
        wmin, wmax = emin + wlo / 20.0, emin + (wlo + nb) / 20.0
        fields = quantised_fields(np.random.default_rng(seed + 1000), N, sig)
        _replay_case("at", name, L, K, wmin, wmax, 0.05, nb, seed, k1, k2, fields=fields, corr=True)


def gen_glazier():
    so = build_ref.build("ising", 8, 4.0)
    ref = pyoracle.RefWalker(so, -128, -20, 4.0, 27, 1)
    cases = {
        "C1_L16": (-512.0, 516.0, 4.0, 4, 1, 0.75),
        "C2_L32": (-2048.0, 2052.0, 4.0, 16, 8, 0.75),
        "L64_64w": (-8192.0, 8196.0, 4.0, 64, 8, 0.75),
        "L24_16w": (-1152.0, 1156.0, 4.0, 16, 4, 0.75),
        "ref_default_L24_bw8": (-1152.0, 0.0, 8.0, 8, 1, 0.75),
        "at_L32_bw005": (-5120.0, 0.0, 0.05, 8, 4, 0.75),
    }
    out = {}
    for k, (a, b, bw, n, r, ov) in cases.items():
        mins, maxs, nb = ref.glazier(a, b, bw, n, r, ov)
        out[k] = dict(args=[a, b, bw, n, r, ov], mins=[float(x) for x in mins], maxs=[float(x) for x in maxs],
                      nbins=[int(x) for x in nb])
    (OUT / "glazier.json").write_text(json.dumps(out, indent=1))
    print("wrote glazier.json")


def gen_rng():
    so = build_ref.build("ising", 8, 4.0)
    ref = pyoracle.RefWalker(so, -128, -20, 4.0, 27, 1)
    import ctypes as C
    out = {}
    for seed in (1, 12345, 3141592653):
        u = np.zeros(64)
        ref.lib.ref_uniforms(seed, 64, u.ctypes.data_as(C.c_void_p))
        out[str(seed)] = [float(x).hex() for x in u]
    (OUT / "ref_uniforms.json").write_text(json.dumps(out, indent=1))
    print("wrote ref_uniforms.json")


def gen_fields():
    """The reference's random-field generator (Disorder::generate_random_field) from fixed seeds."""
    so = build_ref.build("ising", 8, 4.0)
    ref = pyoracle.RefWalker(so, -128, -20, 4.0, 27, 1)
    import ctypes as C
    cases = []
    for seed, strength, kind, n in ((1, 0.5, 1, 50), (2024, 1.25, 1, 50), (3141592653, 0.25, 0, 50), (7, 2.0, 0, 50)):
        h = np.zeros(n)
        ref.lib.ref_random_fields(seed, strength, kind, n, h.ctypes.data_as(C.c_void_p))
        cases.append(dict(seed=seed, strength=strength, distribution=kind, fields=[float(x).hex() for x in h]))
    (OUT / "random_fields.json").write_text(json.dumps(cases, indent=1))
    print("wrote random_fields.json")


def gen_concatenate():
    """The reference's concatenate_tables (multiple overlap) + normalize_logDoS on window tables cut
    from exact ln g with per-window offsets and noise (Ising), and from a smooth synthetic ln g on a
    0.05 grid (half spectrum, Ashkin-Teller-like)."""
    so = build_ref.build("ising", 8, 4.0)
    ref = pyoracle.RefWalker(so, -128, -20, 4.0, 27, 1)
    import ctypes as C
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rng = np.random.default_rng(11)
    cases = {}

    def cut(E, g, bounds, noise):
        wins = []
        for a, b in bounds:
            gw = g[a:b] - g[a] + rng.uniform(-3, 3) + rng.normal(0, noise, b - a)
            wins.append((E[a:b].astype(float), gw))
        return wins

    z16 = np.load(OUT / "exact_ising_L16.npz")
    z8 = np.load(OUT / "exact_ising_L8.npz")
    e = np.round(np.arange(-30.0, 0.0001, 0.05), 2)
    s_at = 20.0 * np.sqrt(np.clip((e + 30.0) / 30.0, 0, 1)) + 0.02 * np.sin(e)
    specs = [("ising_L16_3win", z16["E"], z16["lng"], [(0, 80), (50, 160), (130, len(z16["E"]))], 0.05, 2.0, 256, 1.0),
             ("ising_L16_4win_clean", z16["E"], z16["lng"], [(0, 70), (40, 130), (100, 200), (170, len(z16["E"]))], 0.0,
              2.0, 256, 1.0),
             ("ising_L8_2win_noisy", z8["E"], z8["lng"], [(0, 40), (25, len(z8["E"]))], 0.3, 2.0, 64, 1.0),
             ("at_half_3win", e, s_at, [(0, 270), (195, 480), (405, len(e))], 0.02, 4.0, 36, 0.0)]
    K = 3                                              # two observables and a count column
    for name, E, g, bounds, noise, spp, N, emax in specs:
        wins = cut(E, g, bounds, noise)
        sizes = np.array([len(w[0]) for w in wins], dtype=np.uint64)
        Ef = np.concatenate([w[0] for w in wins])
        Gf = np.concatenate([w[1] for w in wins])
        Of = np.column_stack([rng.uniform(0, 1, len(Ef)), rng.normal(0, 1, len(Ef)),
                              rng.integers(1, 1000, len(Ef)).astype(float)]).ravel()
        cap = C.c_size_t(len(Ef))
        oe, og, oo = np.zeros(len(Ef)), np.zeros(len(Ef)), np.zeros(len(Ef) * K)
        ref.lib.ref_concatenate(len(wins), p(sizes), p(Ef), p(Gf), K, p(Of), spp, N, emax, p(oe), p(og), p(oo),
                                C.byref(cap))
        n = cap.value
        for key, val in (("meta", np.array([spp, N, float(emax == 0.0), K])), ("sizes", sizes.astype(np.int64)),
                         ("energies", Ef), ("logdos", Gf), ("obs", Of), ("out_energies", oe[:n]),
                         ("out_logdos", og[:n]), ("out_obs", oo[:n * K])):
            cases[f"{name}.{key}"] = val
    np.savez_compressed(OUT / "concatenate.npz", **cases)
    print("wrote concatenate.npz")


def gen_normalize():
    so = build_ref.build("ising", 8, 4.0)
    ref = pyoracle.RefWalker(so, -128, -20, 4.0, 27, 1)
    import ctypes as C
    rng = np.random.default_rng(4)
    cases = {}
    for name, n, spp, N, emax in (("half", 60, 2.0, 64, 0.0), ("full", 61, 2.0, 64, 128.0), ("at", 300, 4.0, 36, 0.0)):
        x = np.cumsum(rng.normal(0.3, 0.2, n))
        y = x.copy()
        ref.lib.ref_normalize_logdos(spp, N, emax, n, y.ctypes.data_as(C.c_void_p))
        cases[name] = dict(states_per_site=spp, N=N, energy_max=emax, inp=[v.hex() for v in x], out=[v.hex() for v in y])
    (OUT / "normalize.json").write_text(json.dumps(cases, indent=1))
    print("wrote normalize.json")


def gen_exact():
    for L in (4, 6, 8, 16, 24, 32, 64):
        E, lng = beale.exact_lng(L)
        extra = {}
        if L <= 8:
            g = beale.exact_dos(L)
            extra["g_decimal"] = np.array([str(v) for v in g])
        np.savez_compressed(OUT / f"exact_ising_L{L}.npz", E=E, lng=lng, **extra)
        print("wrote exact L", L)


def _thermo_inputs(at: bool):
    if not at:
        z = np.load(OUT / "exact_ising_L16.npz")
        ok = np.isfinite(z["lng"])
        E, lng, N = z["E"][ok].astype(np.float64), z["lng"][ok], 256
        m = np.sqrt(np.clip(1.0 - (E / E[-1]) ** 2, 0.0, None)) * (E < 0) + 0.05
        obs = np.stack([m, m * m + 0.01, (m * m + 0.01) ** 2 + 0.001, 1000.0 + (np.arange(E.size) % 7) * 13.0], axis=1)
        return E, lng, obs, N, 3
    N = 64
    E = np.arange(-320.0, 0.0, 0.5)                      # AT L = 8, K = 0.5 range, bins of 0.5
    x = E / E[0]
    lng = 2 * N * np.log(2.0) * (1.0 - x ** 2) + np.log(4.0) * x ** 8
    cols = []
    for k in range(12):
        cols.append(0.1 + 0.8 * x ** (1 + k % 3) * (1.0 + 0.01 * k))
    obs = np.stack(cols + [500.0 + (np.arange(E.size) % 5) * 11.0], axis=1)
    return E, lng, obs, N, 12


def gen_thermo():
    import ctypes as C
    for trap in (True, False):
        lib = C.CDLL(str(build_ref.build_thermo(trapezoid=trap, force=True)))
        lib.ref_thermo.restype = C.c_int
        lib.ref_thermo.argtypes = [C.c_int, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_double,
                                   C.c_double, C.c_size_t, C.c_void_p, C.c_void_p]
        for at in (False, True):
            E, lng, obs, N, cc = _thermo_inputs(at)
            obs = np.ascontiguousarray(obs)
            Tmin, Tmax, nT = 0.01, 50.01, 2000
            out = np.zeros((nT, 5 + obs.shape[1]))
            T = np.zeros(nT)
            p = lambda a: a.ctypes.data_as(C.c_void_p)
            lib.ref_thermo(int(at), E.size, p(E), p(lng), p(obs), N, Tmin, Tmax, nT, p(out), p(T))
            name = f"thermo_{'at' if at else 'ising'}{'' if trap else '_plain'}.npz"
            np.savez_compressed(OUT / name, E=E, lng=lng, obs=obs, N=N, counts_col=cc, Tmin=Tmin, Tmax=Tmax, nT=nT,
                                trapezoid=int(trap), model=int(at), temperatures=T, out=out)
            print("wrote", name)


WRITER_HEADER = "# Model: 2D Ising, L = 16\n# REWL: 4 windows, 75 % overlap\n"
WRITER_NAMES = "Magnetization\nMagnetization2\nMagnetization4\nCounts per Bin"
THERMAL_NAMES = "Free Energy\nEnergy\nEnergy2\nEntropy\nSpecific Heat\n" + WRITER_NAMES


def gen_writers():
    import ctypes as C
    lib = C.CDLL(str(build_ref.build_writers(force=True)))
    lib.ref_write.argtypes = [C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t, C.c_size_t,
                              C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    z = np.load(OUT / "thermo_ising.npz")
    d = OUT / "writers"
    d.mkdir(exist_ok=True)
    p = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.c_void_p)
    E, lng, obs, out, T = z["E"], z["lng"], np.ascontiguousarray(z["obs"]), np.ascontiguousarray(z["out"]), z["temperatures"]
    nl = np.ascontiguousarray(out[:, 5:7])
    args = [(0, WRITER_NAMES, E.size, obs.shape[1], 256.0, E, lng, obs),
            (1, THERMAL_NAMES, T.size, out.shape[1], 1.0, T, None, out),
            (2, "Susceptibility\nBinder Cumulant", T.size, 2, 1.0, T, None, nl)]
    keep = []
    for kind, names, rows, cols, N, a, b, v in args:
        arrs = [np.ascontiguousarray(a, dtype=np.float64), None if b is None else np.ascontiguousarray(b, dtype=np.float64),
                np.ascontiguousarray(v, dtype=np.float64)]
        keep.append(arrs)
        lib.ref_write(kind, str(d).encode(), b"golden", WRITER_HEADER.encode(), names.encode(), rows, cols, N,
                      arrs[0].ctypes.data_as(C.c_void_p), None if arrs[1] is None else arrs[1].ctypes.data_as(C.c_void_p),
                      arrs[2].ctypes.data_as(C.c_void_p))
    print("wrote", sorted(x.name for x in d.iterdir()))


def gen_cumulants():
    """The reference's order_parameter_cumulants.hpp on random thermal averages (including a
    vanishing G, where the correlation length is DBL_MAX / L, and G above <m^2>)."""
    import ctypes as C
    lib = C.CDLL(str(build_ref.build_thermo(True, force=True)))
    rng = np.random.default_rng(77)
    n, N = 64, 256
    m = rng.uniform(0.05, 0.95, n)
    m2 = m * m + rng.uniform(0.0, 0.05, n)
    m4 = m2 * m2 + rng.uniform(0.0, 0.05, n)
    G = m2 * rng.uniform(0.01, 0.9, n)
    G[0], G[1] = 0.0, 1.5 * m2[1]
    T = rng.uniform(0.1, 10.0, n)
    out = np.zeros((n, 4))
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
    lib.ref_cumulants(C.c_size_t(n), p(m), p(m2), p(m4), p(G), p(T), C.c_size_t(N), p(out))
    np.savez_compressed(OUT / "cumulants.npz", m=m, m2=m2, m4=m4, G=G, T=T, N=N, out=out)
    print("wrote cumulants", out[:2])


if __name__ == "__main__":
    groups = sys.argv[1:] or ["replay", "replay_corr", "glazier", "rng", "fields", "concatenate", "normalize", "exact",
                              "thermo", "cumulants", "writers"]
    for g in groups:
        globals()[f"gen_{g}"]()
