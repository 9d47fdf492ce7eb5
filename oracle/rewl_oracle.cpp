// TEST INFRASTRUCTURE ONLY -- the CPU oracle.  Never linked into the product;
// used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py.
//
// A plain C++ restatement of the reference's REWL hot path, written for this
// project (no reference code is compiled in).  Each piece cites the reference
// function it restates:
//
//   Ising2d::local_field/local_energy/change_state/set_state/recalculate_state
//       src/Hamiltonians/Ising2d/ising2d_hamiltonian.hpp:162-231
//   Ising2d::update_observables, Ising2d_Obs::update_observable_average
//       src/Hamiltonians/Ising2d/ising2d_hamiltonian.hpp:234-256, ising2d_observables.hpp:134-145
//   Ashkin_Teller2d::local_energy/recalculate_state/change_state/set_state/update_observables
//       src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_hamiltonian.hpp:169-318
//   neighbour order (x,y-1),(x-1,y),(x+1,y),(x,y+1), site = y*L + x
//       src/Hamiltonians/Address_Books/Square_Periodic_Lattices/square_2d_grid_helpers.hpp:14,37-63
//   Wang_Landau::wang_landau_update / wang_landau_sweep
//       src/REWL/wang_landau.hpp:51-120
//   rewl_histograms reset (REDUCE_LOGDOS) and count_flatness
//       src/REWL/rewl_histograms.hpp:83-95,115-152
//   REWL_Walker::adjust_state_to_range / update_histograms
//       src/REWL/rewl_walker.hpp:79-115,209-214
//   glazier::construct_windows (EQUAL_WINDOWS)
//       src/REWL/glazier.hpp:70-115
//   REWL_simulation::replica_exchange_update / average_and_redistribute_window /
//   check_if_window_is_flat / simulate (ln f schedule, termination)
//       src/Simulation/rewl_simulation.hpp:228-346,361-454,458-470,473-691
// (Window concatenation and normalize_logDoS are not restated here: the tests compare the
// product's versions with the reference's own, run by oracle/ref_harness.cpp.)
//
// Two semantics are implemented:
//   * REFERENCE: each walker owns std::mt19937_64(seed) with
//     uniform_real_distribution<double>(0,1) (src/util/random_number_generators.hpp:14-31);
//     a uniform is drawn only when the trial energy is in range and the float
//     entropy change is positive; acceptance is u < exp(-dg) in double; logDoS in
//     plain FP64.  This reproduces the reference walker bit for bit and is the
//     timed CPU baseline.
//   * ENGINE: the semantics of the CUDA engine: one Philox4x32-10 draw per attempt
//     (Salmon et al., SC'11), acceptance dg < -ln(u) with a deterministic float
//     log, logDoS held on a 2^-36 grid (averaged values are rounded back onto it),
//     exact integer energies and bins, Philox pairing for the exchange.  The GPU
//     engine must agree with this bit for bit.
//
// Energies: Ising uses integer energies; Ashkin-Teller energies are multiples of
// 2^-20 (Baxter fields are quantised to that grid by the caller) so every double
// sum below is exact.

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

namespace orc {

// ----------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Multipliers and Weyl key increments from that paper.
// ----------------------------------------------------------------------------
struct U4 { uint32_t v[4]; };

static inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r)
    {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.v[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.v[2];
        U4 n;
        n.v[0] = (uint32_t)(p1 >> 32) ^ c.v[1] ^ k0;
        n.v[1] = (uint32_t)p1;
        n.v[2] = (uint32_t)(p0 >> 32) ^ c.v[3] ^ k1;
        n.v[3] = (uint32_t)p0;
        c = n;
    }
    return c;
}

// Counter streams (third counter word) of the engine semantics.
enum : uint32_t { STREAM_WL = 0x574C0001u, STREAM_EXCH = 0x45580002u, STREAM_INIT = 0x494E0003u, STREAM_ADJ = 0x41440004u };

// An instance's Philox key comes from its seed through the SplitMix64 finaliser
// (Steele, Lea, Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014), so
// that seeds differing only in low bits do not give walkers the same (seed ^ walker) key.
static inline uint64_t instance_key(uint64_t seed)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint32_t key0(uint64_t seed, uint32_t uid) { return (uint32_t)seed ^ uid; }
static inline uint32_t key1(uint64_t seed) { return (uint32_t)(seed >> 32); }

static inline uint32_t philox_word(uint64_t seed, uint32_t uid, uint64_t ctr, uint32_t stream, uint32_t w3 = 0)
{
    U4 c = {{(uint32_t)(ctr >> 2), (uint32_t)(ctr >> 34), stream, w3}};
    U4 r = philox4x32_10(c, key0(seed, uid), key1(seed));
    return r.v[ctr & 3];
}

// ----------------------------------------------------------------------------
// Deterministic -ln(u) for u = (2*(x>>1)+1) * 2^-32, float arithmetic only with
// every rounding explicit (compiled with -ffp-contract=off).  For u > 1/sqrt(2)
// the exact 1 - u is used; otherwise u = m 2^-k with m in [sqrt(1/2), sqrt(2)].
// ln from the atanh series ln((1+s)/(1-s)) = 2 (s + s^3/3 + ... + s^9/9).
// ----------------------------------------------------------------------------
static inline float neglog_u32(uint32_t x)
{
    const uint32_t v = x | 1u;
    float s;
    int k = 0;
    if (v > 0xB504F333u)
    {   // u > 1/sqrt(2): 1 - u = (2^32 - v) 2^-32 is exact; -ln u = 2 atanh(d / (2 - d))
        const float d = (float)(0u - v) * 2.3283064365386963e-10f;
        s = d / (2.0f - d);
    }
    else
    {
        const int e = 31 - __builtin_clz(v);           // v in [2^e, 2^(e+1))
        float m = (float)v;                            // round to nearest
        uint32_t sb = (uint32_t)(127 - e) << 23;       // 2^-e
        float scale; std::memcpy(&scale, &sb, 4);
        m = m * scale;                                 // exact, m in [1,2]
        k = 32 - e;                                    // -ln u = k ln2 - ln m
        if (m > 1.41421354f) { m = m * 0.5f; k -= 1; }
        s = (1.0f - m) / (m + 1.0f);                   // -ln m = 2 atanh((1-m)/(1+m))
    }
    const float s2 = s * s;
    float p = ::fmaf(s2, 0.111111112f, 0.142857149f);
    p = ::fmaf(p, s2, 0.200000003f);
    p = ::fmaf(p, s2, 0.333333343f);
    p = ::fmaf(p, s2, 1.0f);
    const float q = (2.0f * s) * p;
    return ::fmaf((float)k, 0.693147182f, q);
}

// Smallest integer d (>= 1) with fl32(d * 2^-36) >= thr, for thr > 0.  Then
// "float(dg) < thr" is exactly "d < T" for dg = d * 2^-36.
static inline int64_t accept_threshold(float thr)
{
    uint32_t b; std::memcpy(&b, &thr, 4);
    const int be = (int)((b >> 23) & 0xFF);
    const int64_t m = (int64_t)((b & 0x7FFFFFu) | 0x800000u);
    const int e = be - 150;                            // thr = m * 2^e
    int64_t A; int s; bool inclusive;
    if (m == 0x800000) { A = 4 * m - 1; s = e - 2; inclusive = true; }
    else { A = 2 * m - 1; s = e - 1; inclusive = (m & 1) == 0; }
    const int sh = s + 36;
    if (sh >= 0) { const int64_t D = A << sh; return inclusive ? D : D + 1; }
    return (A >> (-sh)) + 1;
}

static constexpr int QBITS = 36;
static constexpr double QSCALE = 68719476736.0;        // 2^36

// ----------------------------------------------------------------------------
// Lattice helpers: neighbour order (x,y-1),(x-1,y),(x+1,y),(x,y+1).
// ----------------------------------------------------------------------------
static inline void neighbours(size_t site, size_t L, size_t nb[4])
{
    const size_t x = site % L, y = site / L;
    nb[0] = (y == 0 ? L - 1 : y - 1) * L + x;
    nb[1] = y * L + (x == 0 ? L - 1 : x - 1);
    nb[2] = y * L + (x == L - 1 ? 0 : x + 1);
    nb[3] = (y == L - 1 ? 0 : y + 1) * L + x;
}

// ----------------------------------------------------------------------------
// Models (double spins and energies, as in the reference).
// ----------------------------------------------------------------------------
enum { MODEL_ISING = 0, MODEL_AT = 1 };

// Transform_Kernel (src/Hamiltonians/Correlations/fourier_correlator.hpp:14-42):
// cos and sin of q_min * x, q_min = 2 pi / L, for x = 0 .. L-1.
struct QTable
{
    std::vector<double> re, im;
    void build(size_t L)
    {
        const double qmin = 2. * std::acos(-1.) / static_cast<double>(L);
        re.resize(L); im.resize(L);
        for (size_t i = 0; i != L; ++i) { re[i] = std::cos(qmin * static_cast<double>(i)); im[i] = std::sin(qmin * static_cast<double>(i)); }
    }
};

// Fourier_Correlator::compute_correlator (fourier_correlator.hpp:65-118) in the
// reference's summation order: f(row, col) = field[(row L + col) nt + t1], times
// field[... + t2] when mixed.  The x part transforms the row sums against the row
// index, the y part every site against its column index; the result is half the
// sum of the two squared magnitudes.
static double fourier_correlator(const QTable& q, size_t L, const double* field, size_t t1, size_t t2, size_t nt, bool mixed)
{
    double rx = 0., ix = 0., ry = 0., iy = 0.;
    for (size_t row = 0; row != L; ++row)
    {
        double rowsum = 0.;
        for (size_t col = 0; col != L; ++col)
        {
            double v = field[(row * L + col) * nt + t1];
            v *= (!mixed) + mixed * field[(row * L + col) * nt + t2];
            rowsum += v;
            ry += v * q.re[col];
            iy += v * q.im[col];
        }
        rx += rowsum * q.re[row];
        ix += rowsum * q.im[row];
    }
    rx = rx * rx + ix * ix;
    ry = ry * ry + iy * iy;
    return 0.5 * (rx + ry);
}

struct IsingState { double energy = 0, magnetization = 0, dof = 0; };

struct Ising
{
    static constexpr int num_obs = 4;                  // |m|, m^2, m^4, counts
    static constexpr int num_obs_corr = 5;             // |m|, m^2, m^4, G(q_min), counts
    static int corr_col(int k) { return k; }
    size_t L = 0, N = 0; double J = 1.0;
    std::vector<double> spin, field;                   // field empty => h = 0
    IsingState st;
    int which = 0;                                     // unused (single flavour)

    size_t num_dof() const { return N; }
    double local_field(size_t i) const
    {
        double f = field.empty() ? 0.0 : field[i];
        size_t nb[4]; neighbours(i, L, nb);
        for (int k = 0; k < 4; ++k) f += J * spin[nb[k]];
        return f;
    }
    double local_energy(size_t i, double s) const { return -1. * s * local_field(i); }
    void recalculate()
    {
        double e = 0., m = 0.;
        for (size_t i = 0; i != N; ++i)
        {
            m += spin[i];
            const double h = field.empty() ? 0.0 : field[i];
            e += -0.5 * h * spin[i] + 0.5 * local_energy(i, spin[i]);
        }
        st.energy = e; st.magnetization = m;
    }
    void change_state(size_t i, IsingState& t) const
    {
        t.dof = -spin[i];
        t.magnetization = st.magnetization + t.dof - spin[i];
        t.energy = st.energy + local_energy(i, t.dof) - local_energy(i, spin[i]);
    }
    void set_state(size_t i, const IsingState& t) { st.energy = t.energy; st.magnetization = t.magnetization; spin[i] = t.dof; }
    void switch_flavor() {}
    template <class F> void observables(F&& upd) const
    {
        const double m = (1.0 / (double)N) * std::fabs(st.magnetization);
        upd(0, m); upd(1, m * m); upd(2, m * m * m * m);
    }
    // Ising2d::update_observables, CORRELATION_LENGTHS (ising2d_hamiltonian.hpp:246-252)
    template <class F> void correlators(const QTable& q, F&& upd) const
    {
        const double dn = 1.0 / (double)N;
        upd(3, dn * dn * fourier_correlator(q, L, spin.data(), 0, 0, 1, false));
    }
};

struct ATState { int which = 0; double energy = 0, sm = 0, tm = 0, bax = 0; double dof[2] = {1., 1.}; };

struct AshkinTeller
{
    static constexpr int num_obs = 13;                 // 12 moments + counts
    static constexpr int num_obs_corr = 17;            // 4 x (3 moments, G(q_min)) + counts
    static int corr_col(int k) { return k + k / 3; }
    size_t L = 0, N = 0; double J = 1.0, K = 0.5;
    std::vector<double> spin;                          // interleaved [sigma, tau] per site
    std::vector<double> field;                         // Baxter field per site (may be empty)
    ATState st;

    size_t num_dof() const { return 2 * N; }
    double local_energy(size_t i, const double* s) const
    {
        double en = 0.;
        const double si = s[0], ti = s[1];
        if (!field.empty()) en += field[i] * (si * ti);
        size_t nb[4]; neighbours(i, L, nb);
        for (int k = 0; k < 4; ++k)
        {
            const double sn = spin[2 * nb[k]], tn = spin[2 * nb[k] + 1];
            en += J * si * sn;
            en += J * ti * tn;
            en += K * si * ti * sn * tn;
        }
        return -en;
    }
    void recalculate()
    {
        double e = 0., sm = 0., tm = 0., bx = 0.;
        for (size_t i = 0; i != N; ++i)
        {
            sm += spin[2 * i]; tm += spin[2 * i + 1]; bx += spin[2 * i] * spin[2 * i + 1];
            if (!field.empty()) e += -0.5 * field[i] * spin[2 * i] * spin[2 * i + 1];
            e += 0.5 * local_energy(i, &spin[2 * i]);
        }
        st.energy = e; st.sm = sm; st.tm = tm; st.bax = bx;
    }
    void change_state(size_t i, ATState& t)
    {
        const double s0 = spin[2 * i], t0 = spin[2 * i + 1];
        t.dof[0] = s0; t.dof[1] = t0;
        t.dof[0] += -2. * t.dof[0] * (st.which == 0);
        t.dof[1] += -2. * t.dof[1] * (st.which == 1);
        t.which = (st.which == 0) ? 1 : 0;
        t.sm = st.sm + t.dof[0] - s0;
        t.tm = st.tm + t.dof[1] - t0;
        t.bax = st.bax + (t.dof[0] * t.dof[1]) - (s0 * t0);
        t.energy = st.energy + local_energy(i, t.dof) - local_energy(i, &spin[2 * i]);
        if (i == N - 1) st.which = t.which;            // flavour toggles at the last site
    }
    void set_state(size_t i, const ATState& t)
    {
        st.energy = t.energy; st.sm = t.sm; st.tm = t.tm; st.bax = t.bax;
        spin[2 * i] = t.dof[0]; spin[2 * i + 1] = t.dof[1];
    }
    void switch_flavor() { st.which = st.which == 0 ? 1 : 0; }
    template <class F> void observables(F&& upd) const
    {
        const double dn = 1.0 / (double)N;
        const double s = dn * std::fabs(st.sm), t = dn * std::fabs(st.tm), b = dn * std::fabs(st.bax);
        const double p2 = s * s + t * t;
        upd(0, s); upd(1, s * s); upd(2, s * s * s * s);
        upd(3, t); upd(4, t * t); upd(5, t * t * t * t);
        upd(6, std::sqrt(p2)); upd(7, p2); upd(8, p2 * p2);
        upd(9, b); upd(10, b * b); upd(11, b * b * b * b);
    }
    // Ashkin_Teller2d::update_observables, CORRELATION_LENGTHS (ashkin_teller2d_hamiltonian.hpp:295-315):
    // the tau correlator is computed from sigma as in the reference (:298-299), phi's is their sum,
    // the Baxter one from sigma * tau.
    template <class F> void correlators(const QTable& q, F&& upd) const
    {
        const double dn = 1.0 / (double)N;
        const double gs = dn * dn * fourier_correlator(q, L, spin.data(), 0, 1, 2, false);
        const double gt = dn * dn * fourier_correlator(q, L, spin.data(), 0, 1, 2, false);
        const double gb = dn * dn * fourier_correlator(q, L, spin.data(), 0, 1, 2, true);
        upd(3, gs); upd(7, gt); upd(11, gs + gt); upd(15, gb);
    }
};

// ----------------------------------------------------------------------------
// Configuration shared by both semantics (mirrors rewl_batch_desc's fields).
// ----------------------------------------------------------------------------
enum { SEM_REFERENCE = 0, SEM_ENGINE = 1 };
enum { FLAT_MIN_OVER_MEAN = 0, FLAT_MAX_MIN_RATIO = 1, FLAT_ALL_VISITED = 2 };
enum { MASK_STATIC = 0, MASK_VISITED = 1 };

struct Config
{
    int model = MODEL_ISING;
    int L = 4;
    double J = 1.0, K = 0.5;
    int escale_bits = 0;            // energies are multiples of 2^-escale_bits
    double emin = 0, emax = 0;      // global energy range [emin, emax)
    double bw = 4.0;                // bin width (1/bw an integer or bw an integer)
    int nwin = 1, R = 1;
    double overlap = 0.75;
    int sweeps_per_exchange = 1000, sweeps_per_check = 1000;
    double lnf0 = 1.0, lnf_final = 1e-6;
    int flat_mode = FLAT_MIN_OVER_MEAN; double flat_param = 0.8;
    int mask_mode = MASK_STATIC;
    int one_over_t = 0, reduce_logdos = 1, observables = 0;
    uint64_t seed = 1;
    int semantics = SEM_ENGINE;
    int init_mode = 0;              // 0: spins uniform from seed, 1: all +1
    int nthreads = 1;
};

// Global bin of an energy, exact for the energies of both models: integer
// widths divide integer energy offsets; fractional widths 1/n multiply dyadic
// offsets by the integer n (no rounding).  Same cost as the reference's one
// division per lookup (src/REWL/histogram_index.hpp:18).
struct Binning
{
    double emin = 0, bw = 1, inv = 1; bool int_width = true;
    int64_t gbin(double e) const
    {
        return int_width ? (int64_t)std::floor((e - emin) / bw) : (int64_t)std::floor((e - emin) * inv);
    }
};

static Binning make_binning(const Config& c)
{
    Binning b;
    b.emin = c.emin; b.bw = c.bw;
    b.int_width = c.bw >= 1.0;
    b.inv = b.int_width ? 1.0 : (double)std::llround(1.0 / c.bw);
    return b;
}

// glazier::construct_windows with EQUAL_WINDOWS (src/REWL/glazier.hpp:305-351),
// in units of bins: each window starts on the global bin grid at the previous
// start plus the whole bins to its nominal start and covers its nominal width
// in whole bins, clipped to the global range.  Identical to the reference for
// integer widths; exact for fractional ones.
struct WinDef { double min, max; size_t nbins; int64_t gb_lo; };

static std::vector<WinDef> make_windows(const Config& c, const Binning& bn)
{
    std::vector<WinDef> w(c.nwin);
    const int64_t G = (int64_t)std::llround((c.emax - c.emin) / c.bw);
    const double denom = 1 + (c.nwin - 1) * (1 - c.overlap);
    const double size = (c.emax - c.emin) / denom;
    const double eps = 1e-9;
    for (int k = 0; k < c.nwin; ++k)
    {
        const double raw_min = c.emin + (double)k * (1 - c.overlap) * size;
        const double raw_max = raw_min + size;
        int64_t lo = 0;
        if (k != 0) lo = w[k - 1].gb_lo + (int64_t)std::floor((raw_min - w[k - 1].min) / c.bw + eps);
        const double wmin = c.emin + c.bw * (double)lo;
        int64_t hi = lo + (int64_t)std::ceil((raw_max - wmin) / c.bw - eps);
        if (hi > G) hi = G;
        w[k].gb_lo = lo;
        w[k].nbins = (size_t)(hi - lo);
        w[k].min = wmin;
        w[k].max = c.emin + c.bw * (double)hi;
    }
    (void)bn;
    return w;
}

// ----------------------------------------------------------------------------
// One walker slot (window w, replica r).
// ----------------------------------------------------------------------------
template <class M> struct alignas(128) Walker
{
    M sys;
    int win = 0, rep = 0; uint32_t uid = 0;
    int64_t gb_lo = 0; size_t nb = 0;
    std::vector<uint64_t> count;       // per-stage histogram
    std::vector<uint64_t> visits;      // cumulative visits (counts_per_bin)
    std::vector<double> logdos;
    std::vector<double> obs;           // AoS running averages [bin][num_obs] (reference layout)
    double lnf = 1.0;
    int64_t lnf_u = 0;                 // engine semantics: ln f in 2^-36 units
    uint64_t sweeps_done = 0;          // engine semantics: attempt counter base
    std::mt19937_64 gen;               // reference semantics
    std::uniform_real_distribution<double> U{0., 1.};
    uint64_t draws = 0;
};

template <class M> struct Sim
{
    Config c;
    uint64_t key = 0;                   // Philox key of the engine semantics: instance_key(c.seed)
    Binning bn;
    std::vector<WinDef> wins;
    std::vector<Walker<M>> wk;          // slot = w*R + r
    std::vector<uint8_t> static_mask;   // per window-local bin, concatenated by window
    std::vector<size_t> mask_off;
    std::vector<int> done;              // per window
    std::vector<int> oot;               // per window (1/t engaged)
    std::vector<uint64_t> iteration, sweep_counter;   // per window (1/t bookkeeping)
    int direction = 0;                  // 0: even pairs (0-1, 2-3, ...), 1: odd pairs
    uint64_t exch_round = 0;
    uint64_t total_sweeps = 0;
    uint64_t exch_accepted = 0, exch_attempted = 0;
    int nobs = M::num_obs;              // observable columns per bin (with correlators: M::num_obs_corr)
    QTable q;                           // correlator kernel (observables == 2)

    int64_t gbin(double e) const { return bn.gbin(e); }
    bool in_range(const Walker<M>& w, double e) const
    {
        const int64_t g = gbin(e);
        return g >= w.gb_lo && g < w.gb_lo + (int64_t)w.nb;
    }
    size_t lbin(const Walker<M>& w, double e) const { return (size_t)(gbin(e) - w.gb_lo); }
};

// ---------------------------- setup ---------------------------------------------
template <class M> static void init_model(Sim<M>& S, M& m, const double* fields);

template <> void init_model<Ising>(Sim<Ising>& S, Ising& m, const double* fields)
{
    m.L = S.c.L; m.N = (size_t)S.c.L * S.c.L; m.J = S.c.J;
    m.spin.assign(m.N, 1.0);
    if (fields) m.field.assign(fields, fields + m.N);
}
template <> void init_model<AshkinTeller>(Sim<AshkinTeller>& S, AshkinTeller& m, const double* fields)
{
    m.L = S.c.L; m.N = (size_t)S.c.L * S.c.L; m.J = S.c.J; m.K = S.c.K;
    m.spin.assign(2 * m.N, 1.0);
    if (fields) m.field.assign(fields, fields + m.N);
}

static inline void set_flavour(Ising&, int) {}
static inline void set_flavour(AshkinTeller& m, int f) { m.st.which = f; }

// adjust_state_to_range (src/REWL/rewl_walker.hpp:79-115); returns false when
// the deterministic walk did not reach the window within max_steps.  Without a
// flip the walk's next decisions depend only on (site, flavour), which repeat
// within 2N steps, so 2N steps without a flip mean it can never move again: it
// stops there with the same outcome it would reach at max_steps.
template <class M> static bool adjust(Sim<M>& S, Walker<M>& w, size_t start_site, size_t max_steps)
{
    const size_t N = w.sys.N;
    size_t site = start_site;
    bool in = S.in_range(w, w.sys.st.energy);
    size_t steps = 0, idle = 0;
    while (!in)
    {
        if (++steps > max_steps || ++idle > 2 * N) return false;
        ++site;
        if (site == N) { site = 0; w.sys.switch_flavor(); }
        typename std::conditional<std::is_same<M, Ising>::value, IsingState, ATState>::type t;
        w.sys.change_state(site, t);
        const double e = w.sys.st.energy;
        const int64_t g = S.gbin(e);
        const bool too_low = g < w.gb_lo, too_high = g >= w.gb_lo + (int64_t)w.nb;
        if ((too_low && t.energy > e) || (too_high && t.energy <= e)) { w.sys.set_state(site, t); idle = 0; }
        in = S.in_range(w, w.sys.st.energy);
    }
    return true;
}

static void static_mask_for(const Config& c, const WinDef& w, std::vector<uint8_t>& m)
{
    m.assign(w.nbins, 1);
    if (c.model != MODEL_ISING) return;
    // Ising on an L x L torus: E = -2N + 4 and E = 2N - 4 cannot occur.
    const double N = (double)c.L * c.L;
    for (size_t b = 0; b < w.nbins; ++b)
    {
        const double lo = w.min + c.bw * (double)b, hi = lo + c.bw;
        bool any = false;
        for (double e = std::ceil((lo + 2 * N) / 4.0) * 4.0 - 2 * N; e < hi; e += 4.0)
        {
            if (e < -2 * N || e > 2 * N) continue;
            if (e == -2 * N + 4 || e == 2 * N - 4) continue;
            any = true;
        }
        m[b] = any ? 1 : 0;
    }
}

template <class M> static Sim<M>* create(const Config& c, const double* fields, const double* init_dofs)
{
    auto* S = new Sim<M>();
    S->c = c;
    S->key = instance_key(c.seed);
    S->bn = make_binning(c);
    S->nobs = c.observables == 2 ? M::num_obs_corr : M::num_obs;
    if (c.observables == 2) S->q.build((size_t)c.L);
    S->wins = make_windows(c, S->bn);
    const int W = c.nwin, R = c.R;
    S->wk.resize((size_t)W * R);
    S->done.assign(W, 0); S->oot.assign(W, 0);
    S->iteration.assign(W, 1); S->sweep_counter.assign(W, 0);
    S->mask_off.resize(W + 1, 0);
    for (int w = 0; w < W; ++w)
    {
        std::vector<uint8_t> m; static_mask_for(c, S->wins[w], m);
        S->mask_off[w + 1] = S->mask_off[w] + m.size();
        S->static_mask.insert(S->static_mask.end(), m.begin(), m.end());
    }
    for (int w = 0; w < W; ++w)
        for (int r = 0; r < R; ++r)
        {
            Walker<M>& k = S->wk[(size_t)w * R + r];
            k.win = w; k.rep = r; k.uid = (uint32_t)(w * R + r);
            k.gb_lo = S->wins[w].gb_lo; k.nb = S->wins[w].nbins;
            // spare capacity keeps neighbouring walkers' hot entries on separate cache lines
            k.count.reserve(k.nb + 32); k.visits.reserve(k.nb + 32); k.logdos.reserve(k.nb + 32);
            k.count.assign(k.nb, 0); k.visits.assign(k.nb, 0); k.logdos.assign(k.nb, 0.0);
            k.obs.assign(k.nb * S->nobs, 0.0);
            k.lnf = c.lnf0;
            k.lnf_u = std::max<int64_t>(1, (int64_t)std::llround(c.lnf0 * QSCALE));
            init_model<M>(*S, k.sys, fields);
            const size_t nd = k.sys.num_dof();
            if (init_dofs) { for (size_t i = 0; i < nd; ++i) k.sys.spin[i] = init_dofs[i]; }
            else if (c.init_mode == 0)
            {
                if (c.semantics == SEM_ENGINE)
                    for (size_t i = 0; i < nd; ++i)
                    {   // engine layout: sigma plane then tau plane; ours is interleaved
                        const size_t e_idx = (M::num_obs == 13) ? ((i & 1) ? (i >> 1) + k.sys.N : (i >> 1)) : i;
                        k.sys.spin[i] = (philox_word(S->key, k.uid, e_idx, STREAM_INIT) >> 31) ? -1.0 : 1.0;
                    }
                else
                {
                    std::mt19937_64 g(c.seed * 1000003ULL + k.uid);
                    for (size_t i = 0; i < nd; ++i) k.sys.spin[i] = (g() >> 63) ? -1.0 : 1.0;
                }
            }
            k.sys.recalculate();
            if (c.semantics == SEM_REFERENCE) k.gen.seed((uint32_t)(c.seed + k.uid));
            size_t start;
            if (c.semantics == SEM_ENGINE)
                start = (size_t)(((uint64_t)philox_word(S->key, k.uid, 0, STREAM_ADJ) * k.sys.N) >> 32);
            else { start = (size_t)(k.U(k.gen) * (double)k.sys.N); ++k.draws; }
            const size_t cap = 4000 * nd;
            bool ok = adjust(*S, k, start, cap);
            // stuck in a local extremum: restart from all +1 (walk up), then from
            // the checkerboard (walk down)
            for (int attempt = 1; attempt <= 2 && !ok; ++attempt)
            {
                const size_t N = k.sys.N, L = (size_t)c.L;
                for (size_t i = 0; i < nd; ++i)
                {
                    const size_t site = (M::num_obs == 13) ? i / 2 : i;   // AT layout is interleaved
                    const size_t x = site % L, y = site / L;
                    k.sys.spin[i] = (attempt == 1 || ((x + y) & 1) == 0) ? 1.0 : -1.0;
                }
                (void)N;
                k.sys.recalculate();
                set_flavour(k.sys, 0);
                ok = adjust(*S, k, start, cap);
            }
            if (!ok) { delete S; return nullptr; }
        }
    return S;
}

// ---------------------------- the Wang-Landau update -------------------------
// update_observables at bin b: the running means (v + c avg) / (c + 1) of the model's
// moments over the bin's count c (ising2d_observables.hpp:134-145); with correlators
// (observables == 2, the reference's default CORRELATION_LENGTHS build) the G(q_min)
// columns are updated by update_qmin_correlator (ising2d_observables.hpp:148-159) with
// the number of earlier transforms whenever c is a multiple of counts_per_transform
// = 1000 (fourier_correlator.hpp:11; ising2d_hamiltonian.hpp:246-252); then c += 1.
template <class M> static void observe(const Sim<M>& S, Walker<M>& w, size_t b)
{
    const int n = S.nobs;
    const bool corr = S.c.observables == 2;
    double* o = &w.obs[b * n];
    const double c = o[n - 1];
    w.sys.observables([&](int k, double v) { double& x = o[corr ? M::corr_col(k) : k]; x = (v + c * x) / (c + 1); });
    if (corr && static_cast<size_t>(c) % 1000 == 0)
    {
        const size_t t = static_cast<size_t>(c / static_cast<double>(1000));
        w.sys.correlators(S.q, [&](int col, double v) { o[col] = (v + t * o[col]) / (t + 1); });
    }
    o[n - 1] += 1;
}

template <class M, int SEM> static inline void wl_update(Sim<M>& S, Walker<M>& w, size_t idx, uint64_t attempt)
{
    typename std::conditional<std::is_same<M, Ising>::value, IsingState, ATState>::type t;
    w.sys.change_state(idx, t);
    size_t cur = S.lbin(w, w.sys.st.energy);
    if (S.in_range(w, t.energy))
    {
        const size_t nb = S.lbin(w, t.energy);
        const float dg = (float)(w.logdos[nb] - w.logdos[cur]);
        bool acc;
        if (SEM == SEM_REFERENCE)
        {
            if (dg <= 0.) acc = true;
            else { ++w.draws; acc = w.U(w.gen) < static_cast<double>(std::exp(-(double)dg)); }
        }
        else
        {
            const float thr = neglog_u32(philox_word(S.key, w.uid, attempt, STREAM_WL));
            acc = (dg <= 0.f) || (dg < thr);
        }
        if (acc) { w.sys.set_state(idx, t); cur = nb; }
    }
    w.count[cur] += 1;
    w.visits[cur] += 1;
    w.logdos[cur] += (SEM == SEM_REFERENCE) ? w.lnf : (double)w.lnf_u / QSCALE;
    if (S.c.observables) observe(S, w, cur);
}

template <class M> static void walk(Sim<M>& S, Walker<M>& w, uint64_t nsweeps)
{
    const size_t N = w.sys.N;
    const size_t flavours = w.sys.num_dof() / N;
    for (uint64_t s = 0; s < nsweeps; ++s)
    {
        const uint64_t base = (w.sweeps_done + s) * (uint64_t)(flavours * N);
        for (size_t f = 0; f < flavours; ++f)
            for (size_t i = 0; i < N; ++i)
            {
                if (S.c.semantics == SEM_REFERENCE) wl_update<M, SEM_REFERENCE>(S, w, i, 0);
                else wl_update<M, SEM_ENGINE>(S, w, i, base + f * N + i);
            }
    }
    w.sweeps_done += nsweeps;
}

// update_histograms + update_observables after an exchange attempt (rewl_simulation.hpp:333-338)
template <class M> static void touch(Sim<M>& S, Walker<M>& w)
{
    const size_t b = S.lbin(w, w.sys.st.energy);
    w.count[b] += 1; w.visits[b] += 1;
    w.logdos[b] += (S.c.semantics == SEM_REFERENCE) ? w.lnf : (double)w.lnf_u / QSCALE;
    if (S.c.observables) observe(S, w, b);
}

template <class M> static void swap_configs(Walker<M>& a, Walker<M>& b);

template <> void swap_configs<Ising>(Walker<Ising>& a, Walker<Ising>& b)
{
    std::swap(a.sys.spin, b.sys.spin);
    std::swap(a.sys.st, b.sys.st);
}
template <> void swap_configs<AshkinTeller>(Walker<AshkinTeller>& a, Walker<AshkinTeller>& b)
{
    std::swap(a.sys.spin, b.sys.spin);
    // the whole State travels except which_to_update, which stays with the walker
    // (mpi_exchange_state sends energy, magnetisations, baxter and DoF only,
    //  src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_hamiltonian.hpp:354-365)
    const int wa = a.sys.st.which, wb = b.sys.st.which;
    std::swap(a.sys.st, b.sys.st);
    a.sys.st.which = wa; b.sys.st.which = wb;
}

// replica_exchange_update (src/Simulation/rewl_simulation.hpp:228-346)
template <class M> static void exchange(Sim<M>& S)
{
    const int W = S.c.nwin, R = S.c.R;
    const int first = S.direction == 0 ? 0 : 1;
    for (int lw = first; lw + 1 < W; lw += 2)
    {
        std::vector<int> perm(R);
        for (int r = 0; r < R; ++r) perm[r] = r;
        if (S.c.semantics == SEM_REFERENCE)
        {
            std::vector<int> sp(R);
            for (int r = 0; r < R; ++r) sp[r] = R + r;
            std::shuffle(sp.begin(), sp.end(), S.wk[(size_t)lw * R].gen);
            for (int r = 0; r < R; ++r) perm[r] = sp[r] - R;
        }
        else
        {
            for (int i = R - 1; i >= 1; --i)
            {
                const uint32_t word = philox_word(S.key, 0x80000000u, ((uint64_t)(R - 1 - i)),
                                                  STREAM_EXCH, (uint32_t)((S.exch_round << 8) ^ (uint64_t)lw));
                const int j = (int)(((uint64_t)word * (uint64_t)(i + 1)) >> 32);
                std::swap(perm[i], perm[j]);
            }
        }
        for (int r = 0; r < R; ++r)
        {
            Walker<M>& lo = S.wk[(size_t)lw * R + r];
            Walker<M>& hi = S.wk[(size_t)(lw + 1) * R + perm[r]];
            const double El = lo.sys.st.energy, Eh = hi.sys.st.energy;
            bool accept = false;
            S.exch_attempted++;
            if (S.c.semantics == SEM_REFERENCE)
            {
                double p_lo = 0., p_hi = 0.;
                if (S.in_range(lo, Eh)) p_lo = std::exp(std::min(0., lo.logdos[S.lbin(lo, El)] - lo.logdos[S.lbin(lo, Eh)]));
                if (S.in_range(hi, El)) p_hi = std::exp(std::min(0., hi.logdos[S.lbin(hi, Eh)] - hi.logdos[S.lbin(hi, El)]));
                const double p = p_lo * p_hi;
                if (p != 0.) { ++lo.draws; accept = lo.U(lo.gen) < p; }
            }
            else if (S.in_range(lo, Eh) && S.in_range(hi, El))
            {
                const double a = lo.logdos[S.lbin(lo, Eh)] - lo.logdos[S.lbin(lo, El)];
                const double b = hi.logdos[S.lbin(hi, El)] - hi.logdos[S.lbin(hi, Eh)];
                const double delta = std::max(0., a) + std::max(0., b);
                // after the R - 1 pairing words: counter 32 + r while R <= 32, 64 + r above
                const uint32_t word = philox_word(S.key, 0x80000000u, (uint64_t)((R <= 32 ? 32 : 64) + r),
                                                  STREAM_EXCH, (uint32_t)((S.exch_round << 8) ^ (uint64_t)lw));
                const float thr = neglog_u32(word);
                const int64_t d = (int64_t)std::llround(delta * QSCALE);
                accept = d < accept_threshold(thr);
            }
            if (accept) { swap_configs(lo, hi); S.exch_accepted++; }
            touch(S, lo); touch(S, hi);
        }
    }
    S.direction ^= 1;
    S.exch_round++;
}

template <class M> static bool window_mask(const Sim<M>& S, int w, size_t b)
{
    if (!S.static_mask[S.mask_off[w] + b]) return false;
    if (S.c.mask_mode == MASK_VISITED)
    {
        for (int r = 0; r < S.c.R; ++r) if (S.wk[(size_t)w * S.c.R + r].visits[b]) return true;
        return false;
    }
    return true;
}

template <class M> static bool replica_flat(const Sim<M>& S, const Walker<M>& k, int w)
{
    if (S.c.flat_mode == FLAT_ALL_VISITED)
    {
        if (S.oot[w]) return true;
        for (size_t b = 0; b < k.nb; ++b) if (window_mask(S, w, b) && k.count[b] == 0) return false;
        return true;
    }
    uint64_t mn = UINT64_MAX, mx = 0, sum = 0, n = 0;
    for (size_t b = 0; b < k.nb; ++b)
    {
        if (!window_mask(S, w, b)) continue;
        mn = std::min(mn, k.count[b]); mx = std::max(mx, k.count[b]); sum += k.count[b]; ++n;
    }
    if (n == 0 || mn == 0) return false;
    if (S.c.flat_mode == FLAT_MAX_MIN_RATIO)
        return ((float)(mx - mn) / (float)mn) <= (float)S.c.flat_param;
    // min >= p * mean with p = num/den exactly: min * n * den >= p_num * sum
    const double p = S.c.flat_param;
    const uint64_t den = 1000000; const uint64_t num = (uint64_t)std::llround(p * (double)den);
    return (unsigned __int128)mn * n * den >= (unsigned __int128)num * sum;
}

// check_if_window_is_flat + average_and_redistribute_window + reset + ln f
// (src/Simulation/rewl_simulation.hpp:361-470,515-600)
template <class M> static int flat_step(Sim<M>& S)
{
    const int W = S.c.nwin, R = S.c.R;
    int flat_events = 0;
    for (int w = 0; w < W; ++w)
    {
        bool flat = true;
        for (int r = 0; r < R && flat; ++r) flat = replica_flat(S, S.wk[(size_t)w * R + r], w);
        if (!flat) continue;
        ++flat_events;
        const size_t nb = S.wins[w].nbins;
        if (R > 1)
        {
            std::vector<double> avg(nb, 0.0);
            for (size_t b = 0; b < nb; ++b)
            {
                uint64_t tot = 0;
                for (int r = 0; r < R; ++r) tot += S.wk[(size_t)w * R + r].count[b];
                double acc = 0.0;
                if (tot == 0) acc = S.wk[(size_t)w * R].logdos[b];
                else
                    for (int r = 0; r < R; ++r)
                    {
                        const Walker<M>& k = S.wk[(size_t)w * R + r];
                        const double wt = (double)k.count[b] / (double)tot;
                        const double term = wt * k.logdos[b];
                        acc = acc + term;
                    }
                if (S.c.semantics == SEM_ENGINE) acc = std::nearbyint(acc * QSCALE) / QSCALE;
                avg[b] = acc;
            }
            for (int r = 0; r < R; ++r) S.wk[(size_t)w * R + r].logdos = avg;
        }
        for (int r = 0; r < R; ++r)
        {
            Walker<M>& k = S.wk[(size_t)w * R + r];
            const double red = S.c.reduce_logdos ? -k.logdos[0] : 0.0;
            for (size_t b = 0; b < nb; ++b) { k.count[b] = 0; k.logdos[b] += red; }
        }
        // ln f schedule
        const uint64_t t = S.sweep_counter[w] * S.iteration[w];
        for (int r = 0; r < R; ++r)
        {
            Walker<M>& k = S.wk[(size_t)w * R + r];
            if (S.c.semantics == SEM_REFERENCE)
            {
                if (S.c.one_over_t && !S.oot[w] && k.lnf <= 1. / (double)t) S.oot[w] = 1;
                k.lnf = (0.5 * k.lnf) * (!S.oot[w]) + (1. / (double)t) * S.oot[w];
            }
            else
            {
                if (S.c.one_over_t && !S.oot[w] && (double)k.lnf_u <= QSCALE / (double)t) S.oot[w] = 1;
                k.lnf_u = S.oot[w] ? (int64_t)(((uint64_t)1 << QBITS) + t / 2) / (int64_t)t : (k.lnf_u >> 1);
                if (k.lnf_u < 1) k.lnf_u = 1;           // smallest increment of the 2^-36 grid
                k.lnf = (double)k.lnf_u / QSCALE;
            }
        }
        const double lnf = S.wk[(size_t)w * R].lnf;
        S.done[w] = lnf < S.c.lnf_final ? 1 : 0;
        S.iteration[w] += 1; S.sweep_counter[w] = 0;
    }
    return flat_events;
}

// ---------------------------- thread pool -------------------------------------
struct Pool
{
    std::vector<std::thread> th;
    std::mutex mu; std::condition_variable cv, cv_done;
    std::function<void(size_t)> job; size_t njobs = 0; std::atomic<size_t> next{0};
    size_t active = 0; uint64_t gen = 0; bool stop = false;
    explicit Pool(int n)
    {
        for (int i = 0; i < n; ++i)
            th.emplace_back([this] {
                uint64_t seen = 0;
                for (;;)
                {
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv.wait(lk, [&] { return stop || gen != seen; });
                        if (stop) return;
                        seen = gen;
                    }
                    for (size_t j; (j = next.fetch_add(1)) < njobs;) job(j);
                    std::lock_guard<std::mutex> lk(mu);
                    if (--active == 0) cv_done.notify_all();
                }
            });
    }
    void run(size_t n, std::function<void(size_t)> f)
    {
        if (th.empty()) { for (size_t j = 0; j < n; ++j) f(j); return; }
        std::unique_lock<std::mutex> lk(mu);
        job = std::move(f); njobs = n; next = 0; active = th.size(); ++gen;
        cv.notify_all();
        cv_done.wait(lk, [&] { return active == 0; });
    }
    ~Pool() { { std::lock_guard<std::mutex> lk(mu); stop = true; } cv.notify_all(); for (auto& t : th) t.join(); }
};

// ---------------------------- driver ------------------------------------------
template <class M> static void run_sweeps(Sim<M>& S, Pool* pool, uint64_t n)
{
    auto body = [&](size_t j) { walk(S, S.wk[j], n); };
    if (pool) pool->run(S.wk.size(), body); else for (size_t j = 0; j < S.wk.size(); ++j) body(j);
    for (int w = 0; w < S.c.nwin; ++w) S.sweep_counter[w] += n;
    S.total_sweeps += n;
}

// One check interval: (walk se sweeps, exchange) x (sc/se), then the flat step.
template <class M> static int cycle(Sim<M>& S, Pool* pool)
{
    const int se = S.c.sweeps_per_exchange, sc = S.c.sweeps_per_check;
    const int rounds = std::max(1, sc / se);
    for (int i = 0; i < rounds; ++i)
    {
        run_sweeps(S, pool, (uint64_t)se);
        if (S.c.nwin > 1) exchange(S);
    }
    return flat_step(S);
}

} // namespace orc

// ============================================================================
// C API (ctypes)
// ============================================================================
using namespace orc;

struct OrcHandle
{
    int model;
    void* sim;
    Pool* pool = nullptr;
    ~OrcHandle()
    {
        delete pool;
        if (model == MODEL_ISING) delete static_cast<Sim<Ising>*>(sim);
        else delete static_cast<Sim<AshkinTeller>*>(sim);
    }
};

#define DISPATCH(h, expr)                                                      \
    do {                                                                       \
        if ((h)->model == MODEL_ISING) { auto& S = *static_cast<Sim<Ising>*>((h)->sim); expr; } \
        else { auto& S = *static_cast<Sim<AshkinTeller>*>((h)->sim); expr; }   \
    } while (0)

extern "C" {

uint32_t orc_philox_word(uint64_t seed, uint32_t uid, uint64_t ctr, uint32_t stream, uint32_t w3)
{
    return philox_word(seed, uid, ctr, stream, w3);
}
void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out)
{
    U4 c = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
    U4 r = philox4x32_10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}
float orc_neglog_u32(uint32_t x) { return neglog_u32(x); }
int64_t orc_accept_threshold(float thr) { return accept_threshold(thr); }

// Fill `out` with the reference's uniform stream for `seed`.
void orc_mt64_uniforms(uint64_t seed, size_t n, double* out)
{
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> U(0., 1.);
    for (size_t i = 0; i < n; ++i) out[i] = U(g);
}

struct orc_config
{
    int32_t model, L;
    double J, K;
    int32_t escale_bits, nwin, R, sweeps_per_exchange, sweeps_per_check;
    double emin, emax, bw, overlap, lnf0, lnf_final, flat_param;
    int32_t flat_mode, mask_mode, one_over_t, reduce_logdos, observables, semantics, init_mode, nthreads;
    uint64_t seed;
};

void* orc_create(const orc_config* cc, const double* fields, const double* init_dofs)
{
    Config c;
    c.model = cc->model; c.L = cc->L; c.J = cc->J; c.K = cc->K; c.escale_bits = cc->escale_bits;
    c.nwin = cc->nwin; c.R = cc->R; c.sweeps_per_exchange = cc->sweeps_per_exchange;
    c.sweeps_per_check = cc->sweeps_per_check; c.emin = cc->emin; c.emax = cc->emax; c.bw = cc->bw;
    c.overlap = cc->overlap; c.lnf0 = cc->lnf0; c.lnf_final = cc->lnf_final; c.flat_param = cc->flat_param;
    c.flat_mode = cc->flat_mode; c.mask_mode = cc->mask_mode; c.one_over_t = cc->one_over_t;
    c.reduce_logdos = cc->reduce_logdos; c.observables = cc->observables; c.semantics = cc->semantics;
    c.init_mode = cc->init_mode; c.nthreads = cc->nthreads; c.seed = cc->seed;
    auto* h = new OrcHandle();
    h->model = c.model;
    if (c.model == MODEL_ISING) h->sim = create<Ising>(c, fields, init_dofs);
    else h->sim = create<AshkinTeller>(c, fields, init_dofs);
    if (!h->sim) { delete h; return nullptr; }
    if (c.nthreads > 1) h->pool = new Pool(c.nthreads);
    return h;
}

void orc_destroy(void* p) { delete static_cast<OrcHandle*>(p); }

size_t orc_num_walkers(void* p) { size_t n = 0; DISPATCH(static_cast<OrcHandle*>(p), n = S.wk.size()); return n; }

void orc_window(void* p, int w, double* minmax, int64_t* gb_lo, uint64_t* nbins)
{
    DISPATCH(static_cast<OrcHandle*>(p), { minmax[0] = S.wins[w].min; minmax[1] = S.wins[w].max; *gb_lo = S.wins[w].gb_lo; *nbins = S.wins[w].nbins; });
}

void orc_run_sweeps(void* p, uint64_t n)
{
    auto* h = static_cast<OrcHandle*>(p);
    DISPATCH(h, run_sweeps(S, h->pool, n));
}
void orc_exchange(void* p) { DISPATCH(static_cast<OrcHandle*>(p), exchange(S)); }
int orc_flat_step(void* p) { int n = 0; DISPATCH(static_cast<OrcHandle*>(p), n = flat_step(S)); return n; }
int orc_cycle(void* p) { auto* h = static_cast<OrcHandle*>(p); int n = 0; DISPATCH(h, n = cycle(S, h->pool)); return n; }

int orc_all_done(void* p)
{
    int all = 1; DISPATCH(static_cast<OrcHandle*>(p), for (int d : S.done) all &= d);
    return all;
}
void orc_done_flags(void* p, int32_t* out) { DISPATCH(static_cast<OrcHandle*>(p), for (size_t i = 0; i < S.done.size(); ++i) out[i] = S.done[i]); }

uint64_t orc_total_sweeps(void* p) { uint64_t n = 0; DISPATCH(static_cast<OrcHandle*>(p), n = S.total_sweeps); return n; }
void orc_exchange_stats(void* p, uint64_t* out) { DISPATCH(static_cast<OrcHandle*>(p), { out[0] = S.exch_attempted; out[1] = S.exch_accepted; }); }

// Walker export: state [E, M] (Ising) or [E, sm, tm, bax, which] (AT); dofs as
// +-1 in the model's layout (Ising: N; AT: sigma plane then tau plane).
void orc_walker_state(void* p, size_t slot, double* st)
{
    auto* h = static_cast<OrcHandle*>(p);
    if (h->model == MODEL_ISING)
    {
        auto& k = static_cast<Sim<Ising>*>(h->sim)->wk[slot];
        st[0] = k.sys.st.energy; st[1] = k.sys.st.magnetization;
    }
    else
    {
        auto& k = static_cast<Sim<AshkinTeller>*>(h->sim)->wk[slot];
        st[0] = k.sys.st.energy; st[1] = k.sys.st.sm; st[2] = k.sys.st.tm; st[3] = k.sys.st.bax; st[4] = k.sys.st.which;
    }
}
void orc_walker_dofs(void* p, size_t slot, int8_t* out)
{
    auto* h = static_cast<OrcHandle*>(p);
    if (h->model == MODEL_ISING)
    {
        auto& k = static_cast<Sim<Ising>*>(h->sim)->wk[slot];
        for (size_t i = 0; i < k.sys.N; ++i) out[i] = (int8_t)k.sys.spin[i];
    }
    else
    {
        auto& k = static_cast<Sim<AshkinTeller>*>(h->sim)->wk[slot];
        for (size_t i = 0; i < k.sys.N; ++i) { out[i] = (int8_t)k.sys.spin[2 * i]; out[k.sys.N + i] = (int8_t)k.sys.spin[2 * i + 1]; }
    }
}
void orc_walker_tables(void* p, size_t slot, uint64_t* counts, double* logdos, uint64_t* visits)
{
    DISPATCH(static_cast<OrcHandle*>(p), {
        auto& k = S.wk[slot];
        for (size_t b = 0; b < k.nb; ++b) { if (counts) counts[b] = k.count[b]; if (logdos) logdos[b] = k.logdos[b]; if (visits) visits[b] = k.visits[b]; }
    });
}
void orc_walker_obs(void* p, size_t slot, double* out)
{
    auto* h = static_cast<OrcHandle*>(p);
    if (h->model == MODEL_ISING) { auto& k = static_cast<Sim<Ising>*>(h->sim)->wk[slot]; std::memcpy(out, k.obs.data(), k.obs.size() * 8); }
    else { auto& k = static_cast<Sim<AshkinTeller>*>(h->sim)->wk[slot]; std::memcpy(out, k.obs.data(), k.obs.size() * 8); }
}
double orc_walker_lnf(void* p, size_t slot) { double v = 0; DISPATCH(static_cast<OrcHandle*>(p), v = S.wk[slot].lnf); return v; }
uint64_t orc_walker_draws(void* p, size_t slot) { uint64_t v = 0; DISPATCH(static_cast<OrcHandle*>(p), v = S.wk[slot].draws); return v; }

// Replace a walker's configuration (reference layout for AT: interleaved) and
// recompute its state; used to start from a configuration exported elsewhere.
void orc_walker_set_dofs(void* p, size_t slot, const double* dofs, int which)
{
    DISPATCH(static_cast<OrcHandle*>(p), {
        auto& k = S.wk[slot];
        for (size_t i = 0; i < k.sys.spin.size(); ++i) k.sys.spin[i] = dofs[i];
        k.sys.recalculate();
        (void)which;
    });
    auto* h = static_cast<OrcHandle*>(p);
    if (h->model == MODEL_AT) static_cast<Sim<AshkinTeller>*>(h->sim)->wk[slot].sys.st.which = which;
}
void orc_walker_set_lnf(void* p, size_t slot, double lnf)
{
    DISPATCH(static_cast<OrcHandle*>(p), { S.wk[slot].lnf = lnf; S.wk[slot].lnf_u = std::max<int64_t>(1, (int64_t)std::llround(lnf * QSCALE)); });
}
void orc_walker_set_logdos(void* p, size_t slot, const double* g)
{
    DISPATCH(static_cast<OrcHandle*>(p), { auto& k = S.wk[slot]; for (size_t b = 0; b < k.nb; ++b) k.logdos[b] = g[b]; });
}
void orc_walker_reset(void* p, size_t slot, int reduce)
{
    DISPATCH(static_cast<OrcHandle*>(p), {
        auto& k = S.wk[slot];
        const double red = reduce ? -k.logdos[0] : 0.0;
        for (size_t b = 0; b < k.nb; ++b) { k.count[b] = 0; k.logdos[b] += red; }
    });
}
// Set the reference-semantics generator (seed, already-consumed draws).
void orc_walker_set_rng(void* p, size_t slot, uint64_t seed, uint64_t skip)
{
    DISPATCH(static_cast<OrcHandle*>(p), {
        auto& k = S.wk[slot];
        k.gen.seed(seed); k.U.reset();
        for (uint64_t i = 0; i < skip; ++i) (void)k.U(k.gen);
        k.draws = skip;
    });
}

// Final in-window averaging with cumulative visit weights
// (average_and_redistribute_window with simulation_incomplete == false).
void orc_window_logdos(void* p, int w, double* out)
{
    DISPATCH(static_cast<OrcHandle*>(p), {
        const int R = S.c.R; const size_t nb = S.wins[w].nbins;
        for (size_t b = 0; b < nb; ++b)
        {
            double tot = 0; for (int r = 0; r < R; ++r) tot += (double)S.wk[(size_t)w * R + r].visits[b];
            double acc = 0;
            if (tot == 0 || R == 1) acc = S.wk[(size_t)w * R].logdos[b];
            else for (int r = 0; r < R; ++r) { const auto& k = S.wk[(size_t)w * R + r]; acc = acc + ((double)k.visits[b] / tot) * k.logdos[b]; }
            out[b] = acc;
        }
    });
}

int orc_window_mask(void* p, int w, uint8_t* out)
{
    int n = 0;
    DISPATCH(static_cast<OrcHandle*>(p), { for (size_t b = 0; b < S.wins[w].nbins; ++b) { out[b] = window_mask(S, w, b) ? 1 : 0; n += out[b]; } });
    return n;
}

} // extern "C"
