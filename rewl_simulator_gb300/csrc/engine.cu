// GB300 replica-exchange Wang-Landau engine: host driver, device kernels and
// the C ABI declared in include/rewl.h.
//
// Device layout (HBM), structure of arrays:
//   walker slots  s = first_slot(instance) + window * R + replica
//       slot_cfg[s]      configuration currently held by the slot (an exchange
//                        swaps two entries instead of moving lattices)
//       slot_tab[s]      offset of the slot's tables: g (int64, 2^-36 units),
//                        H (uint32 per-stage counts), visits (uint64 cumulative)
//       slot_sweeps[s]   sweeps done (Philox attempt counter base)
//       slot_flavour[s]  Ashkin-Teller which_to_update
//   configurations c: spins (int8; Ising N, Ashkin-Teller sigma plane then tau
//       plane), energy (int64 units of 2^-escale), magnetisations (int32 x3)
//   windows: ln f (int64 2^-36 units), done / 1/t flags, counters, valid-bin mask
//
// Kernels
//   k_init          one thread per walker: initial spins from Philox, then the
//                   deterministic walk into the window (rewl_walker.hpp:79-115)
//   k_sweep_ising   one warp per walker; lattice, g and H staged in shared
//                   memory; lanes precompute a row-aligned chunk of <= 32 sites
//                   (energy change with and without the left neighbour flipped,
//                   integer acceptance threshold), lane 0 resolves the serial
//                   Wang-Landau chain in integer arithmetic only
//   k_sweep_tables  the same for any model type of models.cuh with the tables in
//                   global memory (Ashkin-Teller: one plane per pass; Ising windows
//                   too large for shared memory)
//   k_exchange      one thread per window pair (rewl_simulation.hpp:228-346)
//   k_flat          one block per window: flatness vote, FP64 count-weighted
//                   averaging, histogram reset, REDUCE_LOGDOS, ln f schedule
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cfloat>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <limits>
#include <new>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/rewl.h"
#include "rng.cuh"
#include "models.cuh"

using namespace rewl;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                 \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess)                                                         \
            return fail(REWL_EDEVICE, "%s: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                        __FILE__, __LINE__);                                           \
    } while (0)

constexpr int kMaxReplicas = 64;
constexpr uint32_t kFull = 0xFFFFFFFFu;

enum : int { ERR_BOUNDS = 1, ERR_ADJUST = 2, ERR_REPLAY_EXHAUSTED = 4, ERR_RANGE = 8, ERR_COUNT = 16 };
// |logDoS| at which a window is reported (REWL_ESTATE) instead of risking int64 overflow: 2^62
// units (6.7e7 nats).  Every kernel that adds to g checks the values it wrote against it, and
// every kernel returns without work once the error word is set, so at most one launch's growth
// lies beyond the limit.  The host splits sweep launches so that one launch adds at most
// kLaunchGrowth to any bin (ln f bound x sweeps x degrees of freedom, plus one exchange visit):
// 2^62 + 2^62 - 2^58 stays below 2^63 with room for the acceptance thresholds (< 2^45).
constexpr long long kLogdosLimit = 1LL << 62;
constexpr double kSetLogdosMax = 16777216.0;                // 2^60 units: the largest |g| rewl_set_logdos takes
constexpr long long kLaunchGrowth = (1LL << 62) - (1LL << 58);

// Any device error stops further work: a kernel that finds the error word set returns at once.
// Another block may set the word while this one reads it, so a warp acts on lane 0's reading
// (all 32 lanes must be active) and a block on thread 0's.
__device__ __forceinline__ bool engine_failed(const int32_t* counters)
{
    return *reinterpret_cast<const volatile int32_t*>(counters) != 0;
}
__device__ __forceinline__ bool engine_failed_warp(const int32_t* counters)
{
    return __shfl_sync(0xFFFFFFFFu, (int)engine_failed(counters), 0) != 0;
}

// A launch's derived visits to bin k (its logDoS change over ln f) into the per-stage count
// (uint32, the reference keeps uint64: a count that would pass 2^32 - 1 saturates and is
// reported) and the cumulative visits; also checks the new logDoS against the range limit.
__device__ __forceinline__ int commit_visits(uint32_t* gH, uint64_t* gv, int k, long long dv, long long gnew)
{
    int err = 0;
    const unsigned long long h = (unsigned long long)gH[k] + (unsigned long long)dv;
    if (h > 0xFFFFFFFFull) { err |= ERR_COUNT; gH[k] = 0xFFFFFFFFu; }
    else gH[k] = (uint32_t)h;
    gv[k] += (uint64_t)dv;
    if (gnew >= kLogdosLimit) err |= ERR_RANGE;
    return err;
}

struct InstDev {
    int32_t model, L, N, ndof;
    int32_t nwin, R, first_win, first_slot;
    int32_t bin_shift, escale, chunk, init_mode;
    int64_t J_u, K_u;        // couplings in energy units
    int64_t eglo_u;          // global range start in energy units
    int64_t bin_mul;         // global bin = ((E - eglo_u) * bin_mul) >> bin_shift
    int64_t field_off;       // offset into fields (int64 units per site) or -1
    int64_t qtab_off;        // offset into qtab (cos then sin of q_min x, x < L) or -1 without correlators
    uint64_t seed;           // Philox key: instance_key(descriptor seed)
};

struct WinDev {
    int32_t inst, local, nb, pad;
    int64_t gblo;            // first global bin
    int64_t mask_off;        // offset into the mask array
    int64_t elo_u;           // lower energy edge in units (exact when bin_mul == 1)
};

struct DevPtrs {
    InstDev* inst;
    WinDev* win;
    int32_t* slot_inst;
    int32_t* slot_win;
    int32_t* slot_cfg;
    int64_t* slot_tab;
    int32_t* slot_nb;
    int32_t* slot_flavour;
    uint64_t* slot_sweeps;
    int64_t* slot_draws;
    int64_t* slot_thr_off;
    int64_t* slot_thr_n;
    int64_t* thr;            // replay thresholds
    int64_t* cfg_off;
    int8_t* spins;
    int64_t* cfg_E;
    int32_t* cfg_M;          // 3 per configuration
    int64_t* fields;         // Baxter field per site (units)
    int64_t* g;
    int64_t* gsnap;          // logDoS at the start of an Ashkin-Teller sweep launch
    uint32_t* H;
    uint64_t* visits;
    uint8_t* mask;
    int64_t* win_lnf;
    int32_t* win_done;
    int32_t* win_oot;
    uint64_t* win_iter;
    uint64_t* win_sweepctr;
    int32_t* pairs;          // exchange pair lists: (instance, lower window) for dir 0 then dir 1
    int32_t* counters;       // [0] error word, [1] flat events (this call)
    unsigned long long* xround;  // [0] exchange round (its parity is the pairing direction), [1] blocks done
    unsigned long long* stats;  // [0] exch attempted, [1] exch accepted
    double* obs;             // per-bin observable sums (obs_stride per bin), or null when off
    int obs_stride;          // 3 (Ising) or 12 (a batch with Ashkin-Teller instances); 4 or 16 with correlators
    int corr;                // observables carry the G(q_min) correlators
    const double* qtab;      // per instance: cos(q_min x) then sin(q_min x), x < L
};

// --------------------------------------------------------------------------
// Energies in integer units: the model types of models.cuh
// --------------------------------------------------------------------------
__host__ __device__ inline int64_t global_bin(const InstDev& I, int64_t E)
{
    return ((E - I.eglo_u) * I.bin_mul) >> I.bin_shift;
}

// --------------------------------------------------------------------------
// k_init: initial configuration and the deterministic walk into the window
// --------------------------------------------------------------------------
// REWL_Walker::adjust_state_to_range (src/REWL/rewl_walker.hpp:79-115): visit the sites in
// typewriter order from `start`, flipping a spin whenever that moves the energy towards the
// window, until the energy is inside it.  Ashkin-Teller alternates the flipped plane at the
// end of every pass (change_state toggles at the last site).
template <class Model>
__device__ bool adjust_walk(const InstDev& I, const WinDev& W, int8_t* sp, int64_t& E, int32_t* M, int32_t& flavour,
                            const int64_t* h, uint32_t start, int64_t max_steps)
{
    const int L = I.L, N = I.N;
    const Couplings cp{I.J_u, I.K_u};
    auto in_range = [&](int64_t e) { const int64_t b = global_bin(I, e) - W.gblo; return b >= 0 && b < W.nb; };
    bool in = in_range(E);
    int site = (int)start;
    int64_t steps = 0, idle = 0;
    while (!in) {
        // without a flip the decisions repeat within 2N steps: the walk is stuck for good
        if (++steps > max_steps || ++idle > 2 * (int64_t)N) return false;
        ++site;
        if (site == N) { site = 0; flavour ^= 1; }
        const int plane = Model::kPlanes == 1 ? 0 : flavour;
        const int8_t* a = sp + plane * N;
        const int8_t* b = sp + (plane ^ 1) * N;
        const int64_t dE = Model::delta_energy(a, b, site, L, cp, h ? h[site] : 0);
        if (Model::kPlanes == 2 && site == N - 1) flavour ^= 1;     // change_state toggles at the last site
        const int64_t gb = global_bin(I, E) - W.gblo;
        const bool too_low = gb < 0, too_high = gb >= W.nb;
        const int64_t En = E + dE;
        if ((too_low && En > E) || (too_high && En <= E)) {
            E = En;
            idle = 0;
            Model::flip(sp, N, site, plane, M);      // the plane chosen before a toggle
        }
        in = in_range(E);
    }
    return true;
}

template <class Model>
__device__ void init_walker(const InstDev& I, const WinDev& W, int8_t* sp, const int64_t* h, uint32_t uid,
                            int64_t& E, int32_t* M, int32_t& flavour, bool& ok)
{
    const Couplings cp{I.J_u, I.K_u};
    const int init_random = (int)(I.init_mode == 0);
    for (int i = 0; i < I.ndof; ++i)
        sp[i] = init_random ? ((philox_word(I.seed, uid, (uint64_t)i, kStreamInit) >> 31) ? -1 : 1) : 1;
    Model::recalculate(sp, I.L, cp, h, E, M);
    flavour = 0;
    const uint32_t start = mulhi32(philox_word(I.seed, uid, 0, kStreamAdjust), (uint32_t)I.N);
    const int64_t cap = 4000LL * I.ndof;
    ok = adjust_walk<Model>(I, W, sp, E, M, flavour, h, start, cap);
    // a greedy walk can stick in a local extremum: retry from all +1 (walks up
    // from the ground state) and then from the checkerboard (walks down from the top)
    for (int attempt = 1; attempt <= 2 && !ok; ++attempt) {
        for (int i = 0; i < I.ndof; ++i) {
            const int site = i % I.N, x = site % I.L, y = site / I.L;
            sp[i] = (attempt == 1 || ((x + y) & 1) == 0) ? 1 : -1;
        }
        Model::recalculate(sp, I.L, cp, h, E, M);
        flavour = 0;
        ok = adjust_walk<Model>(I, W, sp, E, M, flavour, h, start, cap);
    }
}

__global__ void k_init(DevPtrs P, int nslots, int init_mode_mask_unused)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const int ii = P.slot_inst[s];
    const InstDev I = P.inst[ii];
    const WinDev W = P.win[P.slot_win[s]];
    const int c = P.slot_cfg[s];
    int8_t* sp = P.spins + P.cfg_off[c];
    const uint32_t uid = (uint32_t)(s - I.first_slot);
    const int64_t* h = I.field_off >= 0 ? P.fields + I.field_off : nullptr;
    int64_t E = 0; int32_t M[3] = {0, 0, 0}; int32_t flavour = 0;
    bool ok = false;
    if (I.model == REWL_MODEL_ISING2D) init_walker<Ising2dModel>(I, W, sp, h, uid, E, M, flavour, ok);
    else init_walker<AshkinTeller2dModel>(I, W, sp, h, uid, E, M, flavour, ok);
    if (!ok) atomicOr(&P.counters[0], ERR_ADJUST);
    P.cfg_E[c] = E;
    P.cfg_M[3 * c] = M[0]; P.cfg_M[3 * c + 1] = M[1]; P.cfg_M[3 * c + 2] = M[2];
    P.slot_flavour[s] = flavour;
}

// Recompute energies and magnetisations of given configurations (after imports).
__global__ void k_recalc(DevPtrs P, const int32_t* cfgs, const int32_t* insts, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int c = cfgs[k];
    const InstDev I = P.inst[insts[k]];
    const int8_t* sp = P.spins + P.cfg_off[c];
    const int64_t* h = I.field_off >= 0 ? P.fields + I.field_off : nullptr;
    int64_t E; int32_t M[3] = {0, 0, 0};
    const Couplings cp{I.J_u, I.K_u};
    if (I.model == REWL_MODEL_ISING2D) Ising2dModel::recalculate(sp, I.L, cp, h, E, M);
    else AshkinTeller2dModel::recalculate(sp, I.L, cp, h, E, M);
    P.cfg_E[c] = E;
    P.cfg_M[3 * c] = M[0]; P.cfg_M[3 * c + 1] = M[1]; P.cfg_M[3 * c + 2] = M[2];
}

// --------------------------------------------------------------------------
// Sweep kernels
// --------------------------------------------------------------------------
// Per-bin observable sums (observables on): for every attempted flip and every
// exchange touch, the walker's observables after it are added at its bin.  Ising:
// |m|, m^2, m^4 with m = M / N (Ising2d::update_observables,
// src/Hamiltonians/Ising2d/ising2d_hamiltonian.hpp:234-256); Ashkin-Teller: the 12
// moments of Ashkin_Teller2d::update_observables (ashkin_teller2d_hamiltonian.hpp:267-318).
// The reference keeps running means (v + c avg) / (c + 1) (ising2d_observables.hpp:134-145);
// the export divides these sums by the visits instead, equal up to FP64 rounding.
// G(q_min) correlators (CORRELATION_LENGTHS, on in the reference's default build).  At
// every visit of a bin whose count before the visit is a multiple of counts_per_transform
// = 1000 (src/Hamiltonians/Correlations/fourier_correlator.hpp:11), the walker's G is added
// at the bin (Ising2d::update_observables, ising2d_hamiltonian.hpp:246-252;
// Ashkin_Teller2d::update_observables, ashkin_teller2d_hamiltonian.hpp:295-315).  The
// reference keeps the running mean over those transforms (ising2d_observables.hpp:148-159);
// the export divides the sum by their number, ceil(visits / 1000).
constexpr unsigned long long kCountsPerTransform = 1000;

// Fourier_Correlator::compute_correlator (fourier_correlator.hpp:65-118) of one plane of
// +-1 values v(y, x): half the squared magnitude of the transform of the row sums over y
// plus that of the column sums over x, both at q_min = 2 pi / L (q: L cosines then L sines).
// rs and cs are the plane's row and column sums before the chunk; the chunk (row y,
// columns x0 ..) has flipped the sites of its steps 0..j whose acceptance bit is set: row
// y changes by dr and column x0 + k by -2 val(k), val(k) the site's value before the
// chunk.  The reference adds the same products site by site in row-major order; the two
// agree to FP64 rounding.
template <class V>
__device__ double plane_corr(const int* rs, const int* cs, const double* q, int L, int y, int dr, int x0, int j,
                             unsigned acc, V val)
{
    double rx = 0.0, ix = 0.0, ry = 0.0, iy = 0.0;
    for (int t = 0; t < L; ++t) {
        const double c = q[t], sn = q[L + t];
        const double r = (double)(rs[t] + (t == y ? dr : 0));
        const int k = t - x0;
        const int cl = cs[t] - ((k >= 0 && k <= j && ((acc >> k) & 1u)) ? 2 * val(k) : 0);
        rx += r * c;
        ix += r * sn;
        ry += (double)cl * c;
        iy += (double)cl * sn;
    }
    return 0.5 * ((rx * rx + ix * ix) + (ry * ry + iy * iy));
}

// Row and column sums of a plane (value(i) for site i) into rs, cs, by `stride` lanes.
template <class V>
__device__ void plane_sums(int* rs, int* cs, int L, int lane, V value, int stride = 32)
{
    for (int t = lane; t < L; t += stride) {
        int r = 0, c = 0;
        for (int u = 0; u < L; ++u) { r += value(t * L + u); c += value(u * L + t); }
        rs[t] = r;
        cs[t] = c;
    }
}

// flips of a chunk's steps 0..j that turned a +1 into -1 minus those that turned -1 into +1
__device__ __forceinline__ int chunk_dm(unsigned acc, unsigned plus, int j)
{
    const unsigned le = j >= 31 ? 0xFFFFFFFFu : ((2u << j) - 1u);
    return -2 * ((int)__popc(acc & plus & le) - (int)__popc(acc & ~plus & le));
}

struct SweepParams {
    DevPtrs P;
    const int32_t* slots;    // walkers of this launch
    int nslots;
    int nsweeps;
    int smem_per_warp;       // bytes
    int nbcap;               // table capacity per warp (Ising, shared memory)
};

// Per-warp staging of one chunk for the lane-0 resolver: energy change without /
// with the left neighbour flipped, wrap correction (x = L-1 sees the row start),
// acceptance threshold.
struct Stage {
    long long T[32];
    int d0[32];
    int d1[32];
    int wc[32];
    int seq[32];             // bin after each step (observables)
};

// Accept chain of one chunk of C sites, executed identically by all 32 lanes
// (every lane holds the same E, b, gc, acc).  Lane j owns site j's precomputed
// values; they reach every lane by shuffles that depend on nothing in the chain,
// so the unrolled loop issues them early.  The proposal of step j+1 depends on
// step j's outcome only through (E, left-neighbour flip, wrap flip): both
// candidates are formed and their logDoS entries loaded before step j resolves,
// which takes the shared-memory latency off the chain.  The only store that can
// land between such a prefetch and its use is step j's own, to the bin step j
// ends in: that case takes the freshly stored value.
template <int C>
__device__ __forceinline__ void resolve_chunk_all_lanes(int& E, int& b, long long& gc, unsigned& acc,
                                                        long long* gs, const int Ewlo, const int sh, const int nb,
                                                        const long long lnf, const int my_d0, const int my_d1,
                                                        const int my_wc, const long long my_T)
{
    int En = E + __shfl_sync(kFull, my_d0, 0);
    int bn = (En - Ewlo) >> sh;
    bool inr = (unsigned)bn < (unsigned)nb;
    long long gn = gs[inr ? bn : b];
#pragma unroll
    for (int j = 0; j < C; ++j) {
        const long long Tj = __shfl_sync(kFull, my_T, j);
        int E0 = 0, E1 = 0, b0 = 0, b1 = 0;
        bool i0 = false, i1 = false;
        long long g0 = 0, g1 = 0;
        if (j + 1 < C) {
            const int d0n = __shfl_sync(kFull, my_d0, j + 1);
            const int d1n = __shfl_sync(kFull, my_d1, j + 1);
            const int wcn = __shfl_sync(kFull, my_wc, j + 1);
            const int w0 = (acc & 1u) ? wcn : 0;
            const int w1 = (j == 0 || (acc & 1u)) ? wcn : 0;
            E0 = E + d0n + w0;
            E1 = En + d1n + w1;
            b0 = (E0 - Ewlo) >> sh;
            b1 = (E1 - Ewlo) >> sh;
            i0 = (unsigned)b0 < (unsigned)nb;
            i1 = (unsigned)b1 < (unsigned)nb;
            g0 = gs[i0 ? b0 : 0];
            g1 = gs[i1 ? b1 : 0];
        }
        const bool a = inr && (gn - gc < Tj);
        if (a) { E = En; b = bn; gc = gn; acc |= 1u << j; }
        gc += lnf;
        gs[b] = gc;
        if (j + 1 < C) {
            En = a ? E1 : E0;
            bn = a ? b1 : b0;
            inr = a ? i1 : i0;
            gn = a ? g1 : g0;
            if (bn == b) gn = gc;
        }
    }
}

// Ising sweeps.  One warp per walker; lattice and logDoS staged in shared memory
// for the whole launch.  Per-stage counts are not kept in the loop: within a
// launch every visit adds the same ln f, so the counts added to bin k are
// (g_end[k] - g_start[k]) / ln f exactly (ln f >= one 2^-36 unit always).
template <bool REPLAY, int VARIANT>
__global__ void __launch_bounds__(256) k_sweep_ising(const SweepParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int li = blockIdx.x * (blockDim.x >> 5) + wib;
    if (li >= p.nslots || engine_failed_warp(p.P.counters)) return;
    const DevPtrs& P = p.P;
    const int s = p.slots[li];
    const InstDev I = P.inst[P.slot_inst[s]];
    const int w = P.slot_win[s];
    const WinDev W = P.win[w];
    const int L = I.L, N = I.N, C = I.chunk, nb = W.nb;
    unsigned char* base = smem + (size_t)wib * p.smem_per_warp;
    long long* gs = reinterpret_cast<long long*>(base);
    Stage* st = reinterpret_cast<Stage*>(gs + p.nbcap);
    int8_t* lat = reinterpret_cast<int8_t*>(st + 1);
    int* rsum = reinterpret_cast<int*>(lat + ((N + 15) & ~15));   // correlators: row and column sums
    int* csum = rsum + L;

    const int cfg = P.slot_cfg[s];
    int8_t* gl = P.spins + P.cfg_off[cfg];
    for (int i = lane; i < N; i += 32) lat[i] = gl[i];
    long long* gg = reinterpret_cast<long long*>(P.g + P.slot_tab[s]);
    for (int k = lane; k < nb; k += 32) gs[k] = gg[k];
    __syncwarp();
    const bool corr = P.obs != nullptr && P.corr;
    if (corr) {
        plane_sums(rsum, csum, L, lane, [&](int i) { return (int)lat[i]; });
        __syncwarp();
    }

    const int J = (int)I.J_u;
    const int sh = I.bin_shift;
    const int Ewlo = (int)W.elo_u;
    const long long lnf = P.win_lnf[w];
    const uint64_t sweeps0 = P.slot_sweeps[s];
    const uint32_t uid = (uint32_t)(s - I.first_slot);
    const uint64_t seed = I.seed;
    const bool obs_on = P.obs != nullptr;   // observables: the lane-0 resolver records each step's bin
    const bool all_lanes = (!REPLAY) && VARIANT == 3 && !obs_on && (C == 32 || C == 16 || C == 24 || C == 8 || C == 4);
    const double invN = 1.0 / (double)N;

    int E = (int)P.cfg_E[cfg];
    int M = P.cfg_M[3 * cfg];
    int b = (E - Ewlo) >> sh;
    if (b < 0 || b >= nb) {
        if (lane == 0) atomicOr(&P.counters[0], ERR_BOUNDS);
        return;
    }
    long long gc = gs[b];
    long long draws = 0, thr_off = 0, thr_n = 0;
    int err = 0;
    if (REPLAY) { draws = P.slot_draws[s]; thr_off = P.slot_thr_off[s]; thr_n = P.slot_thr_n[s]; }

    for (int sw = 0; sw < p.nsweeps; ++sw) {
        const uint64_t A0 = (sweeps0 + (uint64_t)sw) * (uint64_t)N;
        for (int c0 = 0; c0 < N; c0 += C) {
            // chunk = sites c0 .. c0+C-1 of one row (C divides L)
            const int y = c0 / L, x0 = c0 - y * L, x = x0 + lane;
            const int row = y * L;
            int si = 0, d0 = 0, d1 = 0, wc = 0;
            long long T = 0;
            if (lane < C) {
                si = lat[row + x];
                const Couplings cp{J, 0};
                const int i = row + x;
                d0 = (int)Ising2dModel::delta_energy(lat, nullptr, i, L, cp, 0);
                d1 = lane > 0 ? (int)Ising2dModel::left_flipped(lat, nullptr, i, L, cp, d0) : d0;
                wc = (C == L && lane == L - 1) ? (int)Ising2dModel::right_flipped(lat, nullptr, i, L, cp) : 0;
                if (!REPLAY) {
                    const uint32_t word = philox_word(seed, uid, A0 + (uint64_t)(c0 + lane), kStreamWL);
                    T = accept_threshold(neglog_u32(word));
                }
            }
            unsigned acc = 0;
            if (all_lanes) {
                switch (C) {
                case 32: resolve_chunk_all_lanes<32>(E, b, gc, acc, gs, Ewlo, sh, nb, lnf, d0, d1, wc, T); break;
                case 24: resolve_chunk_all_lanes<24>(E, b, gc, acc, gs, Ewlo, sh, nb, lnf, d0, d1, wc, T); break;
                case 16: resolve_chunk_all_lanes<16>(E, b, gc, acc, gs, Ewlo, sh, nb, lnf, d0, d1, wc, T); break;
                case 8: resolve_chunk_all_lanes<8>(E, b, gc, acc, gs, Ewlo, sh, nb, lnf, d0, d1, wc, T); break;
                default: resolve_chunk_all_lanes<4>(E, b, gc, acc, gs, Ewlo, sh, nb, lnf, d0, d1, wc, T); break;
                }
            } else {
                if (lane < C) { st->d0[lane] = d0; st->d1[lane] = d1; st->wc[lane] = wc; st->T[lane] = T; }
                __syncwarp();
                if (lane == 0) {
                    int En = E + st->d0[0];
                    int bn = (En - Ewlo) >> sh;
                    bool inr = (unsigned)bn < (unsigned)nb;
                    long long gn = gs[inr ? bn : b];
                    for (int j = 0; j < C; ++j) {
                        int E0 = 0, E1 = 0, b0 = 0, b1 = 0;
                        bool i0 = false, i1 = false;
                        long long g0 = 0, g1 = 0;
                        if (j + 1 < C) {
                            const int w0 = (acc & 1u) ? st->wc[j + 1] : 0;
                            const int w1 = (j == 0 || (acc & 1u)) ? st->wc[j + 1] : 0;
                            E0 = E + st->d0[j + 1] + w0;
                            E1 = En + st->d1[j + 1] + w1;
                            b0 = (E0 - Ewlo) >> sh;
                            b1 = (E1 - Ewlo) >> sh;
                            i0 = (unsigned)b0 < (unsigned)nb;
                            i1 = (unsigned)b1 < (unsigned)nb;
                            g0 = gs[i0 ? b0 : 0];
                            g1 = gs[i1 ? b1 : 0];
                        }
                        const long long d = gn - gc;
                        bool a;
                        if (!REPLAY) {
                            a = inr && (d < st->T[j]);
                        } else if (inr && d > 0) {
                            if (draws >= thr_n) { err = ERR_REPLAY_EXHAUSTED; a = false; }
                            else { a = d < P.thr[thr_off + draws]; ++draws; }
                        } else {
                            a = inr;
                        }
                        if (a) { E = En; b = bn; gc = gn; acc |= 1u << j; }
                        gc += lnf;
                        gs[b] = gc;
                        if (obs_on) st->seq[j] = b;
                        En = a ? E1 : E0;
                        bn = a ? b1 : b0;
                        inr = a ? i1 : i0;
                        gn = a ? g1 : g0;
                        if (bn == b) gn = gc;
                    }
                }
                // lane 0 holds the chain state; every lane needs it
                acc = __shfl_sync(kFull, acc, 0);
                E = __shfl_sync(kFull, E, 0);
                b = __shfl_sync(kFull, b, 0);
                gc = __shfl_sync(kFull, gc, 0);
                if (REPLAY) { draws = __shfl_sync(kFull, draws, 0); err = __shfl_sync(kFull, err, 0); }
            }
            const unsigned plus = __ballot_sync(kFull, lane < C && si > 0);
            if (obs_on) {
                __syncwarp();
                if (lane < C)
                {
                    const int32_t Mv[1] = {M + chunk_dm(acc, plus, lane)};
                    Ising2dModel::add_observables(P.obs + (size_t)(P.slot_tab[s] + st->seq[lane]) * P.obs_stride, Mv,
                                                  invN, P.corr);
                }
                if (corr) {
                    const int bin = lane < C ? st->seq[lane] : -1 - lane;
                    const unsigned grp = __match_any_sync(kFull, bin);
                    if (lane < C) {
                        // the bin's count before step `lane`: its visits after the chunk (the
                        // launch's start value plus the change of g over ln f) minus the chunk's
                        // visits to it from step `lane` on
                        const unsigned long long after =
                            P.visits[P.slot_tab[s] + bin] + (unsigned long long)((gs[bin] - gg[bin]) / lnf);
                        const unsigned long long seen = after - (unsigned long long)__popc(grp >> lane);
                        if (seen % kCountsPerTransform == 0) {
                            const double G = plane_corr(rsum, csum, P.qtab + I.qtab_off, L, y, chunk_dm(acc, plus, lane),
                                                        x0, lane, acc, [&](int k) { return (int)lat[row + x0 + k]; });
                            atomicAdd(P.obs + (size_t)(P.slot_tab[s] + bin) * P.obs_stride + 3, invN * invN * G);
                        }
                    }
                    __syncwarp();
                    // the chunk's flips into the row and column sums
                    if (lane < C && ((acc >> lane) & 1u)) csum[x] -= 2 * si;
                    if (lane == 0) rsum[y] += -2 * ((int)__popc(acc & plus) - (int)__popc(acc & ~plus));
                }
            }
            if (lane < C && ((acc >> lane) & 1u)) lat[row + x] = (int8_t)(-si);
            M += -2 * ((int)__popc(acc & plus) - (int)__popc(acc & ~plus));
            __syncwarp();
        }
    }
    // write back: lattice, logDoS, counts and visits derived from the logDoS change
    for (int i = lane; i < N; i += 32) gl[i] = lat[i];
    uint32_t* gH = P.H + P.slot_tab[s];
    uint64_t* gv = P.visits + P.slot_tab[s];
    for (int k = lane; k < nb; k += 32) {
        const long long gnew = gs[k];
        const long long dv = (gnew - gg[k]) / lnf;
        const int e = commit_visits(gH, gv, k, dv, gnew);
        if (e) atomicOr(&P.counters[0], e);
        gg[k] = gnew;
    }
    if (lane == 0) {
        P.cfg_E[cfg] = E;
        P.cfg_M[3 * cfg] = M;
        P.slot_sweeps[s] = sweeps0 + (uint64_t)p.nsweeps;
        if (REPLAY) P.slot_draws[s] = draws;
        if (err) atomicOr(&P.counters[0], err);
    }
}

// ---------------------------------------------------------------------------
// Bin-tracking Ising sweeps (used when every energy change is a whole number of
// bins: 4|J| divisible by the bin width, as for J = 1 and width 4).  The chain
// then carries only the bin index b and the logDoS value g[b].
//
// G walkers share a warp (P = 32/G lanes each).  For each chunk the walker's
// lanes first form, per site: the integer acceptance threshold, the packed bin
// changes (without / with the left neighbour flipped, wrap term for x = L-1)
// and the spin.
// ---------------------------------------------------------------------------
struct __align__(16) SiteRec {
    long long T;    // accept iff d < T
    int pk;         // bytes: bin change, same with left neighbour flipped, wrap term
    int s;          // spin
};


// The accept chain, all lanes of a walker in lockstep, with the table reads one
// site ahead.  While site j is being decided, the two bins site j+1 may propose
// (one if site j is rejected, one if it is accepted -- which moves the walker
// and flips the left neighbour of site j+1) are already being loaded, so the
// load latency overlaps the decision.  Per site the dependent work is then:
// one 64-bit compare of g(proposal) against g(current) + threshold, a select of
// the taken branch and one add.
//
// A prefetched load follows the commit store of the site before it, so it is
// stale only when it reads the bin the next commit writes, i.e. exactly when
// its proposal keeps the bin (offset change 0); the value is then the one just
// committed.
//
// The table carries kGuard sentinel bins on each side holding INT64_MAX, so a
// proposal outside the window fails the compare by itself whatever g holds (no
// range checks): the current bin never leaves the window, and prefetches issued
// from an out-of-window proposal stay inside the table.  Bin
// positions are byte offsets into the table.
//
// The chain runs without a break from chunk to chunk: the first offsets of the
// next chunk are formed from the lattice before the current chunk's flips, then
// corrected for the neighbours the current chunk flips as soon as those are
// decided, and handed to all lanes by shuffle; thresholds come from one Philox
// block per four sites, 4C sites at a time, one batch ahead.
constexpr int kGuard = 8;
constexpr long long kGuardValue = 0x7FFFFFFFFFFFFFFFLL;   // never below g + threshold

__device__ __forceinline__ long long lds64(const char* base, int off)
{
    return *reinterpret_cast<const long long*>(base + off);
}
__device__ __forceinline__ void sts64(char* base, int off, long long v) { *reinterpret_cast<long long*>(base + off) = v; }

// The sweeps of one warp's G walkers (launch position warp_index; its shared memory starts at
// warp_base, one region of p.smem_per_warp bytes per walker).
template <int G, int C, bool OBS, bool LEAN>
__device__ __forceinline__ void sweep_bins_warp(const SweepParams& p, const int warp_index, unsigned char* warp_base)
{
    constexpr int P = 32 / G;
    constexpr int SPL = (C + P - 1) / P;          // sites per lane in a chunk
    constexpr int BPL = (C + P - 1) / P;          // Philox blocks per lane in a batch of 4C sites
    constexpr int kAhead = 4;                     // per-site inputs are read this many sites early
    // LEAN: each step reads g at the next proposal after its own write (no candidate prefetch,
    // no staleness select): five fewer ALU instructions per step and a dependent shared-memory
    // load on the chain, which pays where enough warps share an SM to hide it
    constexpr bool kLean = LEAN;
    static_assert(!LEAN || G > 1, "the lean chain is for warps of several walkers");
    static_assert(C % 4 == 0 && C >= 4 && C <= 32 && P >= 4, "chunk");
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int grp = lane / P, q = lane - grp * P, gbase = grp * P;
    const int li = warp_index * G + grp;
    const bool valid = li < p.nslots;
    if (__ballot_sync(kFull, valid) == 0 || engine_failed_warp(p.P.counters)) return;   // no walkers, or stopped
    const DevPtrs& P_ = p.P;
    const int s = p.slots[valid ? li : 0];                     // idle groups shadow a walker, never write
    const InstDev I = P_.inst[P_.slot_inst[s]];
    const int w = P_.slot_win[s];
    const WinDev W = P_.win[w];
    const int L = I.L, N = I.N, nb = W.nb;
    unsigned char* base = warp_base + (size_t)grp * p.smem_per_warp;
    const int gs_bytes = ((p.nbcap + 2 * kGuard) * 8 + 15) & ~15;
    long long* gs = reinterpret_cast<long long*>(base) + kGuard;     // gs[-kGuard .. nb+kGuard)
    int8_t* lat = reinterpret_cast<int8_t*>(base + gs_bytes);
    long long* Tb = reinterpret_cast<long long*>(base + gs_bytes + ((N + 15) & ~15));   // 2 x 4C thresholds
    int2* Db = reinterpret_cast<int2*>(Tb + 8 * C);                                   // 2 x C offset pairs
    int* seqb = reinterpret_cast<int*>(Db + 2 * C);                                   // C bins (observables)
    int* rsum = seqb + C;                                                             // correlators: row sums,
    int* csum = rsum + L;                                                             // column sums,
    int* bcnt = csum + L;                                                             // bin counts mod 1000
    // table positions are byte offsets from the start of shared memory, so that the
    // accesses need no address arithmetic
    char* const sm = reinterpret_cast<char*>(smem);
    const int gsoff = (int)(reinterpret_cast<char*>(gs) - sm);

    const int cfg = P_.slot_cfg[s];
    int8_t* gl = P_.spins + P_.cfg_off[cfg];
    long long* gg = reinterpret_cast<long long*>(P_.g + P_.slot_tab[s]);
    for (int i = q; i < N; i += P) lat[i] = gl[i];
    for (int k = q; k < nb; k += P) gs[k] = gg[k];
    for (int k = q; k < kGuard; k += P) { gs[-1 - k] = kGuardValue; gs[nb + k] = kGuardValue; }
    __syncwarp();
    const bool corr = OBS && P_.corr;
    if (corr) {
        plane_sums(rsum, csum, L, q, [&](int i) { return (int)lat[i]; }, P);
        const uint64_t* gv0 = P_.visits + P_.slot_tab[s];
        for (int k = q; k < nb; k += P) bcnt[k] = (int)(gv0[k] % kCountsPerTransform);
        __syncwarp();
    }

    const int J = (int)I.J_u;
    const int sh = I.bin_shift;                        // energy change -> bin change (x8: byte offset)
    const int Ewlo = (int)W.elo_u;
    const long long lnf = P_.win_lnf[w];
    const uint64_t sweeps0 = P_.slot_sweeps[s];
    const uint32_t uid = (uint32_t)(s - I.first_slot);
    const uint32_t k0 = (uint32_t)I.seed ^ uid, k1 = (uint32_t)(I.seed >> 32);
    const bool wraps = C == L;                         // a row is one chunk: its last site sees the row start

    const int E0 = (int)P_.cfg_E[cfg];
    const int b0 = (E0 - Ewlo) >> sh;
    const bool bad = ((E0 - Ewlo) & ((1 << sh) - 1)) != 0 || b0 < 0 || b0 >= nb;
    if (__ballot_sync(kFull, valid && bad)) {
        if (lane == 0) atomicOr(&P_.counters[0], ERR_BOUNDS);
        return;
    }
    int M = P_.cfg_M[3 * cfg];

    // thresholds (+ ln f) of the 4C sites from attempt A0 on into Tb[buf]
    auto draw = [&](uint64_t A0, int buf) {
        longlong2* dst = reinterpret_cast<longlong2*>(Tb + buf * 4 * C);
#pragma unroll
        for (int k = 0; k < BPL; ++k) {
            const int bi = q + k * P;
            if (bi < C) {
                const uint64_t a = A0 + (uint64_t)(4 * bi);
                const Philox4 r = philox4x32_10(Philox4{(uint32_t)(a >> 2), (uint32_t)(a >> 34), kStreamWL, 0u}, k0, k1);
                longlong2 t01, t23;
                t01.x = accept_threshold(neglog_u32(r.x)) + lnf;
                t01.y = accept_threshold(neglog_u32(r.y)) + lnf;
                t23.x = accept_threshold(neglog_u32(r.z)) + lnf;
                t23.y = accept_threshold(neglog_u32(r.w)) + lnf;
                dst[2 * bi] = t01;
                dst[2 * bi + 1] = t23;
            }
        }
    };

    // Inputs of a chunk formed from the lattice as it stands, before the flips of the
    // chunk processed meanwhile (which starts at site c0prev, or -1): per site the
    // spin, the energy change without / with the previous site of the sequence
    // flipped, and for the neighbours lying in the chunk at c0prev (other than the
    // previous site) their bit there and the correction 4 J s s_nbr if it flips.
    int ns[SPL], nd0[SPL], nd1[SPL], nbit[SPL][2], ncoef[SPL][2], nwrap = 0;
    auto prepare = [&](int y, int x0, int c0prev) {
        const int row = y * L;
        const int up = (y == 0 ? L - 1 : y - 1) * L, down = (y == L - 1 ? 0 : y + 1) * L;
        nwrap = 0;
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int jj = q + k * P;
            ns[k] = 0; nd0[k] = 0; nd1[k] = 0;
            nbit[k][0] = nbit[k][1] = -1; ncoef[k][0] = ncoef[k][1] = 0;
            if (jj < C) {
                const int x = x0 + jj;
                const int xl = x == 0 ? L - 1 : x - 1, xr = x == L - 1 ? 0 : x + 1;
                const int si = lat[row + x];
                const int su = lat[up + x], sl = lat[row + xl], sr = lat[row + xr];
                const int d0 = 2 * J * si * (su + sl + sr + lat[down + x]);
                ns[k] = si;
                nd0[k] = d0;
                nd1[k] = x > 0 ? d0 - 4 * J * si * sl : d0;        // x > 0: the left site comes just before
                if (jj == C - 1 && wraps) nwrap = -4 * J * si * sr;
                const int ou = up + x - c0prev, orr = row + xr - c0prev;
                if (c0prev >= 0 && (unsigned)ou < (unsigned)C) { nbit[k][0] = ou; ncoef[k][0] = 4 * J * si * su; }
                if (c0prev >= 0 && xr == 0 && (unsigned)orr < (unsigned)C) { nbit[k][1] = orr; ncoef[k][1] = 4 * J * si * sr; }
            }
        }
    };
    // offsets of prepared site slot k once the bits of `acc` it depends on are known
    auto finish = [&](int k, unsigned acc) {
        int corr = 0;
#pragma unroll
        for (int n = 0; n < 2; ++n)
            if (nbit[k][n] >= 0 && ((acc >> nbit[k][n]) & 1u)) corr += ncoef[k][n];
        return make_int2(((nd0[k] - corr) >> sh) * 8, ((nd1[k] - corr) >> sh) * 8);
    };

    // ---- chunk 0 ----
    int cs[SPL];                                        // spins of the current chunk
    int2 E_[4];                                         // offsets of the first 4 sites of the chunk
    long long T_[4];                                    // thresholds of the first 4 sites of the chunk
    int cwrap;
    draw(sweeps0 * (uint64_t)N, 0);
    prepare(0, 0, -1);
    {
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int jj = q + k * P;
            cs[k] = ns[k];
            if (jj < C) Db[jj] = finish(k, 0u);
        }
        cwrap = __shfl_sync(kFull, (nwrap >> sh) * 8, gbase + (C - 1) % P);
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 4; ++i) { E_[i] = Db[i]; T_[i] = Tb[i]; }

    int bc = gsoff + b0 * 8;                            // shared offset of the current bin
    long long gcv = gs[b0];                             // g at the current bin
    int bp = bc + E_[0].x;                              // site 0: proposal (left neighbour unprocessed)
    long long LD = lds64(sm, bp);                       // g at the proposed bin
    int q0 = bc + E_[1].x, q1 = bp + E_[1].y;           // site 1 if site 0 is rejected / accepted
    long long l0 = 0, l1 = 0;
    if (!kLean) { l0 = lds64(sm, q0); l1 = lds64(sm, q1); }
    long long gcT = gcv - lnf + T_[0];                  // g at the current bin + threshold

    const int nch = N / C;
    const int total = p.nsweeps * nch;
    int y = 0, x0 = 0;                                  // position of the current chunk
    for (int t = 0; t < total; ++t) {
        const int tn = t + 1;                           // the next chunk (wraps into the next sweep)
        int yn = y, xn = x0 + C;
        if (xn == L) { xn = 0; yn = y + 1 == L ? 0 : y + 1; }
        const int c0 = y * L + x0;
        const long long* Tc = Tb + ((t >> 2) & 1) * 4 * C + (t & 3) * C;
        const long long* Tn = Tb + ((tn >> 2) & 1) * 4 * C + (tn & 3) * C;
        const int2* Dc = Db + (t & 1) * C;
        int2* Dn = Db + (tn & 1) * C;
        if ((tn & 3) == 0 && tn < total) {
            // the next chunk opens a batch: draw it now (its buffer is not in use)
            const int swn = tn / nch;
            draw((sweeps0 + (uint64_t)swn) * (uint64_t)N + (uint64_t)((tn - swn * nch) * C), (tn >> 2) & 1);
            __syncwarp();
        }
        prepare(yn, xn, c0);
        long long Tnext0 = Tn[0];

        long long Tr[C + 1];
        int2 Er[C];
        Tr[0] = T_[0];
#pragma unroll
        for (int i = 1; i < 4; ++i) Tr[i] = T_[i];
#pragma unroll
        for (int i = 0; i < 4; ++i) Er[i] = E_[i];
        unsigned acc = 0;
#pragma unroll
        for (int j = 0; j < C; ++j) {
            if ((j & 1) == 0 && j + kAhead + 2 <= C) {
                const int jn = j + kAhead;
                const longlong2 tv = reinterpret_cast<const longlong2*>(Tc)[jn >> 1];
                Tr[jn] = tv.x; Tr[jn + 1] = tv.y;
                const int4 d = reinterpret_cast<const int4*>(Dc)[jn >> 1];
                Er[jn] = make_int2(d.x, d.y); Er[jn + 1] = make_int2(d.z, d.w);
            }
            if (j == C - 1) Tr[C] = Tnext0;
            const bool a = LD < gcT;
            const long long sel = a ? LD : gcv;
            const long long gnew = sel + lnf;
            const int bnew = a ? bp : bc;
            sts64(sm, bnew, gnew);
            if (OBS) seqb[j] = bnew;
            if (a) acc |= 1u << j;
            if (j == 1 || j == 3) {
                // next chunk's sites j-1, j: the neighbours they have in this chunk are decided
#pragma unroll
                for (int i = j - 1; i <= j; ++i) {
                    const int2 v = finish(i / P, acc);
                    E_[i] = make_int2(__shfl_sync(kFull, v.x, gbase + i % P), __shfl_sync(kFull, v.y, gbase + i % P));
                }
            }
            gcT = sel + Tr[j + 1];                     // gnew + threshold of site j+1
            bp = a ? q1 : q0;
            if (kLean) {
                LD = lds64(sm, bp);                    // read after this step's write: current
            } else {
                const long long lt = a ? l1 : l0;
                LD = bp == bnew ? gnew : lt;           // the prefetch read the bin just committed
            }
            const int2 ev = (j + 2 < C) ? Er[j + 2] : E_[j + 2 - C];
            int e0 = ev.x, e1 = ev.y;
            if (j + 2 == C - 1) {                      // a row's last site sees the row start
                const int wv = (wraps && (acc & 1u)) ? cwrap : 0;
                e0 += wv; e1 += wv;
            }
            q0 = bnew + e0;
            q1 = bp + e1;
            if (!kLean) {
                l0 = lds64(sm, q0);
                l1 = lds64(sm, q1);
            }
            bc = bnew;
            gcv = gnew;
        }
        // apply the chunk's flips and the magnetisation change
        {
            unsigned plus = 0;
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int jj = q + k * P;
                const unsigned bal = __ballot_sync(kFull, jj < C && cs[k] > 0);
                const unsigned mine = P == 32 ? bal : ((bal >> gbase) & ((1u << P) - 1u));
                plus |= (k * P < 32) ? (mine << (k * P)) : 0u;
                if (jj < C && ((acc >> jj) & 1u)) lat[c0 + jj] = (int8_t)(-cs[k]);
            }
            const unsigned full = C == 32 ? 0xFFFFFFFFu : ((1u << C) - 1u);
            if (OBS) __syncwarp();
            if (OBS && valid) {
                double* ob = P_.obs + (size_t)P_.slot_tab[s] * P_.obs_stride;
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    const int jj = q + k * P;
                    if (jj < C)
                    {
                        const int32_t Mv[1] = {M + chunk_dm(acc, plus, jj)};
                        Ising2dModel::add_observables(ob + (size_t)((seqb[jj] - gsoff) >> 3) * P_.obs_stride, Mv,
                                                      1.0 / (double)N, P_.corr);
                    }
                }
            }
            if (corr) {
                // G(q_min) at the steps whose bin count before the visit is a multiple of 1000:
                // bcnt holds every bin's count before this chunk (mod 1000), to which the chunk's
                // earlier visits to the bin are added.  The chunk's bins are read once into
                // registers (broadcast loads) and compared there.  The lattice already holds the
                // chunk's flips: an accepted site's value before the chunk is minus its value now.
                int first[SPL], total[SPL];
#pragma unroll
                for (int k = 0; k < SPL; ++k) { first[k] = 0; total[k] = 0; }
                if (valid) {
                    int sq[C];
#pragma unroll
                    for (int j2 = 0; j2 < C; j2 += 4) {
                        const int4 v = reinterpret_cast<const int4*>(seqb)[j2 >> 2];
                        sq[j2] = v.x; sq[j2 + 1] = v.y; sq[j2 + 2] = v.z; sq[j2 + 3] = v.w;
                    }
                    const double invN = 1.0 / (double)N;
                    double* ob = P_.obs + (size_t)P_.slot_tab[s] * P_.obs_stride;
#pragma unroll
                    for (int k = 0; k < SPL; ++k) {
                        const int jj = q + k * P;
                        if (jj >= C) continue;
                        const int off = seqb[jj], b = (off - gsoff) >> 3;
                        int earlier = 0, all = 0;
#pragma unroll
                        for (int j2 = 0; j2 < C; ++j2) {
                            const int eq = sq[j2] == off ? 1 : 0;
                            earlier += j2 < jj ? eq : 0;
                            all += eq;
                        }
                        first[k] = earlier == 0;
                        total[k] = all;
                        if ((bcnt[b] + earlier) % (int)kCountsPerTransform == 0) {
                            const double Gq = plane_corr(rsum, csum, P_.qtab + I.qtab_off, L, y, chunk_dm(acc, plus, jj), x0,
                                                         jj, acc, [&](int kk) { return -(int)lat[c0 + kk]; });
                            atomicAdd(ob + (size_t)b * P_.obs_stride + 3, invN * invN * Gq);
                        }
                    }
                }
                __syncwarp();
                // the chunk's flips into the row and column sums, its visits into the counts (by
                // the first step at each bin)
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    const int jj = q + k * P;
                    if (valid && jj < C && ((acc >> jj) & 1u)) csum[x0 + jj] += 2 * (int)lat[c0 + jj];
                    if (valid && jj < C && first[k]) bcnt[(seqb[jj] - gsoff) >> 3] += total[k];
                }
                if (valid && q == 0) rsum[y] += -2 * ((int)__popc(acc & plus) - (int)__popc(acc & ~plus & full));
                __syncwarp();
            }
            M += -2 * ((int)__popc(acc & plus) - (int)__popc(acc & ~plus & full));
        }
        // publish the next chunk: spins, offsets, wrap term, first thresholds
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int jj = q + k * P;
            cs[k] = ns[k];
            if (jj < C) Dn[jj] = finish(k, acc);
        }
        cwrap = __shfl_sync(kFull, (nwrap >> sh) * 8, gbase + (C - 1) % P);
        __syncwarp();
#pragma unroll
        for (int i = 0; i < 4; ++i) T_[i] = Tn[i];
        y = yn; x0 = xn;
    }
    __syncwarp();
    if (valid) {
        for (int i = q; i < N; i += P) gl[i] = lat[i];
        uint32_t* gH = P_.H + P_.slot_tab[s];
        uint64_t* gv = P_.visits + P_.slot_tab[s];
        for (int k = q; k < nb; k += P) {
            const long long gnew = gs[k];
            const long long dv = (gnew - gg[k]) / lnf;
            const int e = commit_visits(gH, gv, k, dv, gnew);
            if (e) atomicOr(&P_.counters[0], e);
            gg[k] = gnew;
        }
        if (q == 0) {
            if ((unsigned)(bc - gsoff) >= (unsigned)(nb * 8)) atomicOr(&P_.counters[0], ERR_BOUNDS);
            P_.cfg_E[cfg] = (long long)Ewlo + ((long long)((bc - gsoff) >> 3) << sh);
            P_.cfg_M[3 * cfg] = M;
            P_.slot_sweeps[s] = sweeps0 + (uint64_t)p.nsweeps;
        }
    }
}

template <int G, int C, bool OBS, bool LEAN>
__global__ void __launch_bounds__(128, 1) k_sweep_ising_bins(const SweepParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int wib = threadIdx.x >> 5;
    sweep_bins_warp<G, C, OBS, LEAN>(p, blockIdx.x * (blockDim.x >> 5) + wib, smem + (size_t)wib * G * p.smem_per_warp);
}

template <int G, bool OBS, bool LEAN>
void launch_bins_t(int C, dim3 grid, dim3 block, size_t smem, cudaStream_t st, const SweepParams& sp)
{
    switch (C) {
    case 32: k_sweep_ising_bins<G, 32, OBS, LEAN><<<grid, block, smem, st>>>(sp); break;
    case 24: k_sweep_ising_bins<G, 24, OBS, LEAN><<<grid, block, smem, st>>>(sp); break;
    case 16: k_sweep_ising_bins<G, 16, OBS, LEAN><<<grid, block, smem, st>>>(sp); break;
    case 8: k_sweep_ising_bins<G, 8, OBS, LEAN><<<grid, block, smem, st>>>(sp); break;
    default: k_sweep_ising_bins<G, 4, OBS, LEAN><<<grid, block, smem, st>>>(sp); break;
    }
}

// lean: the chain without the candidate prefetch (several walkers per warp, enough warps per SM
// to hide the shared-memory latency it exposes; observables off)
template <int G>
void launch_bins(int C, dim3 grid, dim3 block, size_t smem, cudaStream_t st, const SweepParams& sp, bool lean)
{
    if (sp.P.obs) launch_bins_t<G, true, false>(C, grid, block, smem, st, sp);
    else if (G > 1 && lean) launch_bins_t<G, false, (G > 1)>(C, grid, block, smem, st, sp);
    else launch_bins_t<G, false, false>(C, grid, block, smem, st, sp);
}

template <int G, bool OBS, bool LEAN>
cudaError_t allow_bins_smem_t()
{
    cudaError_t e = cudaSuccess;
    e = e != cudaSuccess ? e : cudaFuncSetAttribute(k_sweep_ising_bins<G, 32, OBS, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    e = e != cudaSuccess ? e : cudaFuncSetAttribute(k_sweep_ising_bins<G, 24, OBS, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    e = e != cudaSuccess ? e : cudaFuncSetAttribute(k_sweep_ising_bins<G, 16, OBS, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    e = e != cudaSuccess ? e : cudaFuncSetAttribute(k_sweep_ising_bins<G, 8, OBS, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    e = e != cudaSuccess ? e : cudaFuncSetAttribute(k_sweep_ising_bins<G, 4, OBS, LEAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    return e;
}

template <int G>
cudaError_t allow_bins_smem()
{
    cudaError_t e = allow_bins_smem_t<G, false, false>();
    e = e != cudaSuccess ? e : allow_bins_smem_t<G, true, false>();
    if (G > 1) e = e != cudaSuccess ? e : allow_bins_smem_t<G, false, (G > 1)>();
    return e;
}

// Ashkin-Teller: sweep = sigma pass then tau pass (wang_landau.hpp:109-119); the
// flavour toggles after each pass.  A window holds tens of thousands of bins, so
// its logDoS stays in global memory: each step reads g at the proposal and writes
// g at the current bin, nothing else.  The counts and visits of the launch are
// derived at its end from the change of g against a copy taken at its start
// (every visit adds the same ln f), and the chain loads both possible proposals
// of the next step one step ahead, so a load's latency overlaps a decision.
// bins either side of the walker's bin prefetched into L1 per chunk (measured on the Ashkin-Teller
// benchmark: 256 / 384 / 512 / 768 / 1024 bins 43.5 / 43.3 / 43.4 / 43.9 / 44.1 ms per launch)
constexpr int kTableReach = 512;

struct TableStage {
    longlong2 du[32];        // per site: {proposal, proposal after its left neighbour flipped in this chunk}
    long long T[32];         // acceptance thresholds of the chunk's sites
    long long wcu;           // row-wrap correction of the last site when the chunk is a whole row
    int seq[32];             // bin after each step (observables)
};

// Chain state of one Ashkin-Teller walker (lane 0).  The energy is carried as its
// position v = (E - E_lo) * bin_mul - gblo << bin_shift, in units of the bin
// numerator within the window, so that a proposal's bin is (v + dv) >> bin_shift:
// one add and one shift instead of a multiply per candidate.
struct TableChain {
    long long v, vn, gc, draws;
    long long G0, G1;        // logDoS loaded for step j's proposal if step j-1 was rejected / accepted
    long long T;             // step j's threshold
    longlong2 q;             // step j+1's proposals
    int b, bn, err;
    bool inr, ap;            // step j's proposal in the window; step j-1 accepted
    unsigned acc;
};

// One step j of the chunk, software-pipelined two deep.  On entry (vn, bn, inr) is
// step j's proposal, and its logDoS is G1 or G0 (as step j-1 was accepted or not),
// loaded during step j-1.  With PREFETCH the two proposals of step j+1 (step j
// rejected: from v; accepted: from vn) are loaded first, before step j waits on
// its own loads, so two steps' loads are in flight at once.  A value loaded before
// step j-1's write to bin b is stale exactly when the proposal is b: gc replaces
// it.  LOADQ: step j+2 exists and its proposals are read from shared memory now.
// WRAPFIX: step j+1 is the last site of a whole-row chunk, whose right neighbour
// is the row's first site, flipped in this chunk iff bit 0 of acc.
template <bool REPLAY, bool OBS, bool PREFETCH, bool LOADQ, bool WRAPFIX>
__device__ __forceinline__ void table_step(TableChain& c, const int j, TableStage* st, long long* gg, const int nb,
                                        const int sh, const long long lnf, const DevPtrs& P,
                                        const long long thr_off, const long long thr_n)
{
    long long t0 = 0, t1 = 0, G0 = 0, G1 = 0, Tn = 0;
    longlong2 qn = make_longlong2(0, 0);
    int b0 = 0, b1 = 0;
    bool i0 = false, i1 = false;
    if (LOADQ) qn = st->du[j + 2];
    if (PREFETCH) {
        if (!REPLAY) Tn = st->T[j + 1];
        t0 = c.v + c.q.x;
        t1 = c.vn + c.q.y;
        if (WRAPFIX) {
            const long long wcu = st->wcu;
            if (c.acc & 1u) t0 += wcu;
            if (j == 0 || (c.acc & 1u)) t1 += wcu;
        }
        b0 = (int)(t0 >> sh);
        b1 = (int)(t1 >> sh);
        i0 = (unsigned)b0 < (unsigned)nb;
        i1 = (unsigned)b1 < (unsigned)nb;
        G0 = gg[min((unsigned)b0, (unsigned)(nb - 1))];
        G1 = gg[min((unsigned)b1, (unsigned)(nb - 1))];
    }
    const long long gn = c.bn == c.b ? c.gc : (c.ap ? c.G1 : c.G0);
    const long long d = gn - c.gc;
    bool a;
    if (!REPLAY) {
        a = c.inr && (d < c.T);
    } else if (c.inr && d > 0) {
        if (c.draws >= thr_n) { c.err = ERR_REPLAY_EXHAUSTED; a = false; }
        else { a = d < P.thr[thr_off + c.draws]; ++c.draws; }
    } else {
        a = c.inr;
    }
    if (a) { c.v = c.vn; c.b = c.bn; c.gc = gn; c.acc |= 1u << j; }
    c.gc += lnf;
    gg[c.b] = c.gc;
    if (OBS) st->seq[j] = c.b;
    if (PREFETCH) {
        c.vn = a ? t1 : t0;
        c.bn = a ? b1 : b0;
        c.inr = a ? i1 : i0;
        c.G0 = G0; c.G1 = G1; c.ap = a;
        c.T = Tn;
        c.q = qn;
    }
}

// Sweeps of any model type of models.cuh with the window tables in global memory (the
// Ashkin-Teller instances, whose windows hold tens of thousands of bins, and Ising windows too
// large for shared memory).  One warp per walker; the planes sweep in turn (sigma then tau for
// Ashkin-Teller, wang_landau.hpp:109-119), the flipped plane toggling after each pass.
// The sweeps of one walker (launch position li; the warp's shared memory starts at warp_base).
template <class Model, bool REPLAY, bool OBS>
__device__ __forceinline__ void sweep_tables_warp(const SweepParams& p, const int li, unsigned char* warp_base)
{
    constexpr int NP = Model::kPlanes, NM = Model::kMags, NC = Model::kCorrPlanes;
    const int lane = threadIdx.x & 31;
    if (li >= p.nslots || engine_failed_warp(p.P.counters)) return;
    const DevPtrs& P = p.P;
    const int s = p.slots[li];
    const InstDev I = P.inst[P.slot_inst[s]];
    const int w = P.slot_win[s];
    const WinDev W = P.win[w];
    const int L = I.L, N = I.N, C = I.chunk, nb = W.nb;
    unsigned char* base = warp_base;
    TableStage* st = reinterpret_cast<TableStage*>(base);
    int8_t* sp = reinterpret_cast<int8_t*>(st + 1);       // NP planes of N spins
    const int64_t* hf = I.field_off >= 0 ? P.fields + I.field_off : nullptr;

    const int cfg = P.slot_cfg[s];
    int8_t* gl = P.spins + P.cfg_off[cfg];
    for (int i = lane; i < NP * N; i += 32) sp[i] = gl[i];
    long long* gg = reinterpret_cast<long long*>(P.g + P.slot_tab[s]);
    long long* g0 = reinterpret_cast<long long*>(P.gsnap + P.slot_tab[s]);
    for (int k = lane; k < nb; k += 32) g0[k] = gg[k];
    __syncwarp();
    // correlators: row sums rs[p] and column sums cs[p] of every correlator plane
    int* sums = reinterpret_cast<int*>(sp + ((NP * N + 15) & ~15));
    const bool corr = OBS && P.corr;
    const double invN = 1.0 / (double)N;
    if (corr) {
        for (int cp = 0; cp < NC; ++cp)
            plane_sums(sums + 2 * L * cp, sums + 2 * L * cp + L, L, lane,
                       [&](int i) { return Model::corr_site(sp, N, i, cp); });
        __syncwarp();
    }

    const Couplings cpl{I.J_u, I.K_u};
    const long long lnf = P.win_lnf[w];
    const uint64_t sweeps0 = P.slot_sweeps[s];
    const uint32_t uid = (uint32_t)(s - I.first_slot);
    const uint64_t seed = I.seed;
    const long long eglo = I.eglo_u, mul = I.bin_mul;
    const int sh = I.bin_shift;
    const long long vlo = (long long)W.gblo << sh;     // window start in bin-numerator units
    const bool wraps = C == L;
    int flavour = NP == 1 ? 0 : P.slot_flavour[s];

    TableChain c{};
    int32_t M[3] = {0, 0, 0};                          // lane 0: the magnetisations
    long long thr_off = 0, thr_n = 0;
    int err = 0;
    if (lane == 0) {
        const long long E = P.cfg_E[cfg];
        for (int m = 0; m < NM; ++m) M[m] = P.cfg_M[3 * cfg + m];
        c.v = (E - eglo) * mul - vlo;
        const long long gb = c.v >> sh;
        if (gb < 0 || gb >= nb) err = ERR_BOUNDS;
        c.b = (int)(err ? 0 : gb);
        c.gc = gg[c.b];
        if (REPLAY) { c.draws = P.slot_draws[s]; thr_off = P.slot_thr_off[s]; thr_n = P.slot_thr_n[s]; }
    }
    err = __shfl_sync(kFull, err, 0);
    if (err) {
        if (lane == 0) atomicOr(&P.counters[0], err);
        return;
    }

    for (int sw = 0; sw < p.nsweeps; ++sw) {
        for (int pass = 0; pass < NP; ++pass) {
            const int plane = NP == 1 ? 0 : flavour;
            int8_t* A = sp + plane * N;
            const int8_t* B = NP == 1 ? A : sp + (plane ^ 1) * N;
            const uint64_t A0 = ((sweeps0 + (uint64_t)sw) * (uint64_t)NP + (uint64_t)pass) * (uint64_t)N;
            for (int c0 = 0; c0 < N; c0 += C) {
                {
                    // bring the lines of g within kTableReach bins of the walker's bin into L1
                    // (the chunk's proposals mostly fall there), one line per lane per 512 bins
                    const int bcur = __shfl_sync(kFull, c.b, 0);
                    for (int k = lane * 16 - kTableReach; k <= kTableReach; k += 32 * 16) {
                        const int bb = bcur + k;
                        if ((unsigned)bb < (unsigned)nb) asm volatile("prefetch.global.L1 [%0];" ::"l"(gg + bb));
                    }
                }
                int ai = 0, sg[NM];
                for (int m = 0; m < NM; ++m) sg[m] = 0;
                if (lane < C) {
                    const int i = c0 + lane;
                    ai = A[i];
                    Model::flip_signs(ai, B[i], plane, sg);
                    const long long d0 = Model::delta_energy(A, B, i, L, cpl, hf ? hf[i] : 0);
                    const long long d1 = lane > 0 ? Model::left_flipped(A, B, i, L, cpl, d0) : d0;
                    st->du[lane] = make_longlong2(d0 * mul, d1 * mul);
                    if (wraps && lane == C - 1) st->wcu = Model::right_flipped(A, B, i, L, cpl) * mul;
                    if (!REPLAY) {
                        const uint32_t word = philox_word(seed, uid, A0 + (uint64_t)i, kStreamWL);
                        st->T[lane] = accept_threshold(neglog_u32(word));
                    }
                }
                __syncwarp();
                if (lane == 0) {
                    c.acc = 0;
                    c.vn = c.v + st->du[0].x;
                    c.bn = (int)(c.vn >> sh);
                    c.inr = (unsigned)c.bn < (unsigned)nb;
                    c.G0 = c.G1 = gg[min((unsigned)c.bn, (unsigned)(nb - 1))];
                    c.ap = false;
                    if (!REPLAY) c.T = st->T[0];
                    if (C == 1) {
                        table_step<REPLAY, OBS, false, false, false>(c, 0, st, gg, nb, sh, lnf, P, thr_off, thr_n);
                    } else {
                        c.q = st->du[1];
#pragma unroll 4
                        for (int j = 0; j < C - 2; ++j)
                            table_step<REPLAY, OBS, true, true, false>(c, j, st, gg, nb, sh, lnf, P, thr_off, thr_n);
                        if (wraps) table_step<REPLAY, OBS, true, false, true>(c, C - 2, st, gg, nb, sh, lnf, P, thr_off, thr_n);
                        else table_step<REPLAY, OBS, true, false, false>(c, C - 2, st, gg, nb, sh, lnf, P, thr_off, thr_n);
                        table_step<REPLAY, OBS, false, false, false>(c, C - 1, st, gg, nb, sh, lnf, P, thr_off, thr_n);
                    }
                }
                const unsigned acc = __shfl_sync(kFull, c.acc, 0);
                // per magnetisation: the steps whose accepted flip lowers it (its term was +1)
                // and raises it; the change after step j is -2 (lowered - raised) up to j
                unsigned plus[NM], minus[NM];
                for (int m = 0; m < NM; ++m) {
                    plus[m] = __ballot_sync(kFull, lane < C && sg[m] > 0);
                    minus[m] = __ballot_sync(kFull, lane < C && sg[m] < 0);
                }
                auto dm = [&](int m, int j) {
                    const unsigned le = j >= 31 ? 0xFFFFFFFFu : ((2u << j) - 1u);
                    return -2 * ((int)__popc(acc & plus[m] & le) - (int)__popc(acc & minus[m] & le));
                };
                if (OBS) {
                    int32_t M0[3] = {0, 0, 0};
                    for (int m = 0; m < NM; ++m) M0[m] = __shfl_sync(kFull, M[m], 0);
                    __syncwarp();
                    if (lane < C) {
                        int32_t Mv[3] = {0, 0, 0};
                        for (int m = 0; m < NM; ++m) Mv[m] = M0[m] + dm(m, lane);
                        Model::add_observables(P.obs + (size_t)(P.slot_tab[s] + st->seq[lane]) * P.obs_stride, Mv, invN,
                                               P.corr);
                    }
                    if (corr) {
                        const int y = c0 / L, x0 = c0 - y * L, row = y * L;
                        const int bin = lane < C ? st->seq[lane] : -1 - lane;
                        const unsigned grp = __match_any_sync(kFull, bin);
                        if (lane < C) {
                            // the bin's count before step `lane`: its visits at the launch's start
                            // plus the change of g over ln f, less the chunk's visits from this step on
                            const unsigned long long after =
                                P.visits[P.slot_tab[s] + bin] + (unsigned long long)((gg[bin] - g0[bin]) / lnf);
                            const unsigned long long seen = after - (unsigned long long)__popc(grp >> lane);
                            if (seen % kCountsPerTransform == 0) {
                                const double* q = P.qtab + I.qtab_off;
                                double G[NC];
                                for (int cp = 0; cp < NC; ++cp) {
                                    const int m = Model::corr_mag(cp);
                                    // a correlator plane changes where its magnetisation's terms do
                                    G[cp] = plane_corr(sums + 2 * L * cp, sums + 2 * L * cp + L, q, L, y, dm(m, lane), x0, lane,
                                                       acc & (plus[m] | minus[m]),
                                                       [&](int k) { return Model::corr_site(sp, N, row + x0 + k, cp); });
                                }
                                Model::add_transforms(P.obs + (size_t)(P.slot_tab[s] + bin) * P.obs_stride, G, invN * invN);
                            }
                        }
                        __syncwarp();
                        // the chunk's flips into the sums
                        for (int cp = 0; cp < NC; ++cp) {
                            const int m = Model::corr_mag(cp);
                            if (lane < C && ((acc >> lane) & 1u)) sums[2 * L * cp + L + x0 + lane] -= 2 * sg[m];
                            if (lane == 0) sums[2 * L * cp + y] += dm(m, 31);
                        }
                    }
                }
                if (lane < C && ((acc >> lane) & 1u)) A[c0 + lane] = (int8_t)(-ai);
                if (lane == 0)
                    for (int m = 0; m < NM; ++m) M[m] += dm(m, 31);
                __syncwarp();
            }
            if (NP == 2) flavour ^= 1;
        }
    }
    for (int i = lane; i < NP * N; i += 32) gl[i] = sp[i];
    // counts and visits from the logDoS change (lane 0's stores to g are ordered
    // before the other lanes' loads by the barrier)
    __syncwarp();
    uint32_t* gH = P.H + P.slot_tab[s];
    uint64_t* gv = P.visits + P.slot_tab[s];
    for (int k = lane; k < nb; k += 32) {
        const long long gnew = gg[k], dg = gnew - g0[k];
        if (dg != 0) {
            const int e = commit_visits(gH, gv, k, dg / lnf, gnew);
            if (e) atomicOr(&P.counters[0], e);
        }
    }
    if (lane == 0) {
        P.cfg_E[cfg] = eglo + (c.v + vlo) / mul;
        for (int m = 0; m < NM; ++m) P.cfg_M[3 * cfg + m] = M[m];
        P.slot_sweeps[s] = sweeps0 + (uint64_t)p.nsweeps;
        if (NP == 2) P.slot_flavour[s] = flavour;
        if (REPLAY) P.slot_draws[s] = c.draws;
        if (c.err) atomicOr(&P.counters[0], c.err);
    }
}

template <class Model, bool REPLAY, bool OBS>
__global__ void __launch_bounds__(256, 2) k_sweep_tables(const SweepParams p)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int wib = threadIdx.x >> 5;
    sweep_tables_warp<Model, REPLAY, OBS>(p, blockIdx.x * (blockDim.x >> 5) + wib, smem + (size_t)wib * p.smem_per_warp);
}

// --------------------------------------------------------------------------
// One persistent, work-stealing launch for every launch group of a batch
// (rewl_batch_desc.persistent): a grid sized to the resident capacity, each warp
// taking the next walker from a device counter until all walkers of the sweep phase
// are done.  A task is one walker (one walker per warp); tasks are ordered by
// expected cost, the Ashkin-Teller walkers and the largest lattices first.  Each
// kind of group runs its own kernel's per-warp function, not inlined here, so the
// fused kernel's registers are those of its dispatch loop plus the largest callee.
// --------------------------------------------------------------------------
enum FusedKind : int {
    kFusedBins32 = 0, kFusedBins24 = 1, kFusedBins16 = 2, kFusedBins8 = 3, kFusedBins4 = 4,
    kFusedTablesIsing = 5, kFusedTablesAT = 6
};
constexpr int kMaxFusedGroups = 16;

struct FusedGroup {
    const int32_t* slots;
    int nslots, smem_per_warp, nbcap, kind, first_task, pad;
};

struct FusedParams {
    DevPtrs P;
    int nsweeps, ngroups, ntasks, slot_bytes;
    unsigned int* counter;
    FusedGroup g[kMaxFusedGroups];
};

template <int C, bool OBS>
__device__ __noinline__ void fused_bins(const SweepParams& p, int unit, unsigned char* base)
{
    sweep_bins_warp<1, C, OBS, false>(p, unit, base);
}

template <class Model, bool OBS>
__device__ __noinline__ void fused_tables(const SweepParams& p, int unit, unsigned char* base)
{
    sweep_tables_warp<Model, false, OBS>(p, unit, base);
}

template <bool OBS>
__global__ void __launch_bounds__(128) k_sweep_fused(const FusedParams fp)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    unsigned char* base = smem + (size_t)wib * fp.slot_bytes;
    for (;;) {
        int t = 0;
        if (lane == 0) t = (int)atomicAdd(fp.counter, 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= fp.ntasks) break;
        int gi = 0;
        while (gi + 1 < fp.ngroups && t >= fp.g[gi + 1].first_task) ++gi;
        const FusedGroup& G = fp.g[gi];
        SweepParams sp;
        sp.P = fp.P; sp.slots = G.slots; sp.nslots = G.nslots; sp.nsweeps = fp.nsweeps;
        sp.smem_per_warp = G.smem_per_warp; sp.nbcap = G.nbcap;
        const int unit = t - G.first_task;
        switch (G.kind) {
        case kFusedBins32: fused_bins<32, OBS>(sp, unit, base); break;
        case kFusedBins24: fused_bins<24, OBS>(sp, unit, base); break;
        case kFusedBins16: fused_bins<16, OBS>(sp, unit, base); break;
        case kFusedBins8: fused_bins<8, OBS>(sp, unit, base); break;
        case kFusedBins4: fused_bins<4, OBS>(sp, unit, base); break;
        case kFusedTablesIsing: fused_tables<Ising2dModel, OBS>(sp, unit, base); break;
        default: fused_tables<AshkinTeller2dModel, OBS>(sp, unit, base); break;
        }
        __syncwarp();
    }
}

// --------------------------------------------------------------------------
// Replica exchange: one thread per (instance, lower window) pair of the round
// --------------------------------------------------------------------------
__device__ inline int64_t slot_local_bin(const DevPtrs& P, const InstDev& I, int slot, int64_t E)
{
    const WinDev& W = P.win[P.slot_win[slot]];
    return global_bin(I, E) - W.gblo;
}

__device__ inline void touch(const DevPtrs& P, const InstDev& I, int slot)
{
    const int c = P.slot_cfg[slot];
    const int64_t b = slot_local_bin(P, I, slot, P.cfg_E[c]);
    const int w = P.slot_win[slot];
    if (b < 0 || b >= P.slot_nb[slot]) { atomicOr(&P.counters[0], ERR_BOUNDS); return; }
    const int64_t o = P.slot_tab[slot] + b;
    const long long gnew = P.g[o] + P.win_lnf[w];
    P.g[o] = gnew;
    if (P.H[o] == 0xFFFFFFFFu) atomicOr(&P.counters[0], ERR_COUNT);   // saturated, as in commit_visits
    else P.H[o] += 1u;
    if (gnew >= kLogdosLimit) atomicOr(&P.counters[0], ERR_RANGE);
    const uint64_t seen = P.visits[o];         // the bin's count before this visit
    P.visits[o] = seen + 1u;
    if (P.obs) {
        double* ob = P.obs + (size_t)o * P.obs_stride;
        const double invN = 1.0 / (double)I.N;
        const int32_t* Mc = P.cfg_M + 3 * c;
        const bool due = P.corr && seen % kCountsPerTransform == 0;
        const double* q = P.qtab + I.qtab_off;
        const int8_t* sp = P.spins + P.cfg_off[c];
        if (I.model == REWL_MODEL_ISING2D) {
            Ising2dModel::add_observables(ob, Mc, invN, P.corr);
            if (due) Ising2dModel::add_correlators(ob, sp, I.N, I.L, q, invN * invN);
        } else {
            AshkinTeller2dModel::add_observables(ob, Mc, invN, P.corr);
            if (due) AshkinTeller2dModel::add_correlators(ob, sp, I.N, I.L, q, invN * invN);
        }
    }
}

__device__ void exchange_pair(const DevPtrs& P, const int32_t* pairs, int k, uint64_t round)
{
    const int ii = pairs[2 * k], lw = pairs[2 * k + 1];
    const InstDev I = P.inst[ii];
    const int R = I.R;
    int perm[kMaxReplicas];
    for (int r = 0; r < R; ++r) perm[r] = r;
    // keyed by the instance's own seed only, like its sweeps: an instance's trajectory does not
    // depend on the other instances of the batch or on its position among them
    const uint32_t xuid = 0x80000000u;
    const uint32_t w3 = (uint32_t)((round << 8) ^ (uint64_t)lw);
    for (int i = R - 1; i >= 1; --i) {
        const uint32_t word = philox_word(I.seed, xuid, (uint64_t)(R - 1 - i), kStreamExchange, w3);
        const int j = (int)mulhi32(word, (uint32_t)(i + 1));
        const int t = perm[i]; perm[i] = perm[j]; perm[j] = t;
    }
    unsigned long long att = 0, accn = 0;
    for (int r = 0; r < R; ++r) {
        const int lo = I.first_slot + lw * R + r;
        const int hi = I.first_slot + (lw + 1) * R + perm[r];
        const int cl = P.slot_cfg[lo], ch = P.slot_cfg[hi];
        const int64_t El = P.cfg_E[cl], Eh = P.cfg_E[ch];
        const int64_t bl_l = slot_local_bin(P, I, lo, El), bl_h = slot_local_bin(P, I, lo, Eh);
        const int64_t bh_l = slot_local_bin(P, I, hi, El), bh_h = slot_local_bin(P, I, hi, Eh);
        ++att;
        bool accept = false;
        if (bl_l < 0 || bl_l >= P.slot_nb[lo] || bh_h < 0 || bh_h >= P.slot_nb[hi]) {
            atomicOr(&P.counters[0], ERR_BOUNDS);    // a walker outside its own window: skip the pair
            continue;
        }
        if (bl_h >= 0 && bl_h < P.slot_nb[lo] && bh_l >= 0 && bh_l < P.slot_nb[hi]) {
            const int64_t* gl = P.g + P.slot_tab[lo];
            const int64_t* gh = P.g + P.slot_tab[hi];
            const int64_t a = gl[bl_h] - gl[bl_l];
            const int64_t c = gh[bh_l] - gh[bh_h];
            const int64_t d = (a > 0 ? a : 0) + (c > 0 ? c : 0);
            // acceptance words follow the R - 1 pairing words: counter 32 + r while R <= 32, 64 + r above
            const uint32_t word = philox_word(I.seed, xuid, (uint64_t)((R <= 32 ? 32 : 64) + r), kStreamExchange, w3);
            accept = d < accept_threshold(neglog_u32(word));
        }
        if (accept) { P.slot_cfg[lo] = ch; P.slot_cfg[hi] = cl; ++accn; }
        touch(P, I, lo);
        touch(P, I, hi);
    }
    atomicAdd(&P.stats[0], att);
    atomicAdd(&P.stats[1], accn);
}

// One exchange round: one thread per (instance, lower window) pair of the round's direction.
// The round counter lives on the device (so that a captured cycle replays correctly): every
// thread reads it first, and the last block to finish advances it.
__global__ void k_exchange(DevPtrs P, const int32_t* pairs0, int n0, const int32_t* pairs1, int n1)
{
    __shared__ bool last;
    const uint64_t round = *(volatile unsigned long long*)P.xround;
    const int dir = (int)(round & 1u);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    // after a device error no pair moves; the round still advances with the host's mirror
    if (k < (dir ? n1 : n0) && !engine_failed(P.counters)) exchange_pair(P, dir ? pairs1 : pairs0, k, round);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&P.xround[1], 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        P.xround[1] = 0;
        P.xround[0] = round + 1;
    }
}

// --------------------------------------------------------------------------
// Flatness, averaging, reset, ln f: one block per window
// --------------------------------------------------------------------------
struct FlatParams {
    DevPtrs P;
    int nwin_total;
    int flat_mode;
    int mask_mode;
    int one_over_t;
    int reduce;
    uint64_t flat_num, flat_den;   // min * n * den >= num * sum
    float flat_param_f;
    double lnf_final;
    uint64_t sweeps_since_check;
};

struct OpMin { __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a < b ? a : b; } };
struct OpMax { __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a > b ? a : b; } };
struct OpAdd { __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a + b; } };

template <typename T, typename Op>
__device__ T block_reduce(T v, Op op, T* sh, T identity)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_down_sync(kFull, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (wid == 0) {
        v = lane < nw ? sh[lane] : identity;
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_down_sync(kFull, v, o));
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    const T r = sh[0];
    __syncthreads();
    return r;
}

__device__ inline bool bin_valid(const DevPtrs& P, const WinDev& W, int first_slot_of_win, int R, int b, int mask_mode)
{
    if (!P.mask[W.mask_off + b]) return false;
    if (mask_mode == REWL_MASK_VISITED) {
        for (int r = 0; r < R; ++r)
            if (P.visits[P.slot_tab[first_slot_of_win + r] + b]) return true;
        return false;
    }
    return true;
}

__global__ void __launch_bounds__(256) k_flat(const FlatParams fp)
{
    __shared__ unsigned long long red_u[32];
    __shared__ int flat_sh, stop_sh;
    __shared__ long long g0_sh[kMaxReplicas];
    const DevPtrs& P = fp.P;
    const int w = blockIdx.x;
    const WinDev W = P.win[w];
    const InstDev I = P.inst[W.inst];
    const int R = I.R;
    const int first = I.first_slot + W.local * R;
    const int nb = W.nb;

    if (threadIdx.x == 0) {
        stop_sh = engine_failed(P.counters);
        if (!stop_sh) P.win_sweepctr[w] += fp.sweeps_since_check;
        flat_sh = 1;
    }
    __syncthreads();
    if (stop_sh) return;

    for (int r = 0; r < R; ++r) {
        const uint32_t* H = P.H + P.slot_tab[first + r];
        const int64_t* g = P.g + P.slot_tab[first + r];
        unsigned long long mn = ~0ull, mx = 0, sum = 0, n = 0, zero = 0, big = 0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            // a window that never goes flat (a replica trapped away from part of its
            // range) lets ln g grow without bound: report it before int64 overflows
            big |= (unsigned long long)(g[b] >= kLogdosLimit || g[b] <= -kLogdosLimit);
            if (!bin_valid(P, W, first, R, b, fp.mask_mode)) continue;
            const unsigned long long h = H[b];
            mn = h < mn ? h : mn; mx = h > mx ? h : mx; sum += h; ++n; zero += (h == 0);
        }
        mn = block_reduce(mn, OpMin(), red_u, ~0ull);
        mx = block_reduce(mx, OpMax(), red_u, 0ull);
        sum = block_reduce(sum, OpAdd(), red_u, 0ull);
        n = block_reduce(n, OpAdd(), red_u, 0ull);
        zero = block_reduce(zero, OpAdd(), red_u, 0ull);
        big = block_reduce(big, OpMax(), red_u, 0ull);
        if (threadIdx.x == 0) {
            if (big) { atomicOr(&P.counters[0], ERR_RANGE); flat_sh = 0; }   // no averaging or reset
            bool f;
            if (fp.flat_mode == REWL_FLAT_ALL_VISITED) f = P.win_oot[w] ? true : (zero == 0);
            else if (n == 0 || mn == 0) f = false;
            else if (fp.flat_mode == REWL_FLAT_MAX_MIN_RATIO)
                f = __fdiv_rn(__ull2float_rn(mx - mn), __ull2float_rn(mn)) <= fp.flat_param_f;
            else
                f = (unsigned __int128)mn * n * fp.flat_den >= (unsigned __int128)fp.flat_num * sum;
            if (!f) flat_sh = 0;
        }
        __syncthreads();
    }
    if (!flat_sh) return;

    // count-weighted average of the replicas' logDoS (rewl_simulation.hpp:361-454)
    if (R > 1) {
        const double inv = 1.0 / kLogdosScale;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            unsigned long long tot = 0;
            for (int r = 0; r < R; ++r) tot += P.H[P.slot_tab[first + r] + b];
            long long avg;
            if (tot == 0) avg = P.g[P.slot_tab[first] + b];
            else {
                double acc = 0.0;
                const double dtot = __ull2double_rn(tot);
                for (int r = 0; r < R; ++r) {
                    const int64_t o = P.slot_tab[first + r] + b;
                    const double wt = __ddiv_rn(__uint2double_rn(P.H[o]), dtot);
                    const double gr = __dmul_rn(__ll2double_rn(P.g[o]), inv);
                    acc = __dadd_rn(acc, __dmul_rn(wt, gr));
                }
                avg = __double2ll_rn(__dmul_rn(acc, kLogdosScale));
            }
            for (int r = 0; r < R; ++r) P.g[P.slot_tab[first + r] + b] = avg;
        }
        __syncthreads();
    }
    if (threadIdx.x < R) g0_sh[threadIdx.x] = P.g[P.slot_tab[first + threadIdx.x]];
    __syncthreads();
    for (int r = 0; r < R; ++r) {
        const int64_t o = P.slot_tab[first + r];
        const long long red = fp.reduce ? g0_sh[r] : 0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) { P.H[o + b] = 0; P.g[o + b] -= red; }
    }
    if (threadIdx.x == 0) {
        const uint64_t t = P.win_sweepctr[w] * P.win_iter[w];
        long long lnf = P.win_lnf[w];
        int oot = P.win_oot[w];
        if (fp.one_over_t && !oot && t > 0 && __ll2double_rn(lnf) <= __ddiv_rn(kLogdosScale, __ull2double_rn(t))) oot = 1;
        if (oot && t > 0) lnf = (long long)((((unsigned long long)1 << kLogdosBits) + t / 2) / t);
        else lnf = lnf >> 1;
        if (lnf < 1) lnf = 1;                  // the 2^-36 grid's smallest increment
        P.win_lnf[w] = lnf;
        P.win_oot[w] = oot;
        P.win_done[w] = (__ll2double_rn(lnf) / kLogdosScale) < fp.lnf_final ? 1 : 0;
        P.win_iter[w] += 1;
        P.win_sweepctr[w] = 0;
        atomicAdd(&P.counters[1], 1);
    }
}

__global__ void k_reset_window(DevPtrs P, int w, int reduce)
{
    const WinDev W = P.win[w];
    const InstDev I = P.inst[W.inst];
    const int first = I.first_slot + W.local * I.R;
    for (int r = 0; r < I.R; ++r) {
        const int64_t o = P.slot_tab[first + r];
        const long long g0 = P.g[o];
        __syncthreads();
        for (int b = threadIdx.x; b < W.nb; b += blockDim.x) { P.H[o + b] = 0; if (reduce) P.g[o + b] -= g0; }
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// Host side
// --------------------------------------------------------------------------
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        n = count;
        if (count == 0) return REWL_OK;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return fail(REWL_ENOMEM, "cudaMalloc of %zu bytes failed", count * sizeof(T));
        return REWL_OK;
    }
    void free_()
    {
        if (p) cudaFree(p);
        p = nullptr; n = 0;
    }
};

struct HostInst {
    rewl_instance_desc d;
    InstDev dev;
    std::vector<double> fields;     // quantised
    double bw;
    std::vector<WinDev> wins;
    std::vector<double> wmin, wmax;
};

struct Launch {
    int model;
    std::vector<int32_t> slots;
    int smem_per_warp = 0;  // per walker for the bin-tracking kernel, per warp otherwise
    int nbcap = 0;
    int wpb = 1;            // warps per block
    int bins = 0;           // Ising bin-tracking kernel with `walkers_per_warp` walkers per warp and chunk `chunk`
    int walkers_per_warp = 1;
    int chunk = 32;
    int tables = 0;         // the global-table kernel (k_sweep_tables)
    int carveout = -1;      // global-table kernel: shared-memory carveout (percent) that leaves the rest to L1
    DBuf<int32_t> d_slots;
};

using SweepKernel = void (*)(const SweepParams);

template <class Model>
SweepKernel table_kernel_t(bool replay, bool obs)
{
    if (replay) return obs ? k_sweep_tables<Model, true, true> : k_sweep_tables<Model, true, false>;
    return obs ? k_sweep_tables<Model, false, true> : k_sweep_tables<Model, false, false>;
}

SweepKernel table_kernel(int model, bool replay, bool obs)
{
    return model == REWL_MODEL_ISING2D ? table_kernel_t<Ising2dModel>(replay, obs)
                                       : table_kernel_t<AshkinTeller2dModel>(replay, obs);
}

} // namespace

struct rewl_engine {
    rewl_batch_desc desc;
    std::vector<HostInst> inst;
    int nslots = 0, nwin_total = 0;
    std::vector<int32_t> h_slot_inst, h_slot_win, h_slot_nb;
    std::vector<int64_t> h_slot_tab;
    std::vector<int64_t> h_cfg_off;
    std::vector<WinDev> h_wins;
    int64_t table_total = 0, spin_total = 0, mask_total = 0;
    std::vector<int32_t> pairs_dir[2];
    int direction = 0;
    uint64_t exch_round = 0;
    uint64_t sweeps_since_check = 0;
    int64_t sweeps_total = 0, cycles = 0, flat_events = 0, flips_total = 0;
    int64_t flips_per_sweep = 0;
    // sweep launches are split so that one launch adds at most kLaunchGrowth to a bin: an upper
    // bound of every window's ln f (2^-36 units; k_flat only lowers it, except the 1/t rule,
    // which never exceeds 1) and the largest number of degrees of freedom of a walker
    int64_t lnf_bound_u = 0, ndof_max = 0;
    // rewl_batch_desc.persistent: every launch group in one work-stealing launch (k_sweep_fused)
    bool fused = false;
    FusedParams fused_p{};
    int fused_grid = 0, fused_block = 128;
    size_t fused_smem = 0;
    DBuf<unsigned int> fused_counter;
    cudaStream_t stream = nullptr;
    std::vector<Launch> launches;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    // one check interval captured as a CUDA graph (rewl_batch_desc.graphs): the host counters it
    // advances per replay, and the timing events recorded inside it
    cudaGraphExec_t cycle_exec = nullptr;
    bool capturing = false;
    int64_t g_sweeps = 0, g_flips = 0, g_launches = 0, g_kernel_launches = 0, g_rounds = 0;
    std::vector<cudaEvent_t> g_events;
    double graph_sweep_ms = 0;          // sweep-phase time of replayed graphs since the last timing read
    bool tuned = false;
    int64_t kernel_launches = 0;        // sweep-kernel launches since the last timing read
    int64_t launches_total = 0;         // every engine kernel since creation
    int sweep_variant = 3;              // REWL_SWEEP_VARIANT: 3 all-lane Ising resolver (default), 2 lane-0, 4 global tables
    int bins_lean = -1;                 // REWL_BINS_LEAN: 1 / 0 forces the lean bin-tracking chain on / off (-1: by occupancy)

    DBuf<InstDev> d_inst;
    DBuf<WinDev> d_win;
    DBuf<int32_t> slot_inst, slot_win, slot_cfg, slot_nb, slot_flavour, pairs[2];
    DBuf<int64_t> slot_tab, slot_draws, slot_thr_off, slot_thr_n, cfg_off, cfg_E, fields, g, win_lnf;
    DBuf<uint64_t> slot_sweeps, visits, win_iter, win_sweepctr;
    DBuf<int8_t> spins;
    DBuf<int32_t> cfg_M, win_done, win_oot, counters;
    DBuf<uint32_t> H;
    DBuf<uint8_t> mask;
    DBuf<unsigned long long> stats;
    DBuf<int64_t> thr;
    DBuf<double> obs;           // per-bin observable sums (observables on)
    DBuf<int64_t> gsnap;        // Ashkin-Teller engines: logDoS copy taken by each sweep launch
    DBuf<double> qtab;          // correlator kernels (observables == 2)
    DBuf<unsigned long long> xround;   // exchange round and the exchange kernel's done-block count
    std::vector<cudaStream_t> gstreams; // one per launch group when there are several (they run concurrently)
    cudaEvent_t fork_ev = nullptr;
    std::vector<cudaEvent_t> join_ev;
    int obs_stride = 0;
    std::vector<int64_t> h_thr_off, h_thr_n;
    std::vector<int64_t> h_fields;
    std::vector<uint8_t> h_mask;
    std::vector<double> h_qtab;

    DevPtrs ptrs() const
    {
        DevPtrs P;
        P.inst = d_inst.p; P.win = d_win.p;
        P.slot_inst = slot_inst.p; P.slot_win = slot_win.p; P.slot_cfg = slot_cfg.p; P.slot_tab = slot_tab.p;
        P.slot_nb = slot_nb.p; P.slot_flavour = slot_flavour.p; P.slot_sweeps = slot_sweeps.p;
        P.slot_draws = slot_draws.p; P.slot_thr_off = slot_thr_off.p; P.slot_thr_n = slot_thr_n.p; P.thr = thr.p;
        P.cfg_off = cfg_off.p; P.spins = spins.p; P.cfg_E = cfg_E.p; P.cfg_M = cfg_M.p; P.fields = fields.p;
        P.g = g.p; P.gsnap = gsnap.p; P.H = H.p; P.visits = visits.p; P.mask = mask.p;
        P.win_lnf = win_lnf.p; P.win_done = win_done.p; P.win_oot = win_oot.p; P.win_iter = win_iter.p;
        P.win_sweepctr = win_sweepctr.p; P.pairs = nullptr; P.counters = counters.p; P.stats = stats.p;
        P.xround = xround.p;
        P.obs = obs.p; P.obs_stride = obs_stride;
        P.corr = desc.observables == 2 ? 1 : 0; P.qtab = qtab.p;
        return P;
    }

    void drop_graph()
    {
        if (cycle_exec) cudaGraphExecDestroy(cycle_exec);
        cycle_exec = nullptr;
        for (auto ev : g_events) cudaEventDestroy(ev);
        g_events.clear();
    }

    void release()
    {
        d_inst.free_(); d_win.free_();
        slot_inst.free_(); slot_win.free_(); slot_cfg.free_(); slot_nb.free_(); slot_flavour.free_();
        pairs[0].free_(); pairs[1].free_();
        obs.free_(); gsnap.free_(); qtab.free_(); xround.free_(); fused_counter.free_();
        for (cudaStream_t st : gstreams) cudaStreamDestroy(st);
        gstreams.clear();
        for (cudaEvent_t ev : join_ev) cudaEventDestroy(ev);
        join_ev.clear();
        if (fork_ev) { cudaEventDestroy(fork_ev); fork_ev = nullptr; }
        slot_tab.free_(); slot_draws.free_(); slot_thr_off.free_(); slot_thr_n.free_(); cfg_off.free_();
        cfg_E.free_(); fields.free_(); g.free_(); win_lnf.free_(); slot_sweeps.free_(); visits.free_();
        win_iter.free_(); win_sweepctr.free_(); spins.free_(); cfg_M.free_(); win_done.free_(); win_oot.free_();
        counters.free_(); H.free_(); mask.free_(); stats.free_(); thr.free_();
        for (auto& l : launches) l.d_slots.free_();
        for (auto e : ev_pool) cudaEventDestroy(e);
        ev_pool.clear();
        drop_graph();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

namespace {

bool is_pow2_multiple(double v, int escale, int& shift)
{
    const double u = std::ldexp(v, escale);
    if (u < 1.0 || u != std::floor(u)) return false;
    const long long x = (long long)u;
    if (x & (x - 1)) return false;
    shift = 0;
    while ((1LL << shift) < x) ++shift;
    return true;
}

int largest_chunk(int L)
{
    for (int c = std::min(L, 32); c >= 1; --c)
        if (L % c == 0) return c;
    return 1;
}

// glazier::construct_windows, EQUAL_WINDOWS branch (src/REWL/glazier.hpp:305-351),
// carried out in units of bins: window k starts at the previous window's start
// plus the whole bins up to its nominal start, and spans the whole bins that
// cover its nominal width, clipped to the global range.  For integer widths
// this is the reference's arithmetic exactly; for fractional widths it avoids
// the bin the reference's double ceil/clip can lose.
int make_windows(const rewl_instance_desc& d, std::vector<double>& mins, std::vector<double>& maxs,
                 std::vector<int64_t>& gblo, std::vector<int>& nbins)
{
    const int nw = d.num_windows;
    const double gmin = d.energy_min, gmax = d.energy_max, bw = d.bin_width, ov = d.window_overlap;
    mins.assign(nw, 0); maxs.assign(nw, 0); gblo.assign(nw, 0); nbins.assign(nw, 0);
    const double span = (gmax - gmin) / bw;
    const int64_t G = (int64_t)std::llround(span);
    if (std::fabs(span - (double)G) > 1e-6 * std::max(1.0, span) || G < 1) return -1;
    const double denom = 1 + (nw - 1) * (1 - ov);
    const double size = (gmax - gmin) / denom;
    const double eps = 1e-9;
    for (int k = 0; k < nw; ++k) {
        const double raw_min = gmin + (double)k * (1 - ov) * size;
        const double raw_max = raw_min + size;
        int64_t lo = 0;
        if (k != 0) lo = gblo[k - 1] + (int64_t)std::floor((raw_min - mins[k - 1]) / bw + eps);
        const double wmin = gmin + bw * (double)lo;
        int64_t hi = lo + (int64_t)std::ceil((raw_max - wmin) / bw - eps);
        if (hi > G) hi = G;
        gblo[k] = lo;
        nbins[k] = (int)(hi - lo);
        mins[k] = wmin;
        maxs[k] = gmin + bw * (double)hi;
    }
    return 0;
}

void static_mask(const rewl_instance_desc& d, double wmin, int nb, uint8_t* m)
{
    for (int b = 0; b < nb; ++b) m[b] = 1;
    if (d.model != REWL_MODEL_ISING2D) return;
    // Ising on an L x L torus: E = -2N + 4 and E = 2N - 4 never occur; all
    // energies are -2N + 4k (with J = 1; scaled by |J| in general).
    const double N = (double)d.L * d.L, J = std::fabs(d.J);
    for (int b = 0; b < nb; ++b) {
        const double lo = wmin + d.bin_width * b, hi = lo + d.bin_width;
        bool any = false;
        for (double e = std::ceil((lo + 2 * N * J) / (4 * J)) * 4 * J - 2 * N * J; e < hi; e += 4 * J) {
            if (e < -2 * N * J || e > 2 * N * J) continue;
            if (e == -2 * N * J + 4 * J || e == 2 * N * J - 4 * J) continue;
            any = true;
        }
        m[b] = any ? 1 : 0;
    }
}

template <typename T>
int upload(DBuf<T>& b, const std::vector<T>& v, cudaStream_t s)
{
    int rc = b.alloc(v.size());
    if (rc) return rc;
    if (!v.empty()) CUDA_TRY(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return REWL_OK;
}

int build_host(rewl_engine* e)
{
    const rewl_batch_desc& D = e->desc;
    if (D.num_instances < 1 || !D.instances) return fail(REWL_EINVAL, "no instances");
    if (D.sweeps_per_exchange < 1 || D.sweeps_per_check < D.sweeps_per_exchange || D.sweeps_per_check % D.sweeps_per_exchange)
        return fail(REWL_EINVAL, "sweeps_per_check must be a positive multiple of sweeps_per_exchange");
    if (!(D.lnf_initial > 0) || !(D.lnf_final > 0) || D.lnf_initial > 64)
        return fail(REWL_EINVAL, "ln f must be positive and the initial ln f at most 64");
    if (D.flatness_mode < 0 || D.flatness_mode > 2) return fail(REWL_EINVAL, "bad flatness mode");
    if (D.mask_mode < 0 || D.mask_mode > 1) return fail(REWL_EINVAL, "bad mask mode");
    if (D.rng_mode != REWL_RNG_PHILOX && D.rng_mode != REWL_RNG_REPLAY) return fail(REWL_EINVAL, "bad rng mode");
    if (D.warps_per_block != 0 && D.warps_per_block != 1 && D.warps_per_block != 2 && D.warps_per_block != 4 && D.warps_per_block != 8)
        return fail(REWL_EINVAL, "warps_per_block must be 0, 1, 2, 4 or 8");
    if (D.observables < 0 || D.observables > 2)
        return fail(REWL_EINVAL, "observables must be 0 (off), 1 (moments) or 2 (moments and G(q_min) correlators)");
    if (D.walkers_per_warp != 0 && D.walkers_per_warp != 1 && D.walkers_per_warp != 2 && D.walkers_per_warp != 4)
        return fail(REWL_EINVAL, "walkers_per_warp must be 0, 1, 2 or 4");
    if (D.persistent != 0 && D.persistent != 1) return fail(REWL_EINVAL, "persistent must be 0 or 1");
    if (D.persistent && D.rng_mode == REWL_RNG_REPLAY)
        return fail(REWL_EINVAL, "the persistent launch runs Philox streams only (rng_mode REWL_RNG_PHILOX)");
    if (D.persistent && D.walkers_per_warp > 1)
        return fail(REWL_EINVAL, "the persistent launch runs one walker per warp");
    int slot = 0, win = 0;
    int64_t tab = 0, spin = 0, maskoff = 0, fieldoff = 0;
    std::vector<int64_t> h_fields;
    std::vector<uint8_t> h_mask;
    std::vector<double> h_qtab;
    e->inst.resize(D.num_instances);
    for (int ii = 0; ii < D.num_instances; ++ii) {
        const rewl_instance_desc& d = D.instances[ii];
        HostInst& H = e->inst[ii];
        H.d = d;
        if (d.model != REWL_MODEL_ISING2D && d.model != REWL_MODEL_ASHKIN_TELLER2D) return fail(REWL_EINVAL, "instance %d: bad model", ii);
        if (d.L < 2 || d.L > 128) return fail(REWL_EINVAL, "instance %d: L must be in [2, 128]", ii);
        if (d.num_windows < 1 || d.replicas_per_window < 1 || d.replicas_per_window > kMaxReplicas)
            return fail(REWL_EINVAL, "instance %d: need >= 1 window and 1..%d replicas", ii, kMaxReplicas);
        if (!(d.window_overlap >= 0 && d.window_overlap < 1)) return fail(REWL_EINVAL, "instance %d: overlap must be in [0,1)", ii);
        if (!(d.energy_max > d.energy_min) || !(d.bin_width > 0)) return fail(REWL_EINVAL, "instance %d: bad energy range", ii);
        if (d.init_mode != 0 && d.init_mode != 1) return fail(REWL_EINVAL, "instance %d: bad init mode", ii);
        InstDev I{};
        I.model = d.model; I.L = d.L; I.N = d.L * d.L; I.ndof = d.model == REWL_MODEL_ISING2D ? I.N : 2 * I.N;
        I.nwin = d.num_windows; I.R = d.replicas_per_window; I.first_win = win; I.first_slot = slot;
        I.seed = instance_key(d.seed); I.chunk = largest_chunk(d.L); I.init_mode = d.init_mode;
        int shift = 0;
        if (d.model == REWL_MODEL_ISING2D) {
            if (d.J != std::floor(d.J) || d.J == 0 || std::fabs(d.J) > 1024) return fail(REWL_EINVAL, "instance %d: Ising J must be a non-zero integer", ii);
            if (d.fields) return fail(REWL_EINVAL, "instance %d: random fields are supported for the Ashkin-Teller model only", ii);
            I.escale = 0; I.J_u = (int64_t)d.J; I.K_u = 0;
            if (!is_pow2_multiple(d.bin_width, 0, shift)) return fail(REWL_EINVAL, "instance %d: Ising bin width must be a power of two >= 1", ii);
            I.bin_mul = 1; I.bin_shift = shift;
            if (d.energy_min != std::floor(d.energy_min)) return fail(REWL_EINVAL, "instance %d: energy_min must be an integer", ii);
            if (std::fabs(d.energy_min) + std::fabs(d.energy_max) > 1e8) return fail(REWL_EINVAL, "instance %d: energy range too large", ii);
        } else {
            I.escale = 20;
            const double Ju = std::ldexp(d.J, 20), Ku = std::ldexp(d.K, 20);
            if (Ju != std::floor(Ju) || Ku != std::floor(Ku)) return fail(REWL_EINVAL, "instance %d: J and K must be multiples of 2^-20", ii);
            I.J_u = (int64_t)Ju; I.K_u = (int64_t)Ku;
            const double inv = 1.0 / d.bin_width;
            if (is_pow2_multiple(d.bin_width, 20, shift)) { I.bin_mul = 1; I.bin_shift = shift; }
            else if (std::fabs(inv - std::nearbyint(inv)) < 1e-9 * inv && inv <= 4096) { I.bin_mul = (int64_t)std::llround(inv); I.bin_shift = 20; }
            else return fail(REWL_EINVAL, "instance %d: Ashkin-Teller bin width must be 1/n or a power of two", ii);
            const double emu = std::ldexp(d.energy_min, 20);
            if (emu != std::floor(emu)) return fail(REWL_EINVAL, "instance %d: energy_min must be a multiple of 2^-20", ii);
        }
        I.eglo_u = (int64_t)std::llround(std::ldexp(d.energy_min, I.escale));
        if (d.fields) {
            I.field_off = fieldoff;
            H.fields.resize(I.N);
            for (int i = 0; i < I.N; ++i) {
                const double q = std::nearbyint(std::ldexp(d.fields[i], 20));
                if (!std::isfinite(q) || std::fabs(q) > 1e15) return fail(REWL_EINVAL, "instance %d: bad field value", ii);
                H.fields[i] = std::ldexp(q, -20);
                h_fields.push_back((int64_t)q);
            }
            fieldoff += I.N;
        } else I.field_off = -1;
        if (D.observables == 2) {
            // Transform_Kernel (src/Hamiltonians/Correlations/fourier_correlator.hpp:14-42), from the
            // host's libm like the reference's own table
            I.qtab_off = (int64_t)h_qtab.size();
            const double qmin = 2. * std::acos(-1.) / static_cast<double>(d.L);
            for (int x = 0; x < d.L; ++x) h_qtab.push_back(std::cos(qmin * static_cast<double>(x)));
            for (int x = 0; x < d.L; ++x) h_qtab.push_back(std::sin(qmin * static_cast<double>(x)));
        } else I.qtab_off = -1;
        std::vector<double> mins, maxs; std::vector<int64_t> gblo; std::vector<int> nbins;
        if (make_windows(d, mins, maxs, gblo, nbins))
            return fail(REWL_EINVAL, "instance %d: the energy range is not a whole number of bins", ii);
        for (int k = 0; k < d.num_windows; ++k) {
            if (nbins[k] < 1) return fail(REWL_EINVAL, "instance %d: window %d is empty", ii, k);
            if (k > 0 && gblo[k] >= gblo[k - 1] + nbins[k - 1]) return fail(REWL_EINVAL, "instance %d: windows %d and %d do not overlap", ii, k - 1, k);
        }
        H.bw = d.bin_width;
        H.wmin = mins; H.wmax = maxs;
        for (int k = 0; k < d.num_windows; ++k) {
            WinDev W{};
            W.inst = ii; W.local = k; W.nb = nbins[k]; W.gblo = gblo[k]; W.mask_off = maskoff;
            W.elo_u = I.eglo_u + (I.bin_mul == 1 ? (gblo[k] << I.bin_shift) : 0);
            std::vector<uint8_t> m(nbins[k]);
            static_mask(d, mins[k], nbins[k], m.data());
            h_mask.insert(h_mask.end(), m.begin(), m.end());
            maskoff += nbins[k];
            H.wins.push_back(W);
            e->h_wins.push_back(W);
            for (int r = 0; r < d.replicas_per_window; ++r) {
                e->h_slot_inst.push_back(ii);
                e->h_slot_win.push_back(win + k);
                e->h_slot_nb.push_back(nbins[k]);
                e->h_slot_tab.push_back(tab);
                tab += nbins[k];
                e->h_cfg_off.push_back(spin);
                spin += I.ndof;
            }
        }
        if (d.model == REWL_MODEL_ISING2D) {
            // integer arithmetic in int32 inside the kernel
            const double emax_abs = 2.0 * I.N * std::fabs(d.J);
            if (emax_abs > 1e9 || std::fabs(d.energy_min) > 1e9 || std::fabs(d.energy_max) > 1e9)
                return fail(REWL_EINVAL, "instance %d: energies exceed int32", ii);
        }
        H.dev = I;
        slot += d.num_windows * d.replicas_per_window;
        win += d.num_windows;
        e->flips_per_sweep += (int64_t)d.num_windows * d.replicas_per_window * I.ndof;
        e->ndof_max = std::max<int64_t>(e->ndof_max, I.ndof);
    }
    e->lnf_bound_u = std::max<int64_t>(std::max<int64_t>(1, (int64_t)std::llround(D.lnf_initial * kLogdosScale)),
                                       D.one_over_t ? (int64_t)kLogdosScale : 0);
    e->nslots = slot; e->nwin_total = win;
    e->table_total = tab; e->spin_total = spin; e->mask_total = maskoff;
    // exchange pair lists
    for (int dir = 0; dir < 2; ++dir) {
        e->pairs_dir[dir].clear();
        for (int ii = 0; ii < D.num_instances; ++ii)
            for (int lw = dir; lw + 1 < D.instances[ii].num_windows; lw += 2) { e->pairs_dir[dir].push_back(ii); e->pairs_dir[dir].push_back(lw); }
    }
    e->h_fields = std::move(h_fields);
    e->h_qtab = std::move(h_qtab);
    e->h_mask = std::move(h_mask);
    return REWL_OK;
}

int upload_all(rewl_engine* e)
{
    const rewl_batch_desc& D = e->desc;
    const int slot = e->nslots, win = e->nwin_total;
    const int64_t tab = e->table_total, spin = e->spin_total;
    cudaStream_t s = e->stream;
    std::vector<InstDev> hinst;
    for (auto& H : e->inst) hinst.push_back(H.dev);
    int rc;
    if ((rc = upload(e->d_inst, hinst, s)) || (rc = upload(e->d_win, e->h_wins, s)) ||
        (rc = upload(e->slot_inst, e->h_slot_inst, s)) || (rc = upload(e->slot_win, e->h_slot_win, s)) ||
        (rc = upload(e->slot_nb, e->h_slot_nb, s)) || (rc = upload(e->slot_tab, e->h_slot_tab, s)) ||
        (rc = upload(e->cfg_off, e->h_cfg_off, s)) || (rc = upload(e->fields, e->h_fields, s)) ||
        (rc = upload(e->qtab, e->h_qtab, s)) ||
        (rc = upload(e->mask, e->h_mask, s)) || (rc = upload(e->pairs[0], e->pairs_dir[0], s)) ||
        (rc = upload(e->pairs[1], e->pairs_dir[1], s)))
        return rc;
    std::vector<int32_t> cfg(slot);
    for (int i = 0; i < slot; ++i) cfg[i] = i;
    if ((rc = upload(e->slot_cfg, cfg, s))) return rc;
    if ((rc = e->slot_flavour.alloc(slot)) || (rc = e->slot_sweeps.alloc(slot)) || (rc = e->slot_draws.alloc(slot)) ||
        (rc = e->slot_thr_off.alloc(slot)) || (rc = e->slot_thr_n.alloc(slot)) || (rc = e->cfg_E.alloc(slot)) ||
        (rc = e->cfg_M.alloc(3 * (size_t)slot)) || (rc = e->spins.alloc(spin)) || (rc = e->g.alloc(tab)) ||
        (rc = e->H.alloc(tab)) || (rc = e->visits.alloc(tab)) || (rc = e->win_lnf.alloc(win)) ||
        (rc = e->win_done.alloc(win)) || (rc = e->win_oot.alloc(win)) || (rc = e->win_iter.alloc(win)) ||
        (rc = e->win_sweepctr.alloc(win)) || (rc = e->counters.alloc(4)) || (rc = e->stats.alloc(2)) ||
        (rc = e->xround.alloc(2)))
        return rc;
    CUDA_TRY(cudaMemsetAsync(e->slot_sweeps.p, 0, slot * sizeof(uint64_t), s));
    CUDA_TRY(cudaMemsetAsync(e->slot_draws.p, 0, slot * sizeof(int64_t), s));
    CUDA_TRY(cudaMemsetAsync(e->slot_thr_off.p, 0, slot * sizeof(int64_t), s));
    CUDA_TRY(cudaMemsetAsync(e->slot_thr_n.p, 0, slot * sizeof(int64_t), s));
    if (tab) {
        CUDA_TRY(cudaMemsetAsync(e->g.p, 0, tab * sizeof(int64_t), s));
        CUDA_TRY(cudaMemsetAsync(e->H.p, 0, tab * sizeof(uint32_t), s));
        CUDA_TRY(cudaMemsetAsync(e->visits.p, 0, tab * sizeof(uint64_t), s));
    }
    bool any_at = false;
    for (const auto& hi : e->inst) any_at = any_at || hi.d.model == REWL_MODEL_ASHKIN_TELLER2D;
    if (any_at && tab && (rc = e->gsnap.alloc(tab))) return rc;
    if (D.observables && tab) {
        e->obs_stride = any_at ? (D.observables == 2 ? 16 : 12) : (D.observables == 2 ? 4 : 3);
        if ((rc = e->obs.alloc((size_t)tab * e->obs_stride))) return rc;
        CUDA_TRY(cudaMemsetAsync(e->obs.p, 0, (size_t)tab * e->obs_stride * sizeof(double), s));
    }
    std::vector<int64_t> lnf(win, std::max<int64_t>(1, (int64_t)std::llround(D.lnf_initial * kLogdosScale)));
    CUDA_TRY(cudaMemcpyAsync(e->win_lnf.p, lnf.data(), win * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemsetAsync(e->win_done.p, 0, win * sizeof(int32_t), s));
    CUDA_TRY(cudaMemsetAsync(e->win_oot.p, 0, win * sizeof(int32_t), s));
    std::vector<uint64_t> ones(win, 1);
    CUDA_TRY(cudaMemcpyAsync(e->win_iter.p, ones.data(), win * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemsetAsync(e->win_sweepctr.p, 0, win * sizeof(uint64_t), s));
    CUDA_TRY(cudaMemsetAsync(e->counters.p, 0, 4 * sizeof(int32_t), s));
    CUDA_TRY(cudaMemsetAsync(e->stats.p, 0, 2 * sizeof(unsigned long long), s));
    CUDA_TRY(cudaMemsetAsync(e->xround.p, 0, 2 * sizeof(unsigned long long), s));
    return REWL_OK;
}

bool bins_eligible(const InstDev& I, const rewl_batch_desc& D, int max_window_bins)
{
    if (I.model != REWL_MODEL_ISING2D || D.rng_mode != REWL_RNG_PHILOX) return false;
    // the window table, with its guard bins, and the lattice live in shared memory (with the
    // correlators also the bin counts and the row and column sums)
    const size_t need = (size_t)(max_window_bins + 2 + 2 * kGuard) * 8 + I.N + 4096 +
                        (D.observables == 2 ? (size_t)4 * (max_window_bins + 2) + 8 * I.L : 0);
    if (need > 200 * 1024) return false;
    const int C = I.chunk;
    if (!(C == 32 || C == 24 || C == 16 || C == 8 || C == 4)) return false;
    const long long step = 4 * std::llabs(I.J_u);            // every energy change is a multiple of 4|J|
    if (step % (1LL << I.bin_shift) != 0) return false;
    // the thresholds are drawn four sites per Philox block, 4C sites at a time
    if (I.N % (4 * C) != 0) return false;
    // a proposal lands at most 8|J| / width bins away, and a prefetch issued from an
    // out-of-window proposal twice that: the guard bins cover both
    const long long maxbins = (8 * std::llabs(I.J_u)) >> I.bin_shift;
    if (2 * maxbins > kGuard) return false;
    return true;
}

// Streaming multiprocessors of the engine's device (152 on a GB300).
int sm_count(const rewl_engine* e)
{
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, e->desc.device) != cudaSuccess || n < 1) n = 152;
    return n;
}

// The logDoS tables of the Ashkin-Teller kernel live in global memory and are read through L1,
// so its shared-memory carveout is the smallest that still holds the blocks resident on an SM
// (the CUDA runtime's default split leaves L1 far less).
int at_carveout(rewl_engine* e, Launch& l)
{
    if (!l.tables) return REWL_OK;
    const int nsm = sm_count(e);
    const SweepKernel fn = table_kernel(l.model, e->desc.rng_mode == REWL_RNG_REPLAY, e->desc.observables != 0);
    const int threads = 32 * l.wpb;
    const size_t smem = (size_t)l.wpb * l.smem_per_warp;
    int occ = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem));
    const int blocks = ((int)l.slots.size() + l.wpb - 1) / l.wpb;
    const int per_sm = std::max(1, std::min(occ, (blocks + nsm - 1) / nsm));
    int smem_sm = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, e->desc.device));
    const size_t need = (size_t)per_sm * (smem + 1024);
    l.carveout = (int)std::min<size_t>(100, (need * 100 + smem_sm - 1) / (size_t)smem_sm);
    return REWL_OK;
}

// A launch group's shape: walkers per warp (bin-tracking kernel) and warps per block, if the
// block's shared memory fits.
bool shape_fits(const Launch& l, int G, int wpb)
{
    return (size_t)wpb * (l.bins ? G : 1) * l.smem_per_warp <= 200 * 1024;
}

// The persistent launch: every group's walkers as tasks of one work-stealing kernel.  Groups are
// ordered by the expected cost of one walker's sweep (degrees of freedom x cycles per flip of
// its kernel, measured: table kernel ~440, bin-tracking ~70), the dearest first, so that the
// last tasks taken are short.  Every warp gets the largest shared-memory region any group needs.
int plan_fused(rewl_engine* e, int nsm)
{
    if (e->launches.size() > (size_t)kMaxFusedGroups)
        return fail(REWL_EINVAL, "the persistent launch takes at most %d launch groups (%zu here)", kMaxFusedGroups,
                    e->launches.size());
    std::vector<std::pair<double, size_t>> order;
    for (size_t gi = 0; gi < e->launches.size(); ++gi) {
        const Launch& l = e->launches[gi];
        int ndof = 0;
        for (int s : l.slots) ndof = std::max(ndof, e->inst[e->h_slot_inst[s]].dev.ndof);
        order.push_back({-(double)ndof * (l.bins ? 70.0 : 440.0), gi});
    }
    std::stable_sort(order.begin(), order.end());
    FusedParams& F = e->fused_p;
    F = FusedParams{};
    int task = 0, slot = 16;
    for (size_t k = 0; k < order.size(); ++k) {
        const Launch& l = e->launches[order[k].second];
        FusedGroup& G = F.g[k];
        G.slots = l.d_slots.p; G.nslots = (int)l.slots.size(); G.smem_per_warp = l.smem_per_warp; G.nbcap = l.nbcap;
        if (l.bins)
            G.kind = l.chunk == 32 ? kFusedBins32 : l.chunk == 24 ? kFusedBins24 : l.chunk == 16 ? kFusedBins16
                   : l.chunk == 8 ? kFusedBins8 : kFusedBins4;
        else if (l.tables)
            G.kind = l.model == REWL_MODEL_ISING2D ? kFusedTablesIsing : kFusedTablesAT;
        else
            return fail(REWL_EINVAL, "internal: a launch group without a persistent form");
        G.first_task = task;
        task += G.nslots;
        slot = std::max(slot, l.smem_per_warp);
    }
    F.ngroups = (int)order.size();
    F.ntasks = task;
    F.slot_bytes = (slot + 15) & ~15;
    int warps = 4;
    while (warps > 1 && (size_t)warps * F.slot_bytes > 200 * 1024) warps >>= 1;
    if ((size_t)F.slot_bytes > 220 * 1024) return fail(REWL_EINVAL, "a walker needs %d bytes of shared memory", F.slot_bytes);
    e->fused_block = 32 * warps;
    e->fused_smem = (size_t)warps * F.slot_bytes;
    CUDA_TRY(cudaFuncSetAttribute(k_sweep_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    CUDA_TRY(cudaFuncSetAttribute(k_sweep_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    int per_sm = 0;
    if (e->desc.observables)
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_fused<true>, e->fused_block, e->fused_smem));
    else
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_fused<false>, e->fused_block, e->fused_smem));
    const int need = (task + warps - 1) / warps;
    e->fused_grid = std::max(1, std::min(need, std::max(1, per_sm) * nsm));
    if (int rc = e->fused_counter.alloc(1)) return rc;
    e->fused = true;
    return REWL_OK;
}

int plan_launches(rewl_engine* e)
{
    const int nsm = sm_count(e);
    // group walkers by (model, bin-tracking kernel, chunk, sites) so each launch has one
    // kernel shape and the walkers sharing a warp run the same number of chunks
    struct Key { int model, bins, chunk, sites; };
    std::vector<Key> keys;
    std::vector<Launch> plans;
    for (int s = 0; s < e->nslots; ++s) {
        const HostInst& H = e->inst[e->h_slot_inst[s]];
        int max_nb = 0;
        for (const auto& wd : H.wins) max_nb = std::max(max_nb, wd.nb);
        const int bins = bins_eligible(H.dev, e->desc, max_nb) && getenv("REWL_SWEEP_VARIANT") == nullptr ? 1 : 0;
        Key k{H.d.model, bins, bins ? H.dev.chunk : 0, bins ? H.dev.N : 0};
        size_t idx = 0;
        for (; idx < keys.size(); ++idx)
            if (keys[idx].model == k.model && keys[idx].bins == k.bins && keys[idx].chunk == k.chunk &&
                keys[idx].sites == k.sites)
                break;
        if (idx == keys.size()) {
            keys.push_back(k);
            Launch l;
            l.model = k.model; l.bins = k.bins; l.chunk = k.chunk ? k.chunk : 32;
            plans.push_back(std::move(l));
        }
        plans[idx].slots.push_back(s);
    }
    for (auto& l : plans) {
        int maxN = 0, maxnb = 0, maxL = 0;
        const bool corr = e->desc.observables == 2;
        for (int s : l.slots) {
            maxN = std::max(maxN, e->inst[e->h_slot_inst[s]].dev.N);
            maxL = std::max(maxL, e->inst[e->h_slot_inst[s]].dev.L);
            maxnb = std::max(maxnb, e->h_slot_nb[s]);
        }
        const int n = (int)l.slots.size();
        if (l.bins) {
            int G = e->desc.persistent ? 1 : e->desc.walkers_per_warp;
            if (G == 0) {
                // one walker per warp while the SM sub-partitions outnumber the walkers
                // (the chain is latency-bound); two per warp beyond that (measured at L = 64: two
                // per warp beat four from 2048 to 4096 walkers, 3.77e10 against 3.43e10 flips/s at
                // 3072); four only for still larger batches
                G = n <= 4 * nsm ? 1 : (n <= 32 * nsm ? 2 : 4);
            }
            l.walkers_per_warp = G;
            l.nbcap = (maxnb + 1) & ~1;
            int raw = (((l.nbcap + 2 * kGuard) * 8 + 15) & ~15) + ((maxN + 15) & ~15) + 8 * l.chunk * 8 + 2 * l.chunk * 8 + l.chunk * 4
                      + (corr ? 8 * maxL + 4 * l.nbcap : 0);
            l.smem_per_warp = ((raw + 127) & ~127) + 16;           // per walker; +16 skews the walkers' banks
            if ((size_t)l.smem_per_warp * G > 220 * 1024) return fail(REWL_EINVAL, "a walker needs %d bytes of shared memory", l.smem_per_warp);
            int wpb = e->desc.warps_per_block;
            if (wpb == 0) {
                const int warps = (n + G - 1) / G;
                wpb = warps <= nsm * 2 ? 1 : warps <= nsm * 8 ? 2 : 4;
            }
            wpb = std::min(wpb, 4);                                // the kernel's launch bounds: 128 threads
            while (wpb > 1 && (size_t)wpb * G * l.smem_per_warp > 200 * 1024) wpb >>= 1;
            l.wpb = wpb;
        } else {
            const size_t ising_smem = (size_t)(((maxnb + 1) & ~1) * 8 + sizeof(Stage) + ((maxN + 15) & ~15) + (corr ? 8 * maxL : 0));
            // Ising windows live in shared memory unless they do not fit there (or the
            // global-table kernel is asked for)
            l.tables = l.model != REWL_MODEL_ISING2D || e->sweep_variant == 4 || ising_smem > 200 * 1024 ||
                       e->desc.persistent;             // the persistent launch has the global-table form only
            if (!l.tables) {
                l.nbcap = (maxnb + 1) & ~1;
                l.smem_per_warp = (int)ising_smem;
            } else {
                const int planes = l.model == REWL_MODEL_ISING2D ? 1 : 2;
                l.nbcap = 0;
                l.smem_per_warp = (int)(sizeof(TableStage) + ((planes * maxN + 15) & ~15) + (corr ? 8 * planes * maxL : 0));
            }
        }
        if (!l.bins) {
            l.smem_per_warp = (l.smem_per_warp + 15) & ~15;
            int wpb = e->desc.warps_per_block;
            if (wpb == 0) wpb = n <= nsm * 2 ? 1 : n <= nsm * 8 ? 2 : 4;
            while (wpb > 1 && (size_t)wpb * l.smem_per_warp > 200 * 1024) wpb >>= 1;
            if ((size_t)l.smem_per_warp > 220 * 1024) return fail(REWL_EINVAL, "a walker needs %d bytes of shared memory (limit 220 KiB)", l.smem_per_warp);
            l.wpb = wpb;
        }
        int rc = upload(l.d_slots, l.slots, e->stream);
        if (rc) return rc;
        e->launches.push_back(std::move(l));
    }
    CUDA_TRY(cudaFuncSetAttribute(k_sweep_ising<false, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    CUDA_TRY(cudaFuncSetAttribute(k_sweep_ising<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    CUDA_TRY(cudaFuncSetAttribute(k_sweep_ising<true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    for (int r = 0; r < 2; ++r)
        for (int o = 0; o < 2; ++o)
            for (int m : {REWL_MODEL_ISING2D, REWL_MODEL_ASHKIN_TELLER2D})
                CUDA_TRY(cudaFuncSetAttribute(table_kernel(m, r, o), cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    for (auto& l : e->launches) {
        if (int rc = at_carveout(e, l)) return rc;
        // the global-table kernel copies each walker's logDoS at the start of a launch
        if (l.tables && !e->gsnap.p && e->table_total > 0)
            if (int rc = e->gsnap.alloc(e->table_total)) return rc;
    }
    CUDA_TRY(allow_bins_smem<1>());
    CUDA_TRY(allow_bins_smem<2>());
    CUDA_TRY(allow_bins_smem<4>());
    if (e->desc.persistent) return plan_fused(e, nsm);
    if (e->launches.size() > 1) {
        CUDA_TRY(cudaEventCreateWithFlags(&e->fork_ev, cudaEventDisableTiming));
        for (size_t gi = 0; gi < e->launches.size(); ++gi) {
            cudaStream_t st;
            cudaEvent_t ev;
            CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            e->gstreams.push_back(st);
            CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            e->join_ev.push_back(ev);
        }
    }
    return REWL_OK;
}

int check_device_error(rewl_engine* e)
{
    int32_t h[4];
    CUDA_TRY(cudaMemcpyAsync(h, e->counters.p, sizeof h, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (h[0] & ERR_BOUNDS) return fail(REWL_EBOUNDS, "a walker's energy left its window (device error word %d)", h[0]);
    if (h[0] & ERR_ADJUST) return fail(REWL_EINVAL, "a walker could not reach its window");
    if (h[0] & ERR_REPLAY_EXHAUSTED) return fail(REWL_EINVAL, "replay uniform stream exhausted");
    if (h[0] & ERR_RANGE)
        return fail(REWL_ESTATE, "a window's logDoS passed 2^62 units (6.7e7 nats) without a flat event: "
                                 "a replica is trapped away from part of its window");
    if (h[0] & ERR_COUNT)
        return fail(REWL_ESTATE, "a per-stage histogram count passed 2^32 - 1 without a flat event");
    return REWL_OK;
}

cudaEvent_t next_event(rewl_engine* e)
{
    if (e->capturing) {                // a timing event owned by the captured graph
        cudaEvent_t ev;
        cudaEventCreate(&ev);
        e->g_events.push_back(ev);
        return ev;
    }
    if (e->ev_used == e->ev_pool.size()) {
        cudaEvent_t ev;
        cudaEventCreate(&ev);
        e->ev_pool.push_back(ev);
    }
    return e->ev_pool[e->ev_used++];
}

// One launch group's sweeps on a stream (its kernel and shape fixed by plan_launches or the
// autotuner).
int launch_group(rewl_engine* e, Launch& l, cudaStream_t stream, int nsweeps, const DevPtrs& P)
{
    const bool replay = e->desc.rng_mode == REWL_RNG_REPLAY;
    SweepParams sp;
    sp.P = P; sp.slots = l.d_slots.p; sp.nslots = (int)l.slots.size(); sp.nsweeps = nsweeps;
    sp.smem_per_warp = l.smem_per_warp; sp.nbcap = l.nbcap;
    if (l.bins) {
        const int G = l.walkers_per_warp;
        const int warps = (sp.nslots + G - 1) / G;
        const int blocks = (warps + l.wpb - 1) / l.wpb;
        const size_t smem = (size_t)l.wpb * G * l.smem_per_warp;
        // the lean chain from 5 warps per SM on (measured at L = 64, two walkers per warp: 2048
        // walkers 3.78e10 against 3.55e10 flips/s, 3072 4.62e10 against 3.78e10; 1024 walkers,
        // 3.4 warps per SM, 2.15e10 against 2.43e10)
        const bool lean = e->bins_lean < 0 ? warps >= 5 * sm_count(e) : e->bins_lean == 1;
        if (G == 1) launch_bins<1>(l.chunk, blocks, 32 * l.wpb, smem, stream, sp, false);
        else if (G == 2) launch_bins<2>(l.chunk, blocks, 32 * l.wpb, smem, stream, sp, lean);
        else launch_bins<4>(l.chunk, blocks, 32 * l.wpb, smem, stream, sp, lean);
    } else {
        const int blocks = (sp.nslots + l.wpb - 1) / l.wpb;
        const size_t smem = (size_t)l.wpb * l.smem_per_warp;
        if (l.tables) {
            const SweepKernel fn = table_kernel(l.model, replay, e->desc.observables != 0);
            if (l.carveout >= 0) CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, l.carveout));
            fn<<<blocks, 32 * l.wpb, smem, stream>>>(sp);
        } else {
            if (replay) k_sweep_ising<true, 2><<<blocks, 32 * l.wpb, smem, stream>>>(sp);
            else if (e->sweep_variant == 2) k_sweep_ising<false, 2><<<blocks, 32 * l.wpb, smem, stream>>>(sp);
            else k_sweep_ising<false, 3><<<blocks, 32 * l.wpb, smem, stream>>>(sp);
        }
    }
    CUDA_TRY(cudaGetLastError());
    e->kernel_launches++;
    e->launches_total++;
    return REWL_OK;
}

// A timing event on the engine stream; inside a stream capture it must become an event node of
// the graph (a plain record there only marks a dependency).
cudaError_t record_timing(rewl_engine* e)
{
    cudaEvent_t ev = next_event(e);
    return e->capturing ? cudaEventRecordWithFlags(ev, e->stream, cudaEventRecordExternal) : cudaEventRecord(ev, e->stream);
}

// Sweeps per launch such that one launch plus one exchange visit add at most kLaunchGrowth to
// any bin: lnf_bound x (sweeps x ndof_max + 1) <= kLaunchGrowth.
int max_launch_sweeps(const rewl_engine* e)
{
    const int64_t visits = kLaunchGrowth / std::max<int64_t>(1, e->lnf_bound_u) - 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>(1 << 20, visits / std::max<int64_t>(1, e->ndof_max)));
}

// Raise the ln f bound (rewl_set_lnf, rewl_restore); a captured check interval split its sweeps
// for the old bound, so it is captured again.
void raise_lnf_bound(rewl_engine* e, int64_t lnf_u)
{
    if (lnf_u <= e->lnf_bound_u) return;
    const int before = max_launch_sweeps(e);
    e->lnf_bound_u = lnf_u;
    if (max_launch_sweeps(e) != before) e->drop_graph();
}

int launch_sweeps_once(rewl_engine* e, int nsweeps);

int launch_sweeps(rewl_engine* e, int nsweeps)
{
    const int most = max_launch_sweeps(e);
    while (nsweeps > 0) {
        const int n = std::min(nsweeps, most);
        if (int rc = launch_sweeps_once(e, n)) return rc;
        nsweeps -= n;
    }
    return REWL_OK;
}

int launch_sweeps_once(rewl_engine* e, int nsweeps)
{
    const DevPtrs P = e->ptrs();
    CUDA_TRY(record_timing(e));
    if (e->fused) {
        FusedParams F = e->fused_p;
        F.P = P;
        F.nsweeps = nsweeps;
        F.counter = e->fused_counter.p;
        CUDA_TRY(cudaMemsetAsync(e->fused_counter.p, 0, sizeof(unsigned int), e->stream));
        if (e->desc.observables) k_sweep_fused<true><<<e->fused_grid, e->fused_block, e->fused_smem, e->stream>>>(F);
        else k_sweep_fused<false><<<e->fused_grid, e->fused_block, e->fused_smem, e->stream>>>(F);
        CUDA_TRY(cudaGetLastError());
        e->kernel_launches++;
        e->launches_total++;
        CUDA_TRY(record_timing(e));
        e->sweeps_total += nsweeps;
        e->sweeps_since_check += nsweeps;
        e->flips_total += (int64_t)nsweeps * e->flips_per_sweep;
        return REWL_OK;
    }
    // several launch groups (models, lattice sizes, kernel shapes) run concurrently, each on
    // its own stream forked from and joined back into the engine stream; they touch disjoint
    // walkers
    const bool fork = e->gstreams.size() == e->launches.size() && e->launches.size() > 1;
    if (fork) CUDA_TRY(cudaEventRecord(e->fork_ev, e->stream));
    for (size_t gi = 0; gi < e->launches.size(); ++gi) {
        const cudaStream_t stream = fork ? e->gstreams[gi] : e->stream;
        if (fork) CUDA_TRY(cudaStreamWaitEvent(stream, e->fork_ev, 0));
        if (int rc = launch_group(e, e->launches[gi], stream, nsweeps, P)) return rc;
        if (fork) {
            CUDA_TRY(cudaEventRecord(e->join_ev[gi], stream));
            CUDA_TRY(cudaStreamWaitEvent(e->stream, e->join_ev[gi], 0));
        }
    }
    CUDA_TRY(record_timing(e));
    e->sweeps_total += nsweeps;
    e->sweeps_since_check += nsweeps;
    e->flips_total += (int64_t)nsweeps * e->flips_per_sweep;
    return REWL_OK;
}

int launch_exchange(rewl_engine* e)
{
    // the kernel reads the round (and from its parity the direction) on the device and
    // advances it; the host keeps a mirror for snapshots
    const int n0 = (int)e->pairs_dir[0].size() / 2, n1 = (int)e->pairs_dir[1].size() / 2;
    const int blocks = std::max(1, (std::max(n0, n1) + 127) / 128);
    k_exchange<<<blocks, 128, 0, e->stream>>>(e->ptrs(), e->pairs[0].p, n0, e->pairs[1].p, n1);
    CUDA_TRY(cudaGetLastError());
    e->launches_total++;
    e->direction ^= 1;
    e->exch_round++;
    return REWL_OK;
}

int launch_flat(rewl_engine* e)
{
    FlatParams fp;
    fp.P = e->ptrs();
    fp.nwin_total = e->nwin_total;
    fp.flat_mode = e->desc.flatness_mode;
    fp.mask_mode = e->desc.mask_mode;
    fp.one_over_t = e->desc.one_over_t;
    fp.reduce = e->desc.reduce_logdos;
    fp.flat_den = 1000000;
    fp.flat_num = (uint64_t)std::llround(e->desc.flatness_param * 1e6);
    fp.flat_param_f = (float)e->desc.flatness_param;
    fp.lnf_final = e->desc.lnf_final;
    fp.sweeps_since_check = e->sweeps_since_check;
    e->sweeps_since_check = 0;
    k_flat<<<e->nwin_total, 256, 0, e->stream>>>(fp);
    CUDA_TRY(cudaGetLastError());
    e->launches_total++;
    return REWL_OK;
}

bool valid_walker(const rewl_engine* e, int w) { return e && w >= 0 && w < e->nslots; }

int window_index(const rewl_engine* e, int ii, int w)
{
    if (!e || ii < 0 || ii >= (int)e->inst.size()) return -1;
    if (w < 0 || w >= e->inst[ii].d.num_windows) return -1;
    return e->inst[ii].dev.first_win + w;
}

// ------------------------------------------------------------------------
// Host restatement of concatenate_tables (multiple overlap) for the logDoS
// (src/util/concatenate_rewl_tables.hpp:167-305) with derivative_of_vector
// (src/util/numerical_derivatives.hpp:47-70) and the concatenation-point
// search (src/util/vector_matching.hpp:38-88).
// ------------------------------------------------------------------------
double derivative(size_t i, const std::vector<double>& f, const std::vector<double>& a)
{
    const size_t n = f.size();
    if (i == 0) return (f[1] - f[0]) / (a[1] - a[0]);
    if (i == n - 1) return (f[i] - f[i - 1]) / (a[i] - a[i - 1]);
    if (i == 1 || i == n - 2) return (f[i + 1] - f[i - 1]) / (2. * (a[i] - a[i - 1]));
    return (-f[i + 2] + 8. * f[i + 1] - 8. * f[i - 1] + f[i - 2]) / (12. * (a[i] - a[i - 1]));
}

// reference_abs: compare derivative differences as the reference's compiled code does.  Its
// find_left_concatenation_indices calls an unqualified abs() on a double in a translation unit
// that includes only <cmath> and <vector>, which resolves to the C library's int abs(int): every
// |difference| is truncated to an integer, so the splice lands on the first overlapping bin unless
// some derivative difference reaches 1.  Without it the true |difference| is minimised.
inline double beta_gap(double d, bool reference_abs)
{
    if (!reference_abs) return std::fabs(d);
    const double t = std::trunc(d);                       // double -> int conversion truncates
    return std::fabs(std::max(-2147483647.0, std::min(2147483647.0, t)));
}

// O (optional): per window, rows of nobs observables; they are averaged in each overlap as the
// reference does (average_two_windows, src/util/concatenate_rewl_tables.hpp:42-49, weighted by
// the number of windows already averaged at the bin) into fo.
int concatenate(const std::vector<std::vector<double>>& E, const std::vector<std::vector<double>>& G,
                std::vector<double>& fe, std::vector<double>& fg, bool reference_abs = false,
                const std::vector<std::vector<double>>* O = nullptr, int nobs = 0, std::vector<double>* fo = nullptr)
{
    fe = E[0]; fg = G[0];
    std::vector<size_t> overlap(fe.size(), 1);
    if (O) *fo = (*O)[0];
    for (size_t w = 1; w < E.size(); ++w) {
        const auto& er = E[w]; const auto& gr = G[w];
        if (er.size() < 2 || fe.size() < 2) return fail(REWL_EINVAL, "window %zu has fewer than 2 valid bins", w);
        long left_start = -1;
        for (long k = (long)fe.size() - 1; k >= 0; --k) if (fe[k] == er[0]) { left_start = k; break; }
        if (left_start < 0) return fail(REWL_EINVAL, "windows %zu and %zu do not overlap", w - 1, w);
        const size_t nleft = fe.size();
        if (nleft - (size_t)left_start > er.size()) return fail(REWL_EINVAL, "window %zu lies inside window %zu", w, w - 1);
        double beta_diff = beta_gap(derivative((size_t)left_start, fg, fe) - derivative(0, gr, er), reference_abs);
        size_t cl = (size_t)left_start;
        for (size_t idx = 1; idx != nleft - (size_t)left_start; ++idx) {
            const double lb = derivative((size_t)left_start + idx, fg, fe), rb = derivative(idx, gr, er);
            const double gap = beta_gap(lb - rb, reference_abs);
            if ((gap + 0.5) < (beta_diff + 0.5)) { beta_diff = gap; cl = (size_t)left_start + idx; }
        }
        double shifter = 0;
        size_t right_idx = 0;
        for (size_t idx = (size_t)left_start; idx != fe.size(); ++idx) {
            right_idx = idx - (size_t)left_start;
            if (O) {
                const double c = (double)overlap[idx];
                for (int k = 0; k < nobs; ++k) {
                    double& v = (*fo)[idx * nobs + k];
                    v = (c * v + 1.0 * (*O)[w][right_idx * nobs + k]) / (double)(overlap[idx] + 1);
                }
            }
            ++overlap[idx];
            if (idx == cl) shifter = fg[idx] - gr[right_idx];
            else if (idx > cl) fg[idx] = gr[right_idx] + shifter;
        }
        for (size_t idx = right_idx + 1; idx < er.size(); ++idx) {
            fe.push_back(er[idx]);
            fg.push_back(gr[idx] + shifter);
            overlap.push_back(1);
            if (O)
                for (int k = 0; k < nobs; ++k) fo->push_back((*O)[w][idx * nobs + k]);
        }
    }
    return REWL_OK;
}

// normalize_logDoS (src/util/array_shift.hpp:15-43) step for step: the shift that makes
// sum_E g(E) = states_per_site^N (halved for a half spectrum).  Its running maximum starts at 0.
double normalisation_shift(const std::vector<double>& g, double states_per_site, double system_size, bool half)
{
    double mx = 0.0;
    for (double v : g) mx = mx > v ? mx : v;
    double sum = 0.0;
    for (double v : g) sum += std::exp(-(mx - v));
    sum = std::log(sum);
    sum += mx;
    return system_size * std::log(states_per_site) - sum - std::log(2.) * (half ? 1.0 : 0.0);
}

} // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char* rewl_last_error_string(void) { return g_last_error.c_str(); }

int rewl_create(const rewl_batch_desc* desc, rewl_engine** out)
{
    if (!desc || !out) return fail(REWL_EINVAL, "null argument");
    *out = nullptr;
    rewl_engine* e = new rewl_engine();
    e->desc = *desc;
    // REWL_SWEEP_VARIANT: 2 the general Ising kernel's lane-0 resolver, 3 its all-lane resolver,
    // 4 the global-table kernel for Ising too (any of them turns the bin-tracking kernel off)
    if (const char* v = std::getenv("REWL_SWEEP_VARIANT")) {
        const int k = std::atoi(v);
        e->sweep_variant = (k == 2 || k == 4) ? k : 3;
    }
    // REWL_BINS_LEAN: 1 / 0 forces the lean chain of the bin-tracking kernel on / off for warps
    // of several walkers (tests; by default it is taken from 5 warps per SM on)
    if (const char* v = std::getenv("REWL_BINS_LEAN")) e->bins_lean = std::atoi(v) == 1 ? 1 : 0;
    int rc = build_host(e);               // descriptor validation and layout: host only
    if (rc) { delete e; return rc; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { delete e; return fail(REWL_EDEVICE, "no CUDA device"); }
    if (desc->device < 0 || desc->device >= ndev) { delete e; return fail(REWL_EINVAL, "device %d out of range", desc->device); }
    if (cudaSetDevice(desc->device) != cudaSuccess || cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete e; return fail(REWL_EDEVICE, "cannot open device %d", desc->device);
    }
    rc = upload_all(e);
    if (!rc) rc = plan_launches(e);
    if (!rc) {
        k_init<<<(e->nslots + 63) / 64, 64, 0, e->stream>>>(e->ptrs(), e->nslots, 0);
        cudaError_t ce = cudaGetLastError();
        if (ce != cudaSuccess) rc = fail(REWL_EDEVICE, "k_init launch: %s", cudaGetErrorString(ce));
    }
    if (!rc) rc = check_device_error(e);
    if (rc) { e->release(); delete e; return rc; }
    *out = e;
    return REWL_OK;
}

int rewl_destroy(rewl_engine* e)
{
    if (!e) return REWL_OK;
    cudaSetDevice(e->desc.device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->release();
    delete e;
    return REWL_OK;
}

int rewl_num_walkers(const rewl_engine* e, int32_t* n)
{
    if (!e || !n) return fail(REWL_EINVAL, "null argument");
    *n = e->nslots;
    return REWL_OK;
}

int rewl_walker_info(const rewl_engine* e, int32_t w, int32_t* inst, int32_t* win, int32_t* rep)
{
    if (!valid_walker(e, w)) return fail(REWL_EINVAL, "walker %d out of range", w);
    const int ii = e->h_slot_inst[w];
    const WinDev& W = e->h_wins[e->h_slot_win[w]];
    if (inst) *inst = ii;
    if (win) *win = W.local;
    if (rep) *rep = (w - e->inst[ii].dev.first_slot) % e->inst[ii].dev.R;
    return REWL_OK;
}

int rewl_window_info(const rewl_engine* e, int32_t ii, int32_t w, double* emin, double* emax, int32_t* nb)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0) return fail(REWL_EINVAL, "window (%d, %d) out of range", ii, w);
    if (emin) *emin = e->inst[ii].wmin[w];
    if (emax) *emax = e->inst[ii].wmax[w];
    if (nb) *nb = e->h_wins[wi].nb;
    return REWL_OK;
}

int rewl_import_dofs(rewl_engine* e, int32_t w, const int8_t* dofs, int32_t flavour)
{
    if (!valid_walker(e, w) || !dofs) return fail(REWL_EINVAL, "bad walker or null dofs");
    if (flavour != 0 && flavour != 1) return fail(REWL_EINVAL, "flavour must be 0 or 1");
    const int ii = e->h_slot_inst[w];
    const InstDev& I = e->inst[ii].dev;
    for (int i = 0; i < I.ndof; ++i)
        if (dofs[i] != 1 && dofs[i] != -1) return fail(REWL_EINVAL, "spins must be +1 or -1");
    cudaSetDevice(e->desc.device);
    int32_t cfg;
    CUDA_TRY(cudaMemcpyAsync(&cfg, e->slot_cfg.p + w, sizeof cfg, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    CUDA_TRY(cudaMemcpyAsync(e->spins.p + e->h_cfg_off[cfg], dofs, I.ndof, cudaMemcpyHostToDevice, e->stream));
    CUDA_TRY(cudaMemcpyAsync(e->slot_flavour.p + w, &flavour, sizeof flavour, cudaMemcpyHostToDevice, e->stream));
    int32_t* tmp = nullptr;
    CUDA_TRY(cudaMalloc(&tmp, 2 * sizeof(int32_t)));
    int32_t hv[2] = {cfg, ii};
    CUDA_TRY(cudaMemcpyAsync(tmp, hv, sizeof hv, cudaMemcpyHostToDevice, e->stream));
    k_recalc<<<1, 32, 0, e->stream>>>(e->ptrs(), tmp, tmp + 1, 1);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    cudaFree(tmp);
    // the energy must be inside the walker's window
    int64_t E;
    CUDA_TRY(cudaMemcpy(&E, e->cfg_E.p + cfg, sizeof E, cudaMemcpyDeviceToHost));
    const WinDev& W = e->h_wins[e->h_slot_win[w]];
    const int64_t gb = (((E - I.eglo_u) * I.bin_mul) >> I.bin_shift) - W.gblo;
    if (gb < 0 || gb >= W.nb) return fail(REWL_EINVAL, "imported configuration has energy outside the walker's window");
    return REWL_OK;
}

// Random fields drawn as the reference's Disorder::generate_random_field does
// (src/Hamiltonians/Disorder/random_fields.hpp:41-75), from the given seed instead of the
// clock.  One std::mt19937_64 stream read through std::uniform_real_distribution<double>(0, 1)
// (random_number_generator, src/util/random_number_generators.hpp:14-31); for every site 20
// values are drawn and discarded, then one is kept.  Uniform: 2 h (2u - 1).  Gaussian
// (get_gaussian, :33-57): Box-Muller on (u, v), both redrawn while u <= DBL_EPSILON; a third
// uniform keeps the cosine value when below 1/2, else the sine value, combined as the
// reference combines them (z0 * c + z1 * !c) so that the doubles agree bit for bit.
int rewl_generate_fields(uint64_t seed, double strength, int32_t distribution, int64_t num_sites, double* out)
{
    if (num_sites < 0 || (num_sites > 0 && !out)) return fail(REWL_EINVAL, "num_sites must be >= 0 and out non-null");
    if (distribution != REWL_DISORDER_UNIFORM && distribution != REWL_DISORDER_GAUSSIAN)
        return fail(REWL_EINVAL, "distribution must be REWL_DISORDER_UNIFORM or REWL_DISORDER_GAUSSIAN");
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<double> unit(0.0, 1.0);
    const double two_pi = 2.0 * std::acos(-1.0);
    auto draw = [&]() -> double {
        if (distribution == REWL_DISORDER_UNIFORM) return 2.0 * strength * (-1.0 + 2.0 * unit(gen));
        double u = unit(gen), v = unit(gen);
        while (u <= std::numeric_limits<double>::epsilon()) {
            u = unit(gen);
            v = unit(gen);
        }
        const double r = strength * std::sqrt(-2.0 * std::log(u));
        const double z0 = r * std::cos(two_pi * v) + 0.0;
        const double z1 = r * std::sin(two_pi * v) + 0.0;
        const bool c = unit(gen) < 0.5;
        return z0 * c + z1 * !c;
    };
    constexpr int kDiscarded = 20;
    for (int64_t i = 0; i < num_sites; ++i) {
        for (int k = 0; k < kDiscarded; ++k) (void)draw();
        out[i] = draw();
    }
    return REWL_OK;
}

int rewl_import_disorder(rewl_engine* e, int32_t ii, const double* fields)
{
    if (!e || ii < 0 || ii >= (int)e->inst.size() || !fields) return fail(REWL_EINVAL, "bad instance or null fields");
    HostInst& H = e->inst[ii];
    if (H.dev.model != REWL_MODEL_ASHKIN_TELLER2D || H.dev.field_off < 0)
        return fail(REWL_EINVAL, "instance %d was created without fields", ii);
    std::vector<int64_t> q(H.dev.N);
    for (int i = 0; i < H.dev.N; ++i) {
        const double v = std::nearbyint(std::ldexp(fields[i], 20));
        if (!std::isfinite(v)) return fail(REWL_EINVAL, "bad field value");
        q[i] = (int64_t)v; H.fields[i] = std::ldexp(v, -20);
    }
    cudaSetDevice(e->desc.device);
    CUDA_TRY(cudaMemcpyAsync(e->fields.p + H.dev.field_off, q.data(), q.size() * 8, cudaMemcpyHostToDevice, e->stream));
    const int n = H.dev.nwin * H.dev.R;
    std::vector<int32_t> cfgs(n), insts(n, ii);
    CUDA_TRY(cudaMemcpyAsync(cfgs.data(), e->slot_cfg.p + H.dev.first_slot, n * 4, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    int32_t* tmp = nullptr;
    CUDA_TRY(cudaMalloc(&tmp, 2 * n * sizeof(int32_t)));
    CUDA_TRY(cudaMemcpyAsync(tmp, cfgs.data(), n * 4, cudaMemcpyHostToDevice, e->stream));
    CUDA_TRY(cudaMemcpyAsync(tmp + n, insts.data(), n * 4, cudaMemcpyHostToDevice, e->stream));
    k_recalc<<<(n + 63) / 64, 64, 0, e->stream>>>(e->ptrs(), tmp, tmp + n, n);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    cudaFree(tmp);
    return REWL_OK;
}

int rewl_set_logdos(rewl_engine* e, int32_t ii, int32_t w, const double* logdos)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0 || !logdos) return fail(REWL_EINVAL, "bad window or null logdos");
    const int nb = e->h_wins[wi].nb;
    std::vector<int64_t> q(nb);
    for (int b = 0; b < nb; ++b) {
        // a quarter of the 2^62-unit ceiling (1.68e7 nats): room for a first stage to follow
        if (!std::isfinite(logdos[b]) || std::fabs(logdos[b]) > kSetLogdosMax) return fail(REWL_EINVAL, "logdos values must be finite and |g| <= 2^60 units (1.68e7 nats)");
        q[b] = (int64_t)std::nearbyint(logdos[b] * kLogdosScale);
    }
    cudaSetDevice(e->desc.device);
    const InstDev& I = e->inst[ii].dev;
    for (int r = 0; r < I.R; ++r) {
        const int s = I.first_slot + w * I.R + r;
        CUDA_TRY(cudaMemcpyAsync(e->g.p + e->h_slot_tab[s], q.data(), nb * 8, cudaMemcpyHostToDevice, e->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    return REWL_OK;
}

int rewl_set_lnf(rewl_engine* e, int32_t ii, int32_t w, double lnf)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0 || !(lnf > 0) || lnf > 64) return fail(REWL_EINVAL, "bad window or ln f");
    const int64_t q = std::max<int64_t>(1, (int64_t)std::llround(lnf * kLogdosScale));
    cudaSetDevice(e->desc.device);
    raise_lnf_bound(e, q);
    CUDA_TRY(cudaMemcpyAsync(e->win_lnf.p + wi, &q, 8, cudaMemcpyHostToDevice, e->stream));
    const int32_t done = (lnf < e->desc.lnf_final) ? 1 : 0;
    CUDA_TRY(cudaMemcpyAsync(e->win_done.p + wi, &done, 4, cudaMemcpyHostToDevice, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    return REWL_OK;
}

int rewl_set_uniform_stream(rewl_engine* e, int32_t w, const double* u, size_t n)
{
    if (!valid_walker(e, w) || (!u && n)) return fail(REWL_EINVAL, "bad walker or null stream");
    if (e->desc.rng_mode != REWL_RNG_REPLAY) return fail(REWL_ESTATE, "engine was not created in replay mode");
    // accept <=> u < exp(-dg) for the float dg; since exp(-f) falls with f, the
    // accepted floats are those below tau = the smallest float with exp(-tau) <= u
    std::vector<int64_t> T(n);
    for (size_t k = 0; k < n; ++k) {
        const double x = u[k];
        if (!(x >= 0.0 && x < 1.0)) return fail(REWL_EINVAL, "uniform %zu not in [0,1)", k);
        if (x == 0.0) { T[k] = INT64_MAX; continue; }
        float f = (float)(-std::log(x));
        if (!(f > 0)) f = 1e-30f;
        while (f > 0 && !(std::exp(-(double)f) > x)) f = std::nextafter(f, 0.0f);
        while (std::exp(-(double)std::nextafter(f, INFINITY)) > x) f = std::nextafter(f, INFINITY);
        const float tau = std::nextafter(f, INFINITY);
        T[k] = (tau < 1e-30f) ? 1 : accept_threshold(tau);
    }
    cudaSetDevice(e->desc.device);
    // append to the walker-private table (reallocate the pool)
    const size_t old = e->thr.n;
    std::vector<int64_t> all(old + n);
    if (old) CUDA_TRY(cudaMemcpy(all.data(), e->thr.p, old * 8, cudaMemcpyDeviceToHost));
    std::copy(T.begin(), T.end(), all.begin() + old);
    e->thr.free_();
    int rc = e->thr.alloc(all.size());
    if (rc) return rc;
    CUDA_TRY(cudaMemcpy(e->thr.p, all.data(), all.size() * 8, cudaMemcpyHostToDevice));
    const int64_t off = (int64_t)old, cnt = (int64_t)n, zero = 0;
    CUDA_TRY(cudaMemcpy(e->slot_thr_off.p + w, &off, 8, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(e->slot_thr_n.p + w, &cnt, 8, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(e->slot_draws.p + w, &zero, 8, cudaMemcpyHostToDevice));
    return REWL_OK;
}

int rewl_run_sweeps(rewl_engine* e, int64_t n)
{
    if (!e || n < 0) return fail(REWL_EINVAL, "bad arguments");
    cudaSetDevice(e->desc.device);
    while (n > 0) {
        const int chunk = (int)std::min<int64_t>(n, 1 << 20);
        int rc = launch_sweeps(e, chunk);
        if (rc) return rc;
        n -= chunk;
    }
    return check_device_error(e);
}

int rewl_exchange(rewl_engine* e)
{
    if (!e) return fail(REWL_EINVAL, "null engine");
    cudaSetDevice(e->desc.device);
    int rc = launch_exchange(e);
    if (rc) return rc;
    return check_device_error(e);
}

namespace {
// After k_flat: the number of windows that went flat, and the device error word.
int finish_check(rewl_engine* e, int32_t* num_flat)
{
    int32_t h[2];
    CUDA_TRY(cudaMemcpyAsync(h, e->counters.p, sizeof h, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->flat_events += h[1];
    e->cycles++;
    if (num_flat) *num_flat = h[1];
    return check_device_error(e);
}

// Capture one check interval (rounds x (sweeps + exchange), then the flatness step) as a CUDA
// graph.  Nothing runs during capture, so the host counters the launches advance are put back
// and applied per replay instead.
int capture_cycle(rewl_engine* e)
{
    const int se = e->desc.sweeps_per_exchange, rounds = e->desc.sweeps_per_check / se;
    const int64_t s0 = e->sweeps_total, f0 = e->flips_total, l0 = e->launches_total, k0 = e->kernel_launches;
    const uint64_t r0 = e->exch_round;
    const int d0 = e->direction;
    const size_t ev0 = e->ev_used;
    e->drop_graph();
    CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed));
    e->capturing = true;
    int rc = REWL_OK;
    for (int r = 0; r < rounds && rc == REWL_OK; ++r) {
        rc = launch_sweeps(e, se);
        if (rc == REWL_OK) rc = launch_exchange(e);
    }
    if (rc == REWL_OK && cudaMemsetAsync(e->counters.p + 1, 0, 4, e->stream) != cudaSuccess)
        rc = fail(REWL_EDEVICE, "memset during capture failed");
    if (rc == REWL_OK) rc = launch_flat(e);
    e->capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
    if (rc == REWL_OK && ce != cudaSuccess) rc = fail(REWL_EDEVICE, "stream capture: %s", cudaGetErrorString(ce));
    if (rc == REWL_OK && cudaGraphInstantiate(&e->cycle_exec, graph, 0) != cudaSuccess) {
        e->cycle_exec = nullptr;
        rc = fail(REWL_EDEVICE, "graph instantiation failed");
    }
    if (graph) cudaGraphDestroy(graph);
    e->g_sweeps = e->sweeps_total - s0; e->g_flips = e->flips_total - f0;
    e->g_launches = e->launches_total - l0; e->g_kernel_launches = e->kernel_launches - k0; e->g_rounds = rounds;
    e->sweeps_total = s0; e->flips_total = f0; e->launches_total = l0; e->kernel_launches = k0;
    e->exch_round = r0; e->direction = d0; e->sweeps_since_check = 0; e->ev_used = ev0;
    if (rc) e->drop_graph();
    return rc;
}

// One check interval by replaying the captured graph.
int replay_cycle(rewl_engine* e, int32_t* num_flat)
{
    if (!e->cycle_exec)
        if (int rc = capture_cycle(e)) return rc;
    CUDA_TRY(cudaGraphLaunch(e->cycle_exec, e->stream));
    e->sweeps_total += e->g_sweeps; e->flips_total += e->g_flips;
    e->launches_total += e->g_launches; e->kernel_launches += e->g_kernel_launches;
    e->exch_round += (uint64_t)e->g_rounds;
    e->direction ^= (int)(e->g_rounds & 1);
    int rc = finish_check(e, num_flat);     // synchronises the stream
    for (size_t k = 0; k + 1 < e->g_events.size(); k += 2) {
        float t = 0;                        // timing only: a failed read leaves it out
        if (cudaEventElapsedTime(&t, e->g_events[k], e->g_events[k + 1]) == cudaSuccess) e->graph_sweep_ms += t;
        else (void)cudaGetLastError();
    }
    return rc;
}
} // namespace

int rewl_check_flat(rewl_engine* e, int32_t* num_flat)
{
    if (!e) return fail(REWL_EINVAL, "null engine");
    cudaSetDevice(e->desc.device);
    CUDA_TRY(cudaMemsetAsync(e->counters.p + 1, 0, 4, e->stream));
    int rc = launch_flat(e);
    if (rc) return rc;
    return finish_check(e, num_flat);
}

int rewl_reset_histograms(rewl_engine* e, int32_t ii, int32_t w, int32_t reduce)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0) return fail(REWL_EINVAL, "bad window");
    cudaSetDevice(e->desc.device);
    k_reset_window<<<1, 256, 0, e->stream>>>(e->ptrs(), wi, reduce);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    return REWL_OK;
}

int rewl_get_status(rewl_engine* e, rewl_status* st)
{
    if (!e || !st) return fail(REWL_EINVAL, "null argument");
    cudaSetDevice(e->desc.device);
    std::vector<int32_t> done(e->nwin_total);
    unsigned long long stats[2];
    int32_t counters[4];
    CUDA_TRY(cudaMemcpyAsync(done.data(), e->win_done.p, done.size() * 4, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaMemcpyAsync(stats, e->stats.p, sizeof stats, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaMemcpyAsync(counters, e->counters.p, sizeof counters, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    std::memset(st, 0, sizeof *st);
    st->sweeps = e->sweeps_total;
    st->cycles = e->cycles;
    st->flat_events = e->flat_events;
    st->windows_total = e->nwin_total;
    for (int d : done) st->windows_done += d;
    st->all_done = st->windows_done == st->windows_total;
    st->exchanges_attempted = (int64_t)stats[0];
    st->exchanges_accepted = (int64_t)stats[1];
    st->attempted_flips = e->flips_total;
    st->device_error = counters[0];
    st->kernel_launches = e->launches_total;
    return REWL_OK;
}

int rewl_run_cycles(rewl_engine* e, int64_t ncycles, int64_t timeout_ms, rewl_status* st)
{
    if (!e || ncycles < 0) return fail(REWL_EINVAL, "bad arguments");
    cudaSetDevice(e->desc.device);
    const auto t0 = std::chrono::steady_clock::now();
    const int se = e->desc.sweeps_per_exchange, rounds = e->desc.sweeps_per_check / se;
    int rc = REWL_OK;
    if (e->desc.autotune && !e->tuned && (rc = rewl_autotune(e, 0))) return rc;
    for (int64_t c = 0; c < ncycles; ++c) {
        int32_t nflat = 0;
        // a whole check interval replays as one graph unless sweeps were run by hand since the
        // last check (the captured flatness step assumes exactly one interval of sweeps)
        const bool graph = e->desc.graphs && e->desc.rng_mode != REWL_RNG_REPLAY && e->sweeps_since_check == 0;
        if (graph) {
            if ((rc = replay_cycle(e, &nflat))) return rc;
        } else {
            for (int r = 0; r < rounds; ++r) {
                if ((rc = launch_sweeps(e, se))) return rc;
                if ((rc = launch_exchange(e))) return rc;
            }
            if ((rc = rewl_check_flat(e, &nflat))) return rc;
        }
        rewl_status s;
        if ((rc = rewl_get_status(e, &s))) return rc;
        if (st) *st = s;
        if (s.all_done) break;
        if (timeout_ms > 0) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (ms > timeout_ms) return fail(REWL_ETIMEDOUT, "run_cycles deadline of %lld ms passed", (long long)timeout_ms);
        }
    }
    if (st) return rewl_get_status(e, st);
    return REWL_OK;
}

namespace {
// Observable columns of a model, before the count column: Ising |m|, m^2, m^4 (+ G(q_min));
// Ashkin-Teller 12 moments (+ a G(q_min) after each group of three).
int obs_columns(int model, bool corr) { return model == REWL_MODEL_ISING2D ? (corr ? 4 : 3) : (corr ? 16 : 12); }
bool is_corr_column(int model, bool corr, int k) { return corr && (model == REWL_MODEL_ISING2D ? k == 3 : (k & 3) == 3); }

// [nb][K + 1] rows of K averages and the update count, from the sums of the given slots.
// Moments: sum over the slots / total count (the count-weighted mean of the replicas' running
// means).  G(q_min): each slot's sum over its transforms, ceil(count / 1000) of them, weighted
// by the slot's count in the same way.
int export_obs(rewl_engine* e, int ii, const std::vector<int>& slots, double* out)
{
    if (!e->obs.p) return fail(REWL_ESTATE, "the engine was created without observables (rewl_batch_desc.observables)");
    const int model = e->inst[ii].d.model;
    const bool corr = e->desc.observables == 2;
    const int K = obs_columns(model, corr);
    const int nb = e->h_slot_nb[slots[0]];
    const bool single = slots.size() == 1;
    std::vector<double> sum((size_t)nb * K, 0.0), part((size_t)nb * e->obs_stride);
    std::vector<uint64_t> cnt(nb, 0), v(nb);
    for (int s : slots) {
        const int64_t off = e->h_slot_tab[s];
        CUDA_TRY(cudaMemcpyAsync(part.data(), e->obs.p + (size_t)off * e->obs_stride, part.size() * 8,
                                 cudaMemcpyDeviceToHost, e->stream));
        CUDA_TRY(cudaMemcpyAsync(v.data(), e->visits.p + off, nb * 8, cudaMemcpyDeviceToHost, e->stream));
        CUDA_TRY(cudaStreamSynchronize(e->stream));
        for (int b = 0; b < nb; ++b) {
            for (int k = 0; k < K; ++k) {
                const double x = part[(size_t)b * e->obs_stride + k];
                if (!is_corr_column(model, corr, k)) { sum[(size_t)b * K + k] += x; continue; }
                if (!v[b]) continue;
                const double mean = x / (double)((v[b] + kCountsPerTransform - 1) / kCountsPerTransform);
                sum[(size_t)b * K + k] += single ? mean : (double)v[b] * mean;
            }
            cnt[b] += v[b];
        }
    }
    for (int b = 0; b < nb; ++b) {
        for (int k = 0; k < K; ++k) {
            const double x = sum[(size_t)b * K + k];
            out[(size_t)b * (K + 1) + k] = !cnt[b] ? 0.0 : (single && is_corr_column(model, corr, k)) ? x : x / (double)cnt[b];
        }
        out[(size_t)b * (K + 1) + K] = (double)cnt[b];
    }
    return REWL_OK;
}
} // namespace

int rewl_export_observables(rewl_engine* e, int32_t w, double* out)
{
    if (!valid_walker(e, w) || !out) return fail(REWL_EINVAL, "walker %d out of range or null output", w);
    cudaSetDevice(e->desc.device);
    return export_obs(e, e->h_slot_inst[w], {w}, out);
}

int rewl_export_window_observables(rewl_engine* e, int32_t ii, int32_t w, double* out)
{
    if (window_index(e, ii, w) < 0 || !out) return fail(REWL_EINVAL, "bad window or null output");
    cudaSetDevice(e->desc.device);
    const InstDev& I = e->inst[ii].dev;
    std::vector<int> slots;
    for (int r = 0; r < I.R; ++r) slots.push_back(I.first_slot + w * I.R + r);
    return export_obs(e, ii, slots, out);
}

int rewl_export_walker(rewl_engine* e, int32_t w, int8_t* dofs, double* state, uint64_t* counts, double* logdos, uint64_t* visits)
{
    if (!valid_walker(e, w)) return fail(REWL_EINVAL, "walker %d out of range", w);
    cudaSetDevice(e->desc.device);
    const int ii = e->h_slot_inst[w];
    const InstDev& I = e->inst[ii].dev;
    int32_t cfg, flav;
    CUDA_TRY(cudaMemcpyAsync(&cfg, e->slot_cfg.p + w, 4, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaMemcpyAsync(&flav, e->slot_flavour.p + w, 4, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (dofs) CUDA_TRY(cudaMemcpyAsync(dofs, e->spins.p + e->h_cfg_off[cfg], I.ndof, cudaMemcpyDeviceToHost, e->stream));
    int64_t E; int32_t M[3];
    CUDA_TRY(cudaMemcpyAsync(&E, e->cfg_E.p + cfg, 8, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaMemcpyAsync(M, e->cfg_M.p + 3 * cfg, 12, cudaMemcpyDeviceToHost, e->stream));
    const int nb = e->h_slot_nb[w];
    const int64_t off = e->h_slot_tab[w];
    std::vector<int64_t> g(nb); std::vector<uint32_t> h(nb);
    CUDA_TRY(cudaMemcpyAsync(g.data(), e->g.p + off, nb * 8, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaMemcpyAsync(h.data(), e->H.p + off, nb * 4, cudaMemcpyDeviceToHost, e->stream));
    if (visits) CUDA_TRY(cudaMemcpyAsync(visits, e->visits.p + off, nb * 8, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (state) {
        const double Ed = std::ldexp((double)E, -I.escale);
        if (I.model == REWL_MODEL_ISING2D) { state[0] = Ed; state[1] = M[0]; }
        else { state[0] = Ed; state[1] = M[0]; state[2] = M[1]; state[3] = M[2]; state[4] = flav; }
    }
    if (counts) for (int b = 0; b < nb; ++b) counts[b] = h[b];
    if (logdos) for (int b = 0; b < nb; ++b) logdos[b] = (double)g[b] / kLogdosScale;
    return REWL_OK;
}

int rewl_export_window_logdos(rewl_engine* e, int32_t ii, int32_t w, double* out)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0 || !out) return fail(REWL_EINVAL, "bad window or null output");
    cudaSetDevice(e->desc.device);
    const InstDev& I = e->inst[ii].dev;
    const int nb = e->h_wins[wi].nb, R = I.R;
    std::vector<int64_t> g((size_t)R * nb);
    std::vector<uint64_t> v((size_t)R * nb);
    for (int r = 0; r < R; ++r) {
        const int s = I.first_slot + w * R + r;
        CUDA_TRY(cudaMemcpyAsync(g.data() + (size_t)r * nb, e->g.p + e->h_slot_tab[s], nb * 8, cudaMemcpyDeviceToHost, e->stream));
        CUDA_TRY(cudaMemcpyAsync(v.data() + (size_t)r * nb, e->visits.p + e->h_slot_tab[s], nb * 8, cudaMemcpyDeviceToHost, e->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    for (int b = 0; b < nb; ++b) {
        double tot = 0;
        for (int r = 0; r < R; ++r) tot += (double)v[(size_t)r * nb + b];
        double acc = 0;
        if (tot == 0 || R == 1) acc = (double)g[b] / kLogdosScale;
        else for (int r = 0; r < R; ++r) acc = acc + ((double)v[(size_t)r * nb + b] / tot) * ((double)g[(size_t)r * nb + b] / kLogdosScale);
        out[b] = acc;
    }
    return REWL_OK;
}

int rewl_export_window_mask(rewl_engine* e, int32_t ii, int32_t w, uint8_t* out)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0 || !out) return fail(REWL_EINVAL, "bad window or null output");
    cudaSetDevice(e->desc.device);
    const WinDev& W = e->h_wins[wi];
    const InstDev& I = e->inst[ii].dev;
    CUDA_TRY(cudaMemcpyAsync(out, e->mask.p + W.mask_off, W.nb, cudaMemcpyDeviceToHost, e->stream));
    std::vector<uint64_t> v((size_t)I.R * W.nb);
    for (int r = 0; r < I.R; ++r)
        CUDA_TRY(cudaMemcpyAsync(v.data() + (size_t)r * W.nb, e->visits.p + e->h_slot_tab[I.first_slot + w * I.R + r], W.nb * 8, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (e->desc.mask_mode == REWL_MASK_VISITED)
        for (int b = 0; b < W.nb; ++b) {
            bool any = false;
            for (int r = 0; r < I.R; ++r) any |= v[(size_t)r * W.nb + b] != 0;
            if (!any) out[b] = 0;
        }
    return REWL_OK;
}

int rewl_window_state(rewl_engine* e, int32_t ii, int32_t w, double* lnf, int32_t* done)
{
    const int wi = window_index(e, ii, w);
    if (wi < 0) return fail(REWL_EINVAL, "bad window");
    cudaSetDevice(e->desc.device);
    int64_t q; int32_t d;
    CUDA_TRY(cudaMemcpyAsync(&q, e->win_lnf.p + wi, 8, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaMemcpyAsync(&d, e->win_done.p + wi, 4, cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    if (lnf) *lnf = (double)q / kLogdosScale;
    if (done) *done = d;
    return REWL_OK;
}

int rewl_global_logdos(rewl_engine* e, int32_t ii, int32_t half_spectrum, double* energies, double* logdos, int32_t* count)
{
    if (!e || ii < 0 || ii >= (int)e->inst.size() || !count) return fail(REWL_EINVAL, "bad arguments");
    const HostInst& H = e->inst[ii];
    std::vector<std::vector<double>> Es, Gs;
    for (int w = 0; w < H.d.num_windows; ++w) {
        const int nb = H.wins[w].nb;
        std::vector<double> g(nb); std::vector<uint8_t> m(nb);
        int rc = rewl_export_window_logdos(e, ii, w, g.data());
        if (!rc) rc = rewl_export_window_mask(e, ii, w, m.data());
        if (rc) return rc;
        std::vector<double> ee, gg;
        for (int b = 0; b < nb; ++b)
            if (m[b]) { ee.push_back(H.wmin[w] + H.bw * b); gg.push_back(g[b]); }
        Es.push_back(ee); Gs.push_back(gg);
    }
    std::vector<double> fe, fg;
    int rc = concatenate(Es, Gs, fe, fg);
    if (rc) return rc;
    const double states = H.dev.model == REWL_MODEL_ISING2D ? 2.0 : 4.0;
    const double shift = normalisation_shift(fg, states, (double)H.dev.N, half_spectrum != 0);
    if ((int)fe.size() > *count) { *count = (int)fe.size(); return fail(REWL_EINVAL, "output capacity too small (%zu needed)", fe.size()); }
    for (size_t k = 0; k < fe.size(); ++k) { if (energies) energies[k] = fe[k]; if (logdos) logdos[k] = fg[k] + shift; }
    *count = (int)fe.size();
    return REWL_OK;
}

// Observables on the concatenated energy axis (the energies of rewl_global_logdos): every
// window's count-weighted replica average (rewl_export_window_observables) is combined across
// the windows that hold an energy by the reference's running mean
// average_two_windows(final, window, overlapping_windows, 1)
// (src/util/concatenate_rewl_tables.hpp:43-49, 241-256), in window order.
int rewl_concatenate_windows(int32_t num_windows, const int32_t* sizes, const double* energies, const double* logdos,
                             int32_t num_obs, const double* obs, double states_per_site, int64_t system_size,
                             int32_t half_spectrum, int32_t match, double* out_energies, double* out_logdos,
                             double* out_obs, int32_t* count)
{
    if (num_windows < 1 || !sizes || !energies || !logdos || !count || system_size < 1 || !(states_per_site > 0) ||
        num_obs < 0 || (num_obs > 0 && !obs))
        return fail(REWL_EINVAL, "bad arguments");
    if (match != REWL_MATCH_DERIVATIVE && match != REWL_MATCH_REFERENCE) return fail(REWL_EINVAL, "bad match rule");
    std::vector<std::vector<double>> Es(num_windows), Gs(num_windows), Os(num_obs > 0 ? num_windows : 0);
    size_t off = 0;
    for (int w = 0; w < num_windows; ++w) {
        if (sizes[w] < 2) return fail(REWL_EINVAL, "window %d has fewer than 2 rows", w);
        Es[w].assign(energies + off, energies + off + sizes[w]);
        Gs[w].assign(logdos + off, logdos + off + sizes[w]);
        if (num_obs > 0) Os[w].assign(obs + off * num_obs, obs + (off + sizes[w]) * num_obs);
        off += (size_t)sizes[w];
    }
    std::vector<double> fe, fg, fo;
    int rc = concatenate(Es, Gs, fe, fg, match == REWL_MATCH_REFERENCE, num_obs > 0 ? &Os : nullptr, num_obs, &fo);
    if (rc) return rc;
    if ((int64_t)fe.size() > *count) { *count = (int32_t)fe.size(); return fail(REWL_EINVAL, "output capacity too small (%zu needed)", fe.size()); }
    const double shift = normalisation_shift(fg, states_per_site, (double)system_size, half_spectrum != 0);
    for (size_t k = 0; k < fe.size(); ++k) {
        if (out_energies) out_energies[k] = fe[k];
        if (out_logdos) out_logdos[k] = fg[k] + shift;
    }
    if (out_obs && num_obs > 0) std::copy(fo.begin(), fo.end(), out_obs);
    *count = (int32_t)fe.size();
    return REWL_OK;
}

int rewl_global_observables(rewl_engine* e, int32_t ii, double* obs, int32_t* count)
{
    if (!e || ii < 0 || ii >= (int)e->inst.size() || !count) return fail(REWL_EINVAL, "bad arguments");
    if (!e->obs.p) return fail(REWL_ESTATE, "the engine was created without observables (rewl_batch_desc.observables)");
    const HostInst& H = e->inst[ii];
    const int cols = obs_columns(H.d.model, e->desc.observables == 2) + 1;
    const bool half = H.d.model != REWL_MODEL_ISING2D && H.d.energy_max <= 0.0;
    int n = 0;
    int rc = rewl_global_logdos(e, ii, half ? 1 : 0, nullptr, nullptr, &n);
    if (rc && n == 0) return rc;
    std::vector<double> E(n);
    if ((rc = rewl_global_logdos(e, ii, half ? 1 : 0, E.data(), nullptr, &n))) return rc;
    if (n > *count) { *count = n; return fail(REWL_EINVAL, "output capacity too small (%d rows needed)", n); }
    // running means keyed by the global bin index
    std::vector<double> mean;
    std::vector<int64_t> key0;
    std::vector<int> nwin;
    int64_t kmin = INT64_MAX, kmax = INT64_MIN;
    for (int w = 0; w < H.d.num_windows; ++w) {
        kmin = std::min<int64_t>(kmin, H.wins[w].gblo);
        kmax = std::max<int64_t>(kmax, H.wins[w].gblo + H.wins[w].nb);
    }
    mean.assign((size_t)(kmax - kmin) * cols, 0.0);
    nwin.assign((size_t)(kmax - kmin), 0);
    for (int w = 0; w < H.d.num_windows; ++w) {
        const int nb = H.wins[w].nb;
        std::vector<double> o((size_t)nb * cols);
        std::vector<uint8_t> m(nb);
        if ((rc = rewl_export_window_observables(e, ii, w, o.data())) || (rc = rewl_export_window_mask(e, ii, w, m.data())))
            return rc;
        for (int b = 0; b < nb; ++b) {
            if (!m[b]) continue;
            const size_t k = (size_t)(H.wins[w].gblo + b - kmin);
            const int c = nwin[k];
            for (int j = 0; j < cols; ++j) {
                double& v = mean[k * cols + j];
                v = c == 0 ? o[(size_t)b * cols + j] : ((double)c * v + o[(size_t)b * cols + j]) / (double)(c + 1);
            }
            ++nwin[k];
        }
    }
    for (int r = 0; r < n; ++r) {
        const int64_t k = (int64_t)std::llround((E[r] - H.d.energy_min) / H.bw) - kmin;
        if (k < 0 || k >= kmax - kmin || nwin[k] == 0) return fail(REWL_ESTATE, "energy %g has no window observables", E[r]);
        for (int j = 0; j < cols; ++j) obs[(size_t)r * cols + j] = mean[(size_t)k * cols + j];
    }
    *count = n;
    return REWL_OK;
}

namespace {
std::vector<std::string> split_names(const char* names)
{
    std::vector<std::string> v;
    if (!names) return v;
    std::stringstream ss(names);
    std::string line;
    while (std::getline(ss, line, '\n'))
        if (!line.empty()) v.push_back(line);
    return v;
}

// '#' header lines naming the columns (first_cols, then names), as the reference's writers do
void column_header(std::ofstream& f, const char* title, const std::vector<std::string>& first_cols,
                   const std::vector<std::string>& names)
{
    f << "# " << title;
    int col = 0;
    for (const auto& c : first_cols) f << "\n#    " << ++col << ": " << c;
    for (const auto& c : names) f << "\n#    " << ++col << ": " << c;
    f << "\n#\n";
}

int write_table(const char* dir, const char* stem, const char* file_string, const char* header, const char* title,
                const std::vector<std::string>& first_cols, const char* names, int32_t rows, int32_t cols,
                const double* a, const double* b, double scale, const double* values)
{
    if (!dir || !file_string || rows < 1 || cols < 0 || !a || (cols > 0 && !values))
        return fail(REWL_EINVAL, "bad arguments");
    const std::filesystem::path path = std::filesystem::path(dir) / (std::string(stem) + "-" + file_string + ".txt");
    std::ofstream f(path);
    if (!f) return fail(REWL_EINVAL, "cannot open %s for writing", path.string().c_str());
    if (header) f << header;
    column_header(f, title, first_cols, split_names(names));
    f << std::setprecision(std::numeric_limits<double>::digits10) << std::scientific;
    for (int32_t r = 0; r < rows; ++r) {
        f << a[r] / scale << ",";
        if (b) f << b[r] / scale << (cols > 0 ? "," : "");
        for (int32_t c = 0; c < cols; ++c) f << values[(size_t)r * cols + c] << (c + 1 < cols ? "," : "");
        if (r + 1 < rows) f << "\n";
    }
    return f.good() ? REWL_OK : fail(REWL_EINVAL, "write to %s failed", path.string().c_str());
}
} // namespace

// Text formats of the reference's writers (comma-delimited rows, src/Simulation/main_headers.hpp:18;
// '#' header lines; std::scientific with 15 digits): write_microcanonical_observables
// (src/util/write_microcanonical_observables.hpp:16-65), write_observables_to_file
// (src/Thermodynamics/write_self_averaged_observables.hpp:15-59), write_nonlinear_obs_to_file
// (src/Thermodynamics/write_nonlinear_observables.hpp:13-57).
int rewl_write_microcanonical(const char* dir, const char* file_string, const char* header, const char* names,
                              int32_t num_bins, int32_t num_obs, double system_size, const double* energies,
                              const double* logdos, const double* obs)
{
    if (!logdos || !(system_size > 0)) return fail(REWL_EINVAL, "bad arguments");
    return write_table(dir, "microcanonical_observables", file_string, header, "Intensive Observable Names by Column",
                       {"Energy", "logDoS"}, names, num_bins, num_obs, energies, logdos, system_size, obs);
}

int rewl_write_self_averaged(const char* dir, const char* file_string, const char* header, const char* names,
                             int32_t num_T, int32_t num_cols, const double* temperatures, const double* rows)
{
    return write_table(dir, "self_averaged_observables", file_string, header, "Intensive Observable Names by Column",
                       {"Temperature"}, names, num_T, num_cols, temperatures, nullptr, 1.0, rows);
}

int rewl_write_nonlinear(const char* dir, const char* file_string, const char* header, const char* names,
                         int32_t num_T, int32_t num_cols, const double* temperatures, const double* rows)
{
    return write_table(dir, "nonlinear_observables", file_string, header,
                       "Intensive Nonlinear Observable Names by Column", {"Temperature"}, names, num_T, num_cols,
                       temperatures, nullptr, 1.0, rows);
}

// The reference's post-processing of one instance (src/Simulation/main.cpp:241-365): concatenated,
// normalised ln g and observables -> microcanonical file; canonical thermodynamics over the
// temperature ladder (GPU, FP64) -> self-averaged file; susceptibilities and cumulants ->
// nonlinear file.  Without observables the files carry the energy columns only.
int rewl_write_outputs(rewl_engine* e, int32_t ii, const char* dir, const char* file_string, const char* header,
                       double Tmin, double Tmax, int32_t num_T)
{
    if (!e || ii < 0 || ii >= (int)e->inst.size() || !dir || !file_string || num_T < 1) return fail(REWL_EINVAL, "bad arguments");
    const HostInst& H = e->inst[ii];
    const bool ising = H.d.model == REWL_MODEL_ISING2D;
    const bool half = !ising && H.d.energy_max <= 0.0;
    int n = 0;
    rewl_global_logdos(e, ii, half ? 1 : 0, nullptr, nullptr, &n);
    std::vector<double> E(n), G(n);
    int rc = rewl_global_logdos(e, ii, half ? 1 : 0, E.data(), G.data(), &n);
    if (rc) return rc;
    const bool corr = e->desc.observables == 2;
    const int cols = e->obs.p ? obs_columns(H.d.model, corr) + 1 : 0;
    std::vector<double> O((size_t)n * std::max(cols, 1));
    if (cols && (rc = rewl_global_observables(e, ii, O.data(), &n))) return rc;
    // Obs::string_names (ising2d_observables.hpp:40-46, ashkin_teller2d_observables.hpp:64-82)
    const char* sys_names = !cols ? "" : ising
        ? (corr ? "Magnetization\nMagnetization2\nMagnetization4\nG(qmin)\nCounts per Bin"
                : "Magnetization\nMagnetization2\nMagnetization4\nCounts per Bin")
        : (corr ? "Sigma Mag\nSigma Mag2\nSigma Mag4\nSigma G(qmin)\nTau Mag\nTau Mag2\nTau Mag4\nTau G(qmin)\n"
                  "Phi\nPhi2\nPhi4\nPhi G(qmin)\nBaxter\nBaxter2\nBaxter4\nBaxter G(qmin)\nCounts per Bin"
                : "Sigma Mag\nSigma Mag2\nSigma Mag4\nTau Mag\nTau Mag2\nTau Mag4\nPhi\nPhi2\nPhi4\nBaxter\nBaxter2\nBaxter4\nCounts per Bin");
    const double N = (double)H.dev.N;
    if ((rc = rewl_write_microcanonical(dir, file_string, header, sys_names, n, cols, N, E.data(), G.data(), O.data())))
        return rc;
    std::vector<double> T(num_T), rows((size_t)num_T * (5 + cols));
    rc = rewl_thermodynamics(E.data(), G.data(), cols ? O.data() : nullptr, n, cols, cols - 1, N, Tmin, Tmax, num_T, 1,
                             e->desc.device, T.data(), rows.data());
    if (rc) return fail(rc, "thermodynamics: %s", rewl_thermo_last_error_string());
    const std::string thermal = std::string("Free Energy\nEnergy\nEnergy2\nEntropy\nSpecific Heat") + (cols ? "\n" : "") + sys_names;
    if ((rc = rewl_write_self_averaged(dir, file_string, header, thermal.c_str(), num_T, 5 + cols, T.data(), rows.data())))
        return rc;
    if (!cols) return REWL_OK;
    const int nl = ising ? (corr ? 3 : 2) : (corr ? 12 : 8);
    std::vector<double> nonlin((size_t)num_T * nl);
    if ((rc = rewl_nonlinear_observables(H.d.model, corr ? 1 : 0, rows.data(), num_T, 5 + cols, T.data(), N, nonlin.data())))
        return fail(rc, "nonlinear observables: %s", rewl_thermo_last_error_string());
    // Obs::nonlinear_obs_strings (ising2d_observables.hpp:40-46, ashkin_teller2d_observables.hpp:64-82)
    const char* nl_names = ising
        ? (corr ? "Susceptibility\nBinder Cumulant\nCorrelation Length over L" : "Susceptibility\nBinder Cumulant")
        : (corr ? "Sigma Susceptibility\nSigma Binder Cumulant\nSigma Correlation Length over L\n"
                  "Tau Susceptibility\nTau Binder Cumulant\nTau Correlation Length over L\n"
                  "Baxter Susceptibility\nBaxter Binder Cumulant\nBaxter Correlation Length over L\n"
                  "Phi Susceptibility\nPhi Binder Cumulant\nPhi Correlation Length over L"
                : "Sigma Susceptibility\nSigma Binder Cumulant\nTau Susceptibility\nTau Binder Cumulant\n"
                  "Baxter Susceptibility\nBaxter Binder Cumulant\nPhi Susceptibility\nPhi Binder Cumulant");
    return rewl_write_nonlinear(dir, file_string, header, nl_names, num_T, nl, T.data(), nonlin.data());
}

int rewl_sweep_kernel_time(rewl_engine* e, double* ms, int64_t* launches)
{
    if (!e) return fail(REWL_EINVAL, "null engine");
    cudaSetDevice(e->desc.device);
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    double total = 0;
    for (size_t k = 0; k + 1 < e->ev_used; k += 2) {
        float t = 0;
        CUDA_TRY(cudaEventElapsedTime(&t, e->ev_pool[k], e->ev_pool[k + 1]));
        total += t;
    }
    if (ms) *ms = total + e->graph_sweep_ms;
    if (launches) *launches = e->kernel_launches;
    e->ev_used = 0;
    e->kernel_launches = 0;
    e->graph_sweep_ms = 0;
    return REWL_OK;
}

namespace {
struct SnapPart { void* dev; size_t bytes; };

std::vector<SnapPart> snapshot_parts(rewl_engine* e)
{
    auto P = [](auto& b) { return SnapPart{(void*)b.p, b.n * sizeof(*b.p)}; };
    return {P(e->slot_cfg), P(e->slot_flavour), P(e->slot_sweeps), P(e->slot_draws), P(e->cfg_E), P(e->cfg_M),
            P(e->spins), P(e->g), P(e->H), P(e->visits), P(e->win_lnf), P(e->win_done), P(e->win_oot),
            P(e->win_iter), P(e->win_sweepctr), P(e->stats), P(e->obs)};
}

struct SnapHeader {
    uint64_t magic, bytes, exch_round, sweeps_since_check;
    int64_t sweeps_total, cycles, flat_events, flips_total;
    int32_t direction, nslots, nwin, pad;
};
constexpr uint64_t kSnapMagic = 0x5245574C534E4150ull;   // "REWLSNAP"
} // namespace

int rewl_snapshot_size(const rewl_engine* e, size_t* bytes)
{
    if (!e || !bytes) return fail(REWL_EINVAL, "null argument");
    size_t n = sizeof(SnapHeader);
    for (auto& p : snapshot_parts(const_cast<rewl_engine*>(e))) n += (p.bytes + 15) & ~size_t(15);
    *bytes = n;
    return REWL_OK;
}

int rewl_snapshot(rewl_engine* e, void* buffer, size_t bytes)
{
    size_t need = 0;
    if (int rc = rewl_snapshot_size(e, &need)) return rc;
    if (!buffer || bytes < need) return fail(REWL_EINVAL, "snapshot buffer too small (%zu bytes needed)", need);
    cudaSetDevice(e->desc.device);
    SnapHeader h{kSnapMagic, need, e->exch_round, e->sweeps_since_check, e->sweeps_total, e->cycles, e->flat_events,
                 e->flips_total, e->direction, e->nslots, e->nwin_total, 0};
    std::memcpy(buffer, &h, sizeof h);
    char* dst = static_cast<char*>(buffer) + sizeof h;
    for (auto& p : snapshot_parts(e)) {
        if (p.bytes) CUDA_TRY(cudaMemcpyAsync(dst, p.dev, p.bytes, cudaMemcpyDeviceToHost, e->stream));
        dst += (p.bytes + 15) & ~size_t(15);
    }
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    return REWL_OK;
}

int rewl_restore(rewl_engine* e, const void* buffer, size_t bytes)
{
    size_t need = 0;
    if (int rc = rewl_snapshot_size(e, &need)) return rc;
    if (!buffer || bytes < need) return fail(REWL_EINVAL, "snapshot buffer too small (%zu bytes needed)", need);
    SnapHeader h;
    std::memcpy(&h, buffer, sizeof h);
    if (h.magic != kSnapMagic || h.bytes != need || h.nslots != e->nslots || h.nwin != e->nwin_total)
        return fail(REWL_EINVAL, "snapshot does not match this engine's layout");
    cudaSetDevice(e->desc.device);
    const char* src = static_cast<const char*>(buffer) + sizeof h;
    for (auto& p : snapshot_parts(e)) {
        if (p.bytes) CUDA_TRY(cudaMemcpyAsync(p.dev, src, p.bytes, cudaMemcpyHostToDevice, e->stream));
        if (p.dev == (void*)e->win_lnf.p)          // the restored ln f values bound the launch size
            for (size_t k = 0; k < p.bytes / 8; ++k) {
                int64_t v;
                std::memcpy(&v, src + 8 * k, 8);
                raise_lnf_bound(e, v);
            }
        src += (p.bytes + 15) & ~size_t(15);
    }
    const unsigned long long xr[2] = {h.exch_round, 0};
    CUDA_TRY(cudaMemcpyAsync(e->xround.p, xr, sizeof xr, cudaMemcpyHostToDevice, e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    e->exch_round = h.exch_round; e->sweeps_since_check = h.sweeps_since_check; e->sweeps_total = h.sweeps_total;
    e->cycles = h.cycles; e->flat_events = h.flat_events; e->flips_total = h.flips_total; e->direction = h.direction;
    return REWL_OK;
}

// Autotuner: for every launch group with more than one admissible shape (walkers per warp 1, 2
// or 4 for the bin-tracking kernel, warps per block 1, 2, 4 or 8, within what the descriptor
// fixes), time sweeps of that group alone in each shape and keep the fastest.  The trials run
// on the live state, which is saved before and restored after, so tuning leaves the simulation
// exactly where it was; a walker's trajectory does not depend on the shape.
int rewl_autotune(rewl_engine* e, int32_t sweeps)
{
    if (!e || sweeps < 0) return fail(REWL_EINVAL, "bad arguments");
    if (e->fused) { e->tuned = true; return REWL_OK; }     // one walker per warp, grid sized to residency
    cudaSetDevice(e->desc.device);
    size_t bytes = 0;
    if (int rc = rewl_snapshot_size(e, &bytes)) return rc;
    std::vector<char> snap;
    try {
        snap.resize(bytes);
    } catch (const std::bad_alloc&) {
        return fail(REWL_ENOMEM, "autotune: no host memory for the %zu-byte state copy", bytes);
    }
    if (int rc = rewl_snapshot(e, snap.data(), bytes)) return rc;
    const int64_t l0 = e->launches_total, k0 = e->kernel_launches;
    cudaEvent_t a = nullptr, b = nullptr;
    int rc = REWL_OK;
    auto ck = [&](cudaError_t ce) {
        if (ce != cudaSuccess && rc == REWL_OK) rc = fail(REWL_EDEVICE, "autotune: %s", cudaGetErrorString(ce));
        return rc == REWL_OK;
    };
    ck(cudaEventCreate(&a));
    ck(cudaEventCreate(&b));
    const DevPtrs P = e->ptrs();
    for (auto& l : e->launches) {
        if (rc) break;
        int64_t dof = 0;
        for (int s : l.slots) dof += e->inst[e->h_slot_inst[s]].dev.ndof;
        // about 2e7 attempted flips of the group per trial, at least one sweep
        const int ts = std::min(max_launch_sweeps(e),
                                sweeps > 0 ? sweeps
                                           : (int)std::max<int64_t>(1, std::min<int64_t>(e->desc.sweeps_per_exchange,
                                                                                          20000000 / std::max<int64_t>(1, dof))));
        std::vector<std::pair<int, int>> cand;
        // the bin-tracking kernel takes at most 4 warps per block (its launch bounds); 4 walkers
        // per warp is left to the planner's rule for very large batches
        for (int G : {1, 2}) {
            if ((!l.bins && G > 1) || (l.bins && G > (int)l.slots.size())) continue;
            if (e->desc.walkers_per_warp && l.bins && G != e->desc.walkers_per_warp) continue;
            for (int W : {1, 2, 4, 8}) {
                if (l.bins && W > 4) continue;
                if (e->desc.warps_per_block && W != std::min(e->desc.warps_per_block, l.bins ? 4 : 8)) continue;
                if (shape_fits(l, G, W)) cand.push_back({G, W});
            }
        }
        if (cand.size() < 2) continue;
        float best = FLT_MAX;
        std::pair<int, int> pick{l.walkers_per_warp, l.wpb};
        for (const auto& c : cand) {
            l.walkers_per_warp = c.first;
            l.wpb = c.second;
            if ((rc = at_carveout(e, l))) break;
            if ((rc = launch_group(e, l, e->stream, ts, P))) break;         // warm-up
            if (!ck(cudaEventRecord(a, e->stream))) break;
            if ((rc = launch_group(e, l, e->stream, ts, P))) break;
            if (!ck(cudaEventRecord(b, e->stream)) || !ck(cudaEventSynchronize(b))) break;
            float ms = 0;
            if (!ck(cudaEventElapsedTime(&ms, a, b))) break;
            if (ms < best) { best = ms; pick = c; }
        }
        l.walkers_per_warp = pick.first;
        l.wpb = pick.second;
        if (int r2 = at_carveout(e, l)) if (rc == REWL_OK) rc = r2;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (rc == REWL_OK) rc = check_device_error(e);
    const int rr = rewl_restore(e, snap.data(), bytes);
    e->launches_total = l0;
    e->kernel_launches = k0;
    e->drop_graph();
    e->tuned = true;
    return rc ? rc : rr;
}

int rewl_launch_shapes(rewl_engine* e, int32_t* shapes, int32_t* count)
{
    if (!e || !count) return fail(REWL_EINVAL, "bad arguments");
    const int n = (int)e->launches.size();
    if (shapes && *count >= n)
        for (int i = 0; i < n; ++i) {
            const Launch& l = e->launches[i];
            shapes[4 * i] = l.model; shapes[4 * i + 1] = l.bins ? 1 : 0;
            shapes[4 * i + 2] = l.bins ? l.walkers_per_warp : 1; shapes[4 * i + 3] = l.wpb;
        }
    *count = n;
    return REWL_OK;
}

int rewl_get_stream(rewl_engine* e, void** stream)
{
    if (!e || !stream) return fail(REWL_EINVAL, "null argument");
    *stream = (void*)e->stream;
    return REWL_OK;
}

} // extern "C"
