// The model plugin surface: the reference's Hamiltonian/observables plugins
// (Hamiltonian_t<T>, State_t<T>, Observables_t<T> chosen at compile time,
// src/Hamiltonians/model_hamiltonians.hpp:6-40) as device-side model types.  A
// model type provides, for a configuration held as int8 +-1 planes (Ising: one
// plane; Ashkin-Teller: sigma then tau) on the L x L periodic square lattice with
// site = y L + x:
//   delta_energy      energy change of flipping plane a's spin at a site (b the other plane)
//   left_flipped      the same after the site's left neighbour in plane a has flipped
//   right_flipped     the correction for a right neighbour in plane a that has flipped
//   recalculate       energy and magnetisations from scratch
//   flip              apply a flip and update the magnetisations
//   add_observables   the per-bin moments of update_observables for the current magnetisations
//   add_correlators   the per-bin G(q_min) transforms of the whole configuration
// and, for the sweep kernels' per-chunk bookkeeping,
//   flip_signs        for each magnetisation, the sign of the site's term before a flip of
//                     plane a (the flip changes it by -2 sign; 0: unchanged)
//   corr_site         a site's value in each correlator plane
//   add_transforms    the G(q_min) of each correlator plane into the observable columns
// kPlanes spin planes, kMags magnetisations, kCorrPlanes correlator planes, corr_mag[p]
// the magnetisation whose terms are correlator plane p's values.
// Energies are integers in the model's units (Ising: J; Ashkin-Teller: 2^-20, with the
// Baxter fields quantised to that grid), so every sum is exact.  The sweep kernels and the
// initial walk are written against these functions; the engine dispatches on the
// per-instance model id (no runtime multi-backend).
#pragma once

#include <cstdint>

__host__ __device__ inline int nb_up(int i, int L) { int x = i % L, y = i / L; return (y == 0 ? L - 1 : y - 1) * L + x; }
__host__ __device__ inline int nb_left(int i, int L) { int x = i % L, y = i / L; return y * L + (x == 0 ? L - 1 : x - 1); }
__host__ __device__ inline int nb_right(int i, int L) { int x = i % L, y = i / L; return y * L + (x == L - 1 ? 0 : x + 1); }
__host__ __device__ inline int nb_down(int i, int L) { int x = i % L, y = i / L; return (y == L - 1 ? 0 : y + 1) * L + x; }

struct Couplings {
    int64_t J, K;            // nearest-neighbour and four-spin couplings in energy units
};

// Fourier_Correlator::compute_correlator (src/Hamiltonians/Correlations/fourier_correlator.hpp:
// 65-118) of plane a, or of the product plane a * b, in the reference's order (one thread):
// half the squared magnitude of the transform of the row sums over y plus that of every site
// over its column x, both at q_min = 2 pi / L (q: L cosines then L sines).
__device__ inline double full_corr(const int8_t* a, const int8_t* b, const double* q, int L)
{
    double rx = 0.0, ix = 0.0, ry = 0.0, iy = 0.0;
    for (int y = 0; y < L; ++y) {
        int rsum = 0;
        for (int x = 0; x < L; ++x) {
            const int v = b ? a[y * L + x] * b[y * L + x] : a[y * L + x];
            rsum += v;
            ry += (double)v * q[x];
            iy += (double)v * q[L + x];
        }
        rx += (double)rsum * q[y];
        ix += (double)rsum * q[L + y];
    }
    return 0.5 * ((rx * rx + ix * ix) + (ry * ry + iy * iy));
}

// 2D Ising, H = -J sum_<ij> s_i s_j (src/Hamiltonians/Ising2d/ising2d_hamiltonian.hpp:162-256).
// One magnetisation M; observables |m|, m^2, m^4 with m = M / N, and G(q_min) of the spins.
struct Ising2dModel {
    static constexpr int kPlanes = 1;
    static constexpr int kMoments = 3;
    static constexpr int kMags = 1;
    static constexpr int kCorrPlanes = 1;
    __host__ __device__ static constexpr int corr_mag(int) { return 0; }

    __host__ __device__ static void flip_signs(int a, int, int, int* sg) { sg[0] = a; }
    __host__ __device__ static int corr_site(const int8_t* sp, int, int i, int) { return sp[i]; }
    __device__ static void add_transforms(double* o, const double* G, double in2) { atomicAdd(o + 3, in2 * G[0]); }

    __host__ __device__ static int64_t delta_energy(const int8_t* a, const int8_t*, int i, int L, Couplings c, int64_t)
    {
        const int sum = a[nb_up(i, L)] + a[nb_left(i, L)] + a[nb_right(i, L)] + a[nb_down(i, L)];
        return 2 * (int64_t)a[i] * c.J * sum;
    }
    __host__ __device__ static int64_t left_flipped(const int8_t* a, const int8_t*, int i, int L, Couplings c, int64_t d0)
    {
        return d0 - 4 * (int64_t)a[i] * a[nb_left(i, L)] * c.J;
    }
    __host__ __device__ static int64_t right_flipped(const int8_t* a, const int8_t*, int i, int L, Couplings c)
    {
        return -4 * (int64_t)a[i] * a[nb_right(i, L)] * c.J;
    }
    // E recomputed as sum_i -1/2 s_i J sum_nb s_nb (ising2d_hamiltonian.hpp:191-210)
    __host__ __device__ static void recalculate(const int8_t* sp, int L, Couplings c, const int64_t*, int64_t& E, int32_t* M)
    {
        const int N = L * L;
        int64_t twiceE = 0;
        int32_t m = 0;
        for (int i = 0; i < N; ++i) {
            const int sum = sp[nb_up(i, L)] + sp[nb_left(i, L)] + sp[nb_right(i, L)] + sp[nb_down(i, L)];
            twiceE -= (int64_t)sp[i] * c.J * sum;
            m += sp[i];
        }
        E = twiceE / 2;
        M[0] = m;
    }
    __host__ __device__ static void flip(int8_t* sp, int, int i, int, int32_t* M)
    {
        M[0] -= 2 * sp[i];
        sp[i] = (int8_t)-sp[i];
    }
    // Ising2d::update_observables (ising2d_hamiltonian.hpp:234-256)
    __device__ static void add_observables(double* o, const int32_t* M, double invN, int)
    {
        const double m = invN * fabs((double)M[0]);
        atomicAdd(o, m);
        atomicAdd(o + 1, m * m);
        atomicAdd(o + 2, m * m * m * m);
    }
    // CORRELATION_LENGTHS (ising2d_hamiltonian.hpp:246-252): G after the three moments
    __device__ static void add_correlators(double* o, const int8_t* sp, int, int L, const double* q, double in2)
    {
        atomicAdd(o + 3, in2 * full_corr(sp, nullptr, q, L));
    }
};

// 2D Ashkin-Teller with Baxter fields, H = -sum_<ij>[J(s s' + t t') + K s t s' t'] - sum_i h_i s_i t_i
// (src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_hamiltonian.hpp:53-62,169-318).  Planes sigma
// and tau; magnetisations sigma, tau and Baxter (sigma tau); the 12 moments of |sigma|, |tau|, phi =
// sqrt(sigma^2 + tau^2) and |Baxter|, and their G(q_min) (tau's from sigma, as the reference does).
struct AshkinTeller2dModel {
    static constexpr int kPlanes = 2;
    static constexpr int kMoments = 12;
    static constexpr int kMags = 3;          // sigma, tau, Baxter
    static constexpr int kCorrPlanes = 2;    // sigma, sigma * tau
    __host__ __device__ static constexpr int corr_mag(int p) { return p == 0 ? 0 : 2; }

    // a: the flipped plane's spin, b: the other plane's
    __host__ __device__ static void flip_signs(int a, int b, int plane, int* sg)
    {
        sg[0] = plane == 0 ? a : 0;
        sg[1] = plane == 0 ? 0 : a;
        sg[2] = a * b;
    }
    __host__ __device__ static int corr_site(const int8_t* sp, int N, int i, int p)
    {
        return p == 0 ? sp[i] : sp[i] * sp[N + i];
    }
    // the tau correlator is computed from sigma, as the reference does (ashkin_teller2d_hamiltonian.hpp:
    // 298-299); phi's is the sum of the two
    __device__ static void add_transforms(double* o, const double* G, double in2)
    {
        const double gs = in2 * G[0], gb = in2 * G[1];
        atomicAdd(o + 3, gs); atomicAdd(o + 7, gs); atomicAdd(o + 11, gs + gs); atomicAdd(o + 15, gb);
    }

    __host__ __device__ static int64_t delta_energy(const int8_t* a, const int8_t* b, int i, int L, Couplings c, int64_t h)
    {
        const int u = nb_up(i, L), l = nb_left(i, L), r = nb_right(i, L), d = nb_down(i, L);
        const int sa = a[u] + a[l] + a[r] + a[d];
        const int sab = a[u] * b[u] + a[l] * b[l] + a[r] * b[r] + a[d] * b[d];
        return 2 * (int64_t)a[i] * (h * b[i] + c.J * sa + c.K * (int64_t)b[i] * sab);
    }
    __host__ __device__ static int64_t left_flipped(const int8_t* a, const int8_t* b, int i, int L, Couplings c, int64_t d0)
    {
        const int l = nb_left(i, L);
        return d0 - 4 * (int64_t)a[i] * a[l] * (c.J + c.K * (int64_t)b[i] * b[l]);
    }
    __host__ __device__ static int64_t right_flipped(const int8_t* a, const int8_t* b, int i, int L, Couplings c)
    {
        const int r = nb_right(i, L);
        return -4 * (int64_t)a[i] * a[r] * (c.J + c.K * (int64_t)b[i] * b[r]);
    }
    __host__ __device__ static void recalculate(const int8_t* sp, int L, Couplings c, const int64_t* h, int64_t& E, int32_t* M)
    {
        const int N = L * L;
        const int8_t* s = sp;
        const int8_t* t = sp + N;
        int64_t twiceE = 0;
        int32_t sm = 0, tm = 0, bx = 0;
        for (int i = 0; i < N; ++i) {
            const int u = nb_up(i, L), l = nb_left(i, L), r = nb_right(i, L), d = nb_down(i, L);
            const int ss = s[u] + s[l] + s[r] + s[d];
            const int tt = t[u] + t[l] + t[r] + t[d];
            const int st = s[u] * t[u] + s[l] * t[l] + s[r] * t[r] + s[d] * t[d];
            twiceE -= (int64_t)s[i] * c.J * ss + (int64_t)t[i] * c.J * tt + (int64_t)s[i] * t[i] * c.K * st;
            if (h) twiceE -= 2 * h[i] * s[i] * t[i];
            sm += s[i]; tm += t[i]; bx += s[i] * t[i];
        }
        E = twiceE / 2;
        M[0] = sm; M[1] = tm; M[2] = bx;
    }
    __host__ __device__ static void flip(int8_t* sp, int N, int i, int plane, int32_t* M)
    {
        int8_t* s = sp;
        int8_t* t = sp + N;
        M[2] -= 2 * s[i] * t[i];
        if (plane == 0) { M[0] -= 2 * s[i]; s[i] = (int8_t)-s[i]; }
        else { M[1] -= 2 * t[i]; t[i] = (int8_t)-t[i]; }
    }
    // Ashkin_Teller2d::update_observables (ashkin_teller2d_hamiltonian.hpp:267-318); with
    // correlators each group of three moments is followed by its G(q_min) column
    // (ashkin_teller2d_observables.hpp:36-41)
    __device__ static void add_observables(double* o, const int32_t* M, double invN, int corr)
    {
        const double a = invN * fabs((double)M[0]), t = invN * fabs((double)M[1]), b = invN * fabs((double)M[2]);
        const double p2 = a * a + t * t;
        const int g = corr ? 1 : 0;
        atomicAdd(o + 0, a); atomicAdd(o + 1, a * a); atomicAdd(o + 2, a * a * a * a);
        o += g;
        atomicAdd(o + 3, t); atomicAdd(o + 4, t * t); atomicAdd(o + 5, t * t * t * t);
        o += g;
        atomicAdd(o + 6, sqrt(p2)); atomicAdd(o + 7, p2); atomicAdd(o + 8, p2 * p2);
        o += g;
        atomicAdd(o + 9, b); atomicAdd(o + 10, b * b); atomicAdd(o + 11, b * b * b * b);
    }
    // CORRELATION_LENGTHS (ashkin_teller2d_hamiltonian.hpp:295-315): the tau correlator is
    // computed from sigma as in the reference (:298-299); phi's is the sum of the two
    __device__ static void add_correlators(double* o, const int8_t* sp, int N, int L, const double* q, double in2)
    {
        const double gs = in2 * full_corr(sp, nullptr, q, L);
        const double gb = in2 * full_corr(sp, sp + N, q, L);
        atomicAdd(o + 3, gs); atomicAdd(o + 7, gs); atomicAdd(o + 11, gs + gs); atomicAdd(o + 15, gb);
    }
};
