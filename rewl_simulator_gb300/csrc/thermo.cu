// Canonical thermodynamics from a density of states, in FP64 on the GPU.
//
// Restates Thermodynamics::calculate_thermodynamics (src/Thermodynamics/thermodynamics.hpp:
// 158-236 with TRAPEZOIDAL_RULE, the reference's default, and 238-297 without): for every
// temperature T_i = Tmin + i (Tmax - Tmin) / nT, a log-sum-exp over the energy bins,
//   x_b = ln g_b - E_b / T,  m = max_b x_b,  w_b = exp(x_b - m) (end bins halved under the
//   trapezoidal rule),  Z = sum_b w_b,
// and the rows [F, U, U2, S, C, observables..., mean count] of its canonical_observables:
// F = -T (m + ln Z) / N, U = sum E w / (N Z), U2 = sum E^2 w / (N^2 Z), S = sum ln g w / (N Z),
// C = N (U2 - U^2) / T^2, O_k = sum O_k w / Z, and the counts column averaged over the bins.
// The reference loops over 50,000 temperatures serially (src/Simulation/main.cpp:13-15,
// 339-351); here one block reduces one temperature, all temperatures in one launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cfloat>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/rewl.h"

namespace {

thread_local std::string g_thermo_error;

int tfail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_thermo_error = buf;
    return code;
}

constexpr int kThreads = 256;
constexpr int kMaxObs = 20;            // Ashkin-Teller with correlators: 16 averages + the count

__device__ double block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < kThreads / 32; ++k) r += sh[k];
    return r;                        // valid in thread 0
}

__device__ double block_max(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xFFFFFFFFu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = sh[0];
        for (int k = 1; k < kThreads / 32; ++k) r = fmax(r, sh[k]);
        sh[kThreads / 32] = r;
    }
    __syncthreads();
    return sh[kThreads / 32];        // valid in every thread
}

__global__ void __launch_bounds__(kThreads) k_thermo(const double* E, const double* lng, const double* obs, int nb,
                                                     int K, int counts_col, double N, double Tmin, double dT,
                                                     int nT, int trapezoid, double* temps, double* out)
{
    __shared__ double sh[kThreads / 32 + 1];
    const int t = blockIdx.x;
    if (t >= nT) return;
    const double T = __dadd_rn(Tmin, __dmul_rn(dT, (double)t));   // rounded as the reference's Tmin + dT * i
    double mx = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += kThreads) mx = fmax(mx, lng[b] - E[b] / T);
    mx = block_max(mx, sh);

    double z = 0.0, u = 0.0, u2 = 0.0, s = 0.0, cnt = 0.0, o[kMaxObs];
#pragma unroll
    for (int k = 0; k < kMaxObs; ++k) o[k] = 0.0;
    for (int b = threadIdx.x; b < nb; b += kThreads) {
        const double e = E[b];
        double w = exp((lng[b] - e / T) - mx);
        if (trapezoid && (b == 0 || b == nb - 1)) w *= 0.5;
        z += w;
        u += e * w;
        u2 += e * e * w;
        s += lng[b] * w;
#pragma unroll
        for (int k = 0; k < kMaxObs; ++k)
            if (k < K) {
                const double v = obs[(size_t)b * K + k];
                if (k == counts_col) cnt += v;
                else o[k] += v * w;
            }
    }
    z = block_sum(z, sh);
    u = block_sum(u, sh);
    u2 = block_sum(u2, sh);
    s = block_sum(s, sh);
    cnt = block_sum(cnt, sh);
#pragma unroll
    for (int k = 0; k < kMaxObs; ++k)
        if (k < K) o[k] = block_sum(o[k], sh);
    if (threadIdx.x == 0) {
        double* row = out + (size_t)t * (5 + K);
        const double U = u / (N * z), U2 = u2 / (N * N * z);
        row[0] = -T * (mx + log(z)) / N;
        row[1] = U;
        row[2] = U2;
        row[3] = s / (N * z);
        row[4] = N * (U2 - U * U) / (T * T);
        for (int k = 0; k < K; ++k) row[5 + k] = k == counts_col ? cnt / (double)nb : o[k] / z;
        temps[t] = T;
    }
}

template <typename T>
struct DevArr {
    T* p = nullptr;
    ~DevArr() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return n ? cudaMalloc(&p, n * sizeof(T)) : cudaSuccess; }
};

} // namespace

extern "C" {

const char* rewl_thermo_last_error_string(void) { return g_thermo_error.c_str(); }

int rewl_thermodynamics(const double* E, const double* lng, const double* obs, int32_t nbins, int32_t num_obs,
                        int32_t counts_col, double system_size, double Tmin, double Tmax, int32_t num_T,
                        int32_t trapezoid, int32_t device, double* temperatures, double* out)
{
    if (!E || !lng || !out || !temperatures || nbins < 2 || num_T < 1 || !(system_size > 0) || !(Tmin > 0) ||
        !(Tmax > Tmin) || num_obs < 0 || num_obs > kMaxObs || (num_obs > 0 && !obs) || counts_col >= num_obs)
        return tfail(REWL_EINVAL, "bad arguments (nbins >= 2, 0 < Tmin < Tmax, num_T >= 1, num_obs <= %d)", kMaxObs);
    for (int b = 0; b < nbins; ++b)
        if (!std::isfinite(E[b]) || !std::isfinite(lng[b])) return tfail(REWL_EINVAL, "non-finite energy or ln g at bin %d", b);
    if (cudaSetDevice(device) != cudaSuccess) return tfail(REWL_EDEVICE, "cannot use device %d", device);
    const size_t nrow = 5 + (size_t)num_obs;
    DevArr<double> dE, dg, dobs, dT, dout;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return tfail(REWL_EDEVICE, "stream creation failed");
    cudaError_t e = dE.alloc(nbins);
    if (e == cudaSuccess) e = dg.alloc(nbins);
    if (e == cudaSuccess) e = dobs.alloc((size_t)nbins * num_obs);
    if (e == cudaSuccess) e = dT.alloc(num_T);
    if (e == cudaSuccess) e = dout.alloc((size_t)num_T * nrow);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dE.p, E, nbins * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dg.p, lng, nbins * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && num_obs) e = cudaMemcpyAsync(dobs.p, obs, (size_t)nbins * num_obs * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_thermo<<<num_T, kThreads, 0, st>>>(dE.p, dg.p, dobs.p, nbins, num_obs, counts_col, system_size, Tmin,
                                               (Tmax - Tmin) / (double)num_T, num_T, trapezoid ? 1 : 0, dT.p, dout.p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, (size_t)num_T * nrow * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(temperatures, dT.p, (size_t)num_T * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return tfail(REWL_EDEVICE, "thermodynamics: %s", cudaGetErrorString(e));
    return REWL_OK;
}

// Susceptibilities and Binder cumulants from the rows of rewl_thermodynamics
// (order_parameter_cumulants.hpp:17-48; calculate_nonlinear_observables,
// ising2d_observables.hpp:166-198 and ashkin_teller2d_observables.hpp:243-282).
int rewl_nonlinear_observables(int32_t model, int32_t correlators, const double* rows, int32_t num_T,
                               int32_t row_len, const double* temperatures, double system_size, double* out)
{
    const bool corr = correlators != 0;
    const int need = 5 + (model == REWL_MODEL_ISING2D ? (corr ? 4 : 3) : (corr ? 16 : 12));
    if (!rows || !temperatures || !out || num_T < 1 || row_len < need || (correlators != 0 && correlators != 1) ||
        (model != REWL_MODEL_ISING2D && model != REWL_MODEL_ASHKIN_TELLER2D))
        return tfail(REWL_EINVAL, "bad arguments (rows of at least %d columns)", need);
    auto susc = [&](double m2, double m, double T) { return system_size * (m2 - m * m) / T; };
    auto binder = [](double m4, double m2) { return 1.0 - (m4 / (m2 * m2)) / 3.0; };
    // calculate_correlation_length(G0, Gq, L) / L with L = (size_t) sqrt(N)
    const size_t Ls = static_cast<size_t>(std::sqrt(system_size));
    auto xi = [&](double G0, double Gq) {
        const double x = Gq == 0. ? DBL_MAX : (static_cast<double>(Ls) / (2. * std::acos(-1.))) * std::sqrt((G0 - Gq) / Gq);
        return x / static_cast<double>(Ls);
    };
    for (int t = 0; t < num_T; ++t) {
        const double* o = rows + (size_t)t * row_len + 5;
        const double T = temperatures[t];
        if (model == REWL_MODEL_ISING2D) {
            double* r = out + (size_t)t * (corr ? 3 : 2);
            r[0] = susc(o[1], o[0], T);
            r[1] = binder(o[2], o[1]);
            if (corr) r[2] = xi(o[1], o[3]);
        } else if (!corr) {
            double* r = out + 8 * (size_t)t;
            const int bases[3] = {0, 3, 9};            // sigma, tau, Baxter
            for (int k = 0; k < 3; ++k) {
                r[2 * k] = susc(o[bases[k] + 1], o[bases[k]], T);
                r[2 * k + 1] = binder(o[bases[k] + 2], o[bases[k] + 1]);
            }
            r[6] = susc(o[7], o[6], T);                 // phi: two-component order parameter
            r[7] = 2.0 * (1.0 - 0.5 * (o[8] / (o[7] * o[7])));
        } else {
            // groups of (|x|, x^2, x^4, G): sigma 0, tau 4, phi 8, Baxter 12; output order
            // sigma, tau, Baxter, phi with (susceptibility, cumulant, correlation length)
            double* r = out + 12 * (size_t)t;
            const int bases[3] = {0, 4, 12};
            for (int k = 0; k < 3; ++k) {
                const double* g = o + bases[k];
                r[3 * k] = susc(g[1], g[0], T);
                r[3 * k + 1] = binder(g[2], g[1]);
                r[3 * k + 2] = xi(g[1], g[3]);
            }
            const double* g = o + 8;
            r[9] = susc(g[1], g[0], T);
            r[10] = 2.0 * (1.0 - 0.5 * (g[2] / (g[1] * g[1])));
            r[11] = xi(g[1], g[3]);
        }
    }
    return REWL_OK;
}

} // extern "C"
