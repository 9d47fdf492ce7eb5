// Canonical thermodynamics from the reference's own header (TEST INFRASTRUCTURE ONLY).
//
// Drives Thermodynamics::calculate_thermodynamics (src/Thermodynamics/thermodynamics.hpp:
// 158-236 with TRAPEZOIDAL_RULE, the reference's default, CMakeLists.txt:40; 238-297
// without) with the Ising (|m|, m^2, m^4, counts) or Ashkin-Teller (12 moments, counts)
// observable layout.  Built by oracle/build_ref.py into oracle/_ref/; never linked by the
// product.
#include <cstddef>
#include <cstring>

#include "thermodynamics.hpp"

namespace {
enum class IsingObs { mag, mag2, mag4, counts_per_bin, NUM_OBS };
enum class ATObs { o0, o1, o2, o3, o4, o5, o6, o7, o8, o9, o10, o11, counts_per_bin, NUM_OBS };

template <class Enum>
void run(size_t nb, const double* E, const double* lng, const double* obs, size_t N, double Tmin, double Tmax,
         size_t nT, double* out, double* temps)
{
    Thermodynamics<double, double, double, Enum> th(nb, Tmin, Tmax, nT);
    th.calculate_thermodynamics(N, E, lng, obs);
    std::memcpy(out, th.canonical_observables, nT * th.total_observables * sizeof(double));
    std::memcpy(temps, th.temperatures, nT * sizeof(double));
}
} // namespace

extern "C" int ref_thermo(int at, size_t nb, const double* E, const double* lng, const double* obs, size_t N,
                          double Tmin, double Tmax, size_t nT, double* out, double* temps)
{
    if (at) run<ATObs>(nb, E, lng, obs, N, Tmin, Tmax, nT, out, temps);
    else run<IsingObs>(nb, E, lng, obs, N, Tmin, Tmax, nT, out, temps);
    return 0;
}

// The reference's nonlinear observables (src/Thermodynamics/order_parameter_cumulants.hpp:17-59)
// on given thermal averages: susceptibility, Binder cumulant, two-component Binder cumulant and
// calculate_correlation_length(G0, Gq, L) / L as calculate_nonlinear_observables uses it
// (src/Hamiltonians/Ising2d/ising2d_observables.hpp:190).
#include "order_parameter_cumulants.hpp"

extern "C" void ref_cumulants(size_t n, const double* m, const double* m2, const double* m4, const double* G,
                              const double* T, size_t N, double* out)
{
    const size_t L = static_cast<size_t>(std::sqrt(N));
    for (size_t i = 0; i < n; ++i) {
        out[4 * i + 0] = calculate_susceptibility<double>(m2[i], m[i], T[i], N);
        out[4 * i + 1] = calculate_Binder_cumulant(m4[i], m2[i]);
        out[4 * i + 2] = calculate_two_component_Binder_cumulant(m4[i], m2[i]);
        out[4 * i + 3] = calculate_correlation_length(m2[i], G[i], L) / L;
    }
}
