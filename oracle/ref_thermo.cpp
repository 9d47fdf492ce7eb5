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
