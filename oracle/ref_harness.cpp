// TEST INFRASTRUCTURE ONLY -- never linked into the product.
//
// C shim around the reference's own single-walker hot path, compiled from the
// reference sources in place (see oracle/build_ref.py).  It instantiates
// REWL_Walker (src/REWL/rewl_walker.hpp:15-158) together with Wang_Landau
// (src/REWL/wang_landau.hpp:51-141), the selected Hamiltonian
// (src/Hamiltonians/Ising2d/ising2d_hamiltonian.hpp or
//  src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_hamiltonian.hpp),
// the glazier (src/REWL/glazier.hpp:70-115) and normalize_logDoS
// (src/util/array_shift.hpp:15-43), so that golden fixtures and the CPU
// restatement in oracle/rewl_oracle.cpp can be pinned against the reference.
//
// The model parameters (L, J, K, bin width) are compile-time constants in the
// reference; build_ref.py writes a parameter header per build that defines the
// same names and include guard, so the reference's own parameter file is not
// used and nothing from the reference tree is copied or patched.
//
// Ashkin-Teller energies with real-valued Baxter fields are not integers, and
// the reference's histogram_index::energy_in_range (src/REWL/histogram_index.hpp:22-30)
// truncates to int, so the harness instantiates the walker with an exact index
// functor for that model (the walker is templated on it, rewl_walker.hpp:15).

#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>

#include <histogram_index.hpp>
#include <rewl_walker.hpp>
#include <glazier.hpp>
#include <array_shift.hpp>
#include <concatenate_rewl_tables.hpp>
#include <Disorder/random_fields.hpp>

// Exact bin index for dyadic energies: bin = floor((E - min) * inv_width) where
// inv_width is an integer (20 for a 0.05 bin).  Energies and window edges are
// multiples of 2^-20, so every product below is exact in double.
struct exact_histogram_index
{
    const double min_value;
    const double max_value;
    const double bin_size;
    const double inv_width;

    exact_histogram_index(const double mn, const double mx, const double bs)
        : min_value(mn), max_value(mx), bin_size(bs), inv_width(std::nearbyint(1.0 / bs)) {}

    size_t operator()(const double value) const { return static_cast<size_t>(std::floor((value - min_value) * inv_width)); }
    double get_bin_min(const size_t bin) const { return min_value + static_cast<double>(bin) / inv_width; }
    bool energy_too_low(const double value) const { return value < min_value; }
    bool energy_too_high(const double value) const { return value >= max_value; }
    bool energy_in_range(const double value) const { return value >= min_value && value < max_value; }
};

#if ASHKIN_TELLER2D
using index_t = exact_histogram_index;
#else
using index_t = histogram_index<double>;
#endif

using walker_t = REWL_Walker<double, double, double, index_t>;

extern "C" {

int ref_model_id()
{
#if ASHKIN_TELLER2D
    return 1;
#else
    return 0;
#endif
}
size_t ref_L() { return System_Parameters::L; }
size_t ref_num_dof() { return System_Parameters::num_DoF; }
size_t ref_num_obs() { return convert(System_Obs_enum_t::NUM_OBS); }

void* ref_walker_new(double wmin, double wmax, double bsize, size_t nbins, uint32_t seed)
{
    return new walker_t(wmin, wmax, bsize, nbins, seed);
}

void ref_walker_free(void* w) { delete static_cast<walker_t*>(w); }

void ref_walker_import_dofs(void* w, const double* dofs)
{
    static_cast<walker_t*>(w)->system.import_DoFs(dofs);
}

void ref_walker_import_disorder(void* w, const double* fields)
{
#if RFAT_BAXTER || RFIM
    static_cast<walker_t*>(w)->system.import_disorder(fields);
#else
    (void)w; (void)fields;
#endif
}

void ref_walker_adjust(void* w) { static_cast<walker_t*>(w)->adjust_state_to_range(); }

void ref_walker_walk(void* w, size_t nsweeps) { static_cast<walker_t*>(w)->wang_landau_walk(nsweeps); }

void ref_walker_set_incrementer(void* w, double lnf) { static_cast<walker_t*>(w)->incrementer = lnf; }

void ref_walker_reset(void* w) { static_cast<walker_t*>(w)->wl_walker.reset_histogram(); }

float ref_walker_flatness(void* w) { return static_cast<walker_t*>(w)->wl_walker.wl_histograms.count_flatness(); }

// state layout: Ising [E, M]; Ashkin-Teller [E, sigma_mag, tau_mag, baxter, which_to_update]
void ref_walker_get_state(void* w, double* out)
{
    const auto& st = static_cast<walker_t*>(w)->system.current_state;
#if ASHKIN_TELLER2D
    out[0] = st.energy; out[1] = st.sigma_magnetization; out[2] = st.tau_magnetization;
    out[3] = st.baxter; out[4] = static_cast<double>(st.which_to_update);
#else
    out[0] = st.energy; out[1] = st.magnetization;
#endif
}

void ref_walker_get_dofs(void* w, double* out)
{
    const double* d = static_cast<walker_t*>(w)->system.get_front_DoFs();
    std::memcpy(out, d, sizeof(double) * System_Parameters::num_DoF);
}

void ref_walker_get_hist(void* w, uint64_t* counts, double* logdos)
{
    const auto& h = static_cast<walker_t*>(w)->wl_walker.wl_histograms;
    for (size_t b = 0; b != h.num_bins; ++b) { counts[b] = h.get_count(b); logdos[b] = h.get_logdos(b); }
}

void ref_walker_get_obs(void* w, double* out)
{
    const auto& o = static_cast<walker_t*>(w)->system_obs;
    std::memcpy(out, o.obs_array, sizeof(double) * o.num_bins * convert(System_Obs_enum_t::NUM_OBS));
}

// The reference's disorder generator, generate_random_field
// (src/Hamiltonians/Disorder/random_fields.hpp:41-75), run from a given seed instead of the clock:
// per site WAIT_BETWEEN_FIELD_GENERATION discarded values, then the kept one, drawn by the
// reference's own gaussian_random_field / uniform_random_field (:27-38).  type follows its
// disorder_distribution enum (0 uniform, 1 gaussian).
void ref_random_fields(uint64_t seed, double strength, int type, size_t n, double* out)
{
    random_number_generator<double> rng(seed);
    double (*gen)(random_number_generator<double>&, const double) =
        type == disorder_distribution::uniform ? &uniform_random_field<double> : &gaussian_random_field<double>;
    for (size_t i = 0; i != n; ++i) {
        double h = 0.;
        for (size_t r = 0; r != WAIT_BETWEEN_FIELD_GENERATION; ++r) h = gen(rng, strength);
        (void)h;
        out[i] = gen(rng, strength);
    }
}

// The reference's post-processing of window tables: concatenate_tables_multiple_overlap
// (src/util/concatenate_rewl_tables.hpp:167-305, with find_left_concatenation_indices,
// src/util/vector_matching.hpp:38-88) on (energy, logDoS) tables of num_windows windows stored
// one after another (sizes[w] rows each), then normalize_logDoS (src/util/array_shift.hpp:15-43).
// num_obs observables per row ride along in O (rows of num_obs, same order as E) and come
// back averaged over the overlaps in outO.  *n: capacity in, rows out.
void ref_concatenate(size_t num_windows, const size_t* sizes, const double* E, const double* G,
                     size_t num_obs, const double* O, double states_per_site, size_t system_size,
                     double energy_max, double* outE, double* outG, double* outO, size_t* n)
{
    table<double> et(num_windows), gt(num_windows), ot(num_windows);
    size_t off = 0;
    for (size_t w = 0; w != num_windows; ++w) {
        et[w].assign(E + off, E + off + sizes[w]);
        gt[w].assign(G + off, G + off + sizes[w]);
        ot[w].assign(O + off * num_obs, O + (off + sizes[w]) * num_obs);
        off += sizes[w];
    }
    std::vector<double> fe, fg, fo;
    concatenate_tables_multiple_overlap<double, double, double>(num_obs, num_obs - 1, et, gt, ot, fe, fg, fo);
    normalize_logDoS<double, true>(states_per_site, system_size, energy_max, fg.size(), fg.data());
    const size_t m = fe.size() < *n ? fe.size() : *n;
    for (size_t i = 0; i != m; ++i) { outE[i] = fe[i]; outG[i] = fg[i]; }
    for (size_t i = 0; i != m * num_obs; ++i) outO[i] = fo[i];
    *n = fe.size();
}

// Uniforms drawn by the reference's generator with a given seed (the stream a
// walker consumes): random_number_generator<double> (src/util/random_number_generators.hpp:14-31).
void ref_uniforms(uint64_t seed, size_t n, double* out)
{
    random_number_generator<double> r(seed);
    for (size_t i = 0; i != n; ++i) out[i] = r();
}

void ref_glazier(double gmin, double gmax, double bw, size_t nwin, size_t rpw, double overlap,
                 double* mins, double* maxs, uint64_t* nbins)
{
    glazier<double, histogram_index<double> > g(gmin, gmax, bw, nwin, rpw, overlap);
    g.construct_windows();
    for (size_t w = 0; w != nwin; ++w)
    {
        mins[w] = g.all_windows[w * rpw].minimum;
        maxs[w] = g.all_windows[w * rpw].maximum;
        nbins[w] = g.all_windows[w * rpw].num_bins;
    }
}

// normalize_logDoS with energy_max == 0 semantics (half spectrum, -ln 2 term) or full spectrum.
void ref_normalize_logdos(double states_per_site, size_t system_size, double energy_max, size_t n, double* logdos)
{
    normalize_logDoS<double, true>(states_per_site, system_size, energy_max, n, logdos);
}

} // extern "C"
