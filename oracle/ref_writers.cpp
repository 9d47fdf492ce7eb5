// The reference's output writers, called on given arrays (TEST INFRASTRUCTURE ONLY).
// write_microcanonical_observables (src/util/write_microcanonical_observables.hpp:16-65),
// write_observables_to_file (src/Thermodynamics/write_self_averaged_observables.hpp:15-59),
// write_nonlinear_obs_to_file (src/Thermodynamics/write_nonlinear_observables.hpp:13-57),
// with the reference's delimiter (src/Simulation/main_headers.hpp:18).  Built by
// oracle/build_ref.py into oracle/_ref/; never linked by the product.
#include <filesystem>
#include <iomanip>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

const std::string DELIMITER = ",";

#include "write_microcanonical_observables.hpp"
#include "write_nonlinear_observables.hpp"
#include "write_self_averaged_observables.hpp"

namespace {
std::vector<std::string> names_of(const char* s)
{
    std::vector<std::string> v;
    std::stringstream ss(s);
    std::string line;
    while (std::getline(ss, line, '\n'))
        if (!line.empty()) v.push_back(line);
    v.push_back("NUM OBS");                 // the reference's name lists end with it
    return v;
}
} // namespace

extern "C" int ref_write(int kind, const char* dir, const char* file_string, const char* header, const char* names,
                         size_t rows, size_t cols, double system_size, const double* a, const double* b,
                         const double* values)
{
    const std::filesystem::path path(dir);
    if (kind == 0)
        write_microcanonical_observables<double, double, double>((size_t)system_size, rows, cols, cols - 1, file_string,
                                                                 header, names_of(names), path, a, b, values);
    else if (kind == 1)
        write_observables_to_file<double, double>(rows, cols, file_string, header, names_of(names), path, a, values);
    else
        write_nonlinear_obs_to_file<double, double>(rows, cols, file_string, header, names_of(names), path, a, values);
    return 0;
}
