"""Build recipe for the reference harness (TEST INFRASTRUCTURE ONLY).

Compiles oracle/ref_harness.cpp against the reference's own headers where they
lie (the directory named by the environment variable REWL_REFERENCE_DIR, which
must be set: without it the harness is simply not available) into oracle/_ref/, one shared
library per (model, L, K, bin width) because the reference fixes those at
compile time (src/Hamiltonians/Ising2d/ising2d_parameters.cxx:13-69,
src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_parameters.cxx:13-70).

The reference's parameter file is bypassed, not patched: a generated header that
defines the same include guard, constants and namespace is force-included first,
so the reference's `#include "..._parameters.cxx"` becomes a no-op.  A one-line
empty mpi.h stands in for MPI, which the hot path includes but does not call
without MPI_ON (src/REWL/wang_landau.hpp:12).

Outputs go only to oracle/_ref/ (git-ignored).  The reference tree is read only.
Nothing on the product path imports this module.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
_REF_ENV = os.environ.get("REWL_REFERENCE_DIR")
REF = Path(_REF_ENV) if _REF_ENV else None


def reference_available() -> bool:
    return REF is not None and (REF / "src" / "REWL" / "rewl_walker.hpp").is_file()


def _ising_params(L: int, bw: float) -> str:
    return f"""#ifndef ISING2D_PARAMETER_DEFINITIONS
#define ISING2D_PARAMETER_DEFINITIONS
#include <cmath>
#include <cstddef>
constexpr size_t SYSTEM_SIZE_L = {L};
constexpr double SYSTEM_EXCHANGE_J = 1.0;
constexpr double SYSTEM_FIELD_H = 0.0;
constexpr size_t SYSTEM_NUM_NEAREST_NEIGHBORS_int = 4;
constexpr double SYSTEM_NUM_NEAREST_NEIGHBORS_double = 4;
constexpr double GROUND_STATE_DEGENERACY = 2.;
constexpr double SYSTEM_ENERGY_MIN = -0.5 * SYSTEM_EXCHANGE_J * SYSTEM_NUM_NEAREST_NEIGHBORS_double * SYSTEM_SIZE_L * SYSTEM_SIZE_L;
constexpr double SYSTEM_ENERGY_MAX = 0.;
constexpr double SYSTEM_ENERGY_BIN_WIDTH = {bw!r};
constexpr size_t SYSTEM_NUM_BINS = static_cast<size_t>((SYSTEM_ENERGY_MAX - SYSTEM_ENERGY_MIN) / SYSTEM_ENERGY_BIN_WIDTH);
namespace Ising2d_Parameters
{{
    constexpr size_t L = SYSTEM_SIZE_L;
    constexpr size_t N = L * L;
    constexpr double divide_N = 1. / static_cast<double>(N);
    constexpr size_t num_DoF = N;
    constexpr double J = SYSTEM_EXCHANGE_J;
    constexpr double h = SYSTEM_FIELD_H;
    constexpr size_t num_neighbors_i = SYSTEM_NUM_NEAREST_NEIGHBORS_int;
    constexpr double num_neighbors_f = SYSTEM_NUM_NEAREST_NEIGHBORS_double;
    constexpr double ground_state_degeneracy = GROUND_STATE_DEGENERACY;
    constexpr double energy_min = SYSTEM_ENERGY_MIN;
    constexpr double energy_max = SYSTEM_ENERGY_MAX;
    constexpr double energy_bin_size = SYSTEM_ENERGY_BIN_WIDTH;
    constexpr size_t num_bins = SYSTEM_NUM_BINS;
}}
#endif
"""


def _at_params(L: int, K: float, bw: float, h: float) -> str:
    return f"""#ifndef ASKIN_TELLER2D_PARAMETER_DEFINITIONS
#define ASKIN_TELLER2D_PARAMETER_DEFINITIONS
#include <cmath>
#include <cstddef>
constexpr size_t SYSTEM_SIZE_L = {L};
constexpr double SYSTEM_EXCHANGE_J = 1.0;
constexpr double SYSTEM_EXCHANGE_K = {K!r};
constexpr double BAXTER_FIELD_H = {h!r};
constexpr size_t SYSTEM_NUM_NEAREST_NEIGHBORS_int = 4;
constexpr double SYSTEM_NUM_NEAREST_NEIGHBORS_double = 4;
constexpr double GROUND_STATE_DEGENERACY = 4.;
constexpr double SYSTEM_ENERGY_MIN = -0.5 * (2 * SYSTEM_EXCHANGE_J + SYSTEM_EXCHANGE_K) * SYSTEM_NUM_NEAREST_NEIGHBORS_double * SYSTEM_SIZE_L * SYSTEM_SIZE_L;
constexpr double SYSTEM_ENERGY_MAX = 0.;
constexpr double SYSTEM_ENERGY_BIN_WIDTH = {bw!r};
constexpr size_t SYSTEM_NUM_BINS = static_cast<size_t>((SYSTEM_ENERGY_MAX - SYSTEM_ENERGY_MIN) / SYSTEM_ENERGY_BIN_WIDTH);
namespace Ashkin_Teller2d_Parameters
{{
    constexpr size_t L = SYSTEM_SIZE_L;
    constexpr size_t N = L * L;
    constexpr double divide_N = 1. / static_cast<double>(N);
    constexpr size_t num_DoF = 2 * N;
    constexpr double J = SYSTEM_EXCHANGE_J;
    constexpr double K = SYSTEM_EXCHANGE_K;
    constexpr double h = BAXTER_FIELD_H;
    constexpr size_t num_neighbors_i = SYSTEM_NUM_NEAREST_NEIGHBORS_int;
    constexpr double num_neighbors_f = SYSTEM_NUM_NEAREST_NEIGHBORS_double;
    constexpr double ground_state_degeneracy = GROUND_STATE_DEGENERACY;
    constexpr double energy_min = SYSTEM_ENERGY_MIN;
    constexpr double energy_max = SYSTEM_ENERGY_MAX;
    constexpr double energy_bin_size = SYSTEM_ENERGY_BIN_WIDTH;
    constexpr size_t num_bins = SYSTEM_NUM_BINS;
}}
#endif
"""


def tag(model: str, L: int, bw: float, K: float = 0.5, fields: bool = True, corr: bool = False) -> str:
    c = "_corr" if corr else ""
    if model == "ising":
        return f"ising_L{L}_bw{bw:g}{c}"
    return f"at_L{L}_K{K:g}_bw{bw:g}_{'rf' if fields else 'clean'}{c}"


def build(model: str, L: int, bw: float, K: float = 0.5, fields: bool = True, force: bool = False,
          corr: bool = False) -> Path:
    """Build (or reuse) oracle/_ref/<tag>.so and return its path.  corr: the reference's
    CORRELATION_LENGTHS build (its CMake default), whose observables carry G(q_min) columns."""
    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REF}")
    t = tag(model, L, bw, K, fields, corr)
    so = OUT / f"libref_{t}.so"
    if so.exists() and not force and so.stat().st_mtime >= (HERE / "ref_harness.cpp").stat().st_mtime:
        return so                                   # built, and not older than the harness source
    gen = OUT / "gen" / t
    stub = OUT / "stub"
    gen.mkdir(parents=True, exist_ok=True)
    stub.mkdir(parents=True, exist_ok=True)
    (stub / "mpi.h").write_text("/* empty: the single-walker hot path makes no MPI calls without MPI_ON */\n")
    params = gen / "params.hpp"
    if model == "ising":
        params.write_text(_ising_params(L, bw))
        defs = ["-DISING2D"]
    else:
        params.write_text(_at_params(L, K, bw, 0.0))
        defs = ["-DASHKIN_TELLER2D", "-DGAUSSIAN_DISORDER"] + (["-DRFAT_BAXTER"] if fields else [])
    src = REF / "src"
    incs = [stub, src / "REWL", src / "util", src / "Hamiltonians", src / "Thermodynamics"]
    if corr:
        defs.append("-DCORRELATION_LENGTHS=1")
    cmd = (["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-DREDUCE_LOGDOS", "-DEQUAL_WINDOWS"]
           + defs + ["-include", str(params)] + [f"-I{p}" for p in incs]
           + [str(HERE / "ref_harness.cpp"), "-o", str(so)])
    subprocess.run(cmd, check=True)
    return so


def build_thermo(trapezoid: bool = True, force: bool = False) -> Path:
    """oracle/_ref/libref_thermo[_plain].so: the reference's thermodynamics.hpp driven by
    oracle/ref_thermo.cpp (TRAPEZOIDAL_RULE on by default, as in the reference's build)."""
    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REF}")
    so = OUT / ("libref_thermo.so" if trapezoid else "libref_thermo_plain.so")
    if so.exists() and not force:
        return so
    OUT.mkdir(parents=True, exist_ok=True)
    cmd = (["g++", "-std=c++17", "-O2", "-fPIC", "-shared"] + (["-DTRAPEZOIDAL_RULE"] if trapezoid else [])
           + [f"-I{REF / 'src' / 'Thermodynamics'}", str(HERE / "ref_thermo.cpp"), "-o", str(so)])
    subprocess.run(cmd, check=True)
    return so


def build_writers(force: bool = False) -> Path:
    """oracle/_ref/libref_writers.so: the reference's three output writers (oracle/ref_writers.cpp)."""
    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REF}")
    so = OUT / "libref_writers.so"
    if so.exists() and not force:
        return so
    OUT.mkdir(parents=True, exist_ok=True)
    src = REF / "src"
    cmd = (["g++", "-std=c++17", "-O1", "-fPIC", "-shared"]
           + [f"-I{src / d}" for d in ("util", "Thermodynamics", "file_management")]
           + [str(HERE / "ref_writers.cpp"), "-o", str(so)])
    subprocess.run(cmd, check=True)
    return so


if __name__ == "__main__":
    m = sys.argv[1] if len(sys.argv) > 1 else "ising"
    L = int(sys.argv[2]) if len(sys.argv) > 2 else 8
    bw = float(sys.argv[3]) if len(sys.argv) > 3 else (4.0 if m == "ising" else 0.05)
    print(build(m, L, bw, force=True))
