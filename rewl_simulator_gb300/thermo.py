"""Canonical thermodynamics from a density of states (C ABI rewl_thermodynamics).

thermodynamics() evaluates, on the GPU in FP64, the reference's
Thermodynamics::calculate_thermodynamics (src/Thermodynamics/thermodynamics.hpp:158-297)
for a ladder of temperatures; nonlinear() derives susceptibilities and Binder
cumulants (order_parameter_cumulants.hpp:17-48).  The defaults are the reference's
run: 50,000 temperatures from 0.01 to 50.01, trapezoidal rule on
(src/Simulation/main.cpp:13-15).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .engine import REWLError

COLUMNS = ["free_energy", "internal_energy", "internal_energy2", "entropy", "specific_heat"]


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def thermodynamics(E, lng, N: int, obs=None, counts_col: int = -1, Tmin: float = 0.01, Tmax: float = 50.01,
                   num_T: int = 50000, trapezoid: bool = True, device: int = 0):
    """Returns (temperatures, rows): rows[i] = [F, U, U2, S, C, observables...] per site."""
    lib = _native.load()
    E = np.ascontiguousarray(E, dtype=np.float64)
    lng = np.ascontiguousarray(lng, dtype=np.float64)
    K = 0
    if obs is not None:
        obs = np.ascontiguousarray(obs, dtype=np.float64)
        K = obs.shape[1]
    T = np.zeros(num_T)
    out = np.zeros((num_T, 5 + K))
    rc = lib.rewl_thermodynamics(_p(E), _p(lng), _p(obs) if obs is not None else None, E.size, K, counts_col,
                                 float(N), Tmin, Tmax, num_T, int(trapezoid), device, _p(T), _p(out))
    if rc != 0:
        raise REWLError(rc, lib.rewl_thermo_last_error_string().decode())
    return T, out


def nonlinear(model: int, T: np.ndarray, rows: np.ndarray, N: int, correlators: bool = False) -> np.ndarray:
    """Susceptibilities and Binder cumulants per temperature (Ising: 2 columns; AT: 8); with
    correlators (rows in the observables = 2 layout) each pair is followed by the correlation
    length over L (Ising: 3 columns; AT: 12)."""
    lib = _native.load()
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    out = np.zeros((T.size, (2 if model == 0 else 8) * (3 if correlators else 2) // 2))
    rc = lib.rewl_nonlinear_observables(model, int(bool(correlators)), _p(rows), T.size, rows.shape[1], _p(T),
                                        float(N), _p(out))
    if rc != 0:
        raise REWLError(rc, lib.rewl_thermo_last_error_string().decode())
    return out
