"""Output files in the reference's text formats (C ABI rewl_write_*).

write_outputs() runs the reference's post-processing of one instance
(src/Simulation/main.cpp:241-365): concatenated, normalised ln g and per-bin
observables -> microcanonical_observables-<name>.txt; canonical thermodynamics over
a temperature ladder (GPU, FP64) -> self_averaged_observables-<name>.txt;
susceptibilities and Binder cumulants -> nonlinear_observables-<name>.txt.  The
files parse like the reference's: '#' header lines naming the columns, then
comma-delimited rows in scientific notation with 15 digits.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _native
from .engine import Engine, REWLError, obs_columns


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(lib, rc):
    if rc != 0:
        raise REWLError(rc, lib.rewl_last_error_string().decode())


def write_outputs(engine: Engine, instance: int, directory, name: str, header: str = "",
                  Tmin: float = 0.01, Tmax: float = 50.01, num_T: int = 50000) -> list[Path]:
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    lib = engine.lib
    _check(lib, lib.rewl_write_outputs(engine.h, instance, str(d).encode(), name.encode(), header.encode(),
                                       Tmin, Tmax, num_T))
    return [d / f"{stem}-{name}.txt" for stem in ("microcanonical_observables", "self_averaged_observables",
                                                 "nonlinear_observables") if (d / f"{stem}-{name}.txt").exists()]


def global_observables(engine: Engine, instance: int) -> np.ndarray:
    """Observables on the energies of global_logdos (rows: K averages, count)."""
    E, _ = engine.global_logdos(instance, half_spectrum=engine.batch.instances[instance].model != 0
                                and engine.batch.instances[instance].energy_max <= 0.0)
    cols = obs_columns(engine.batch.instances[instance].model, engine.batch.observables)
    out = np.zeros((E.size, cols))
    n = C.c_int32(E.size)
    _check(engine.lib, engine.lib.rewl_global_observables(engine.h, instance, _p(out), C.byref(n)))
    return out[:n.value]


def write_table(kind: str, directory, name: str, header: str, names, first, values, second=None,
                system_size: float = 1.0) -> Path:
    """One file in the reference's format: kind is 'microcanonical' (first = E, second = ln g,
    both divided by system_size), 'self_averaged' or 'nonlinear' (first = temperatures)."""
    lib = _native.load()
    first = np.ascontiguousarray(first, dtype=np.float64)
    values = np.ascontiguousarray(values, dtype=np.float64).reshape(first.size, -1)
    nm = "\n".join(names).encode()
    args = (str(directory).encode(), name.encode(), header.encode(), nm)
    if kind == "microcanonical":
        second = np.ascontiguousarray(second, dtype=np.float64)
        rc = lib.rewl_write_microcanonical(*args, first.size, values.shape[1], system_size, _p(first), _p(second),
                                           _p(values))
    elif kind == "self_averaged":
        rc = lib.rewl_write_self_averaged(*args, first.size, values.shape[1], _p(first), _p(values))
    else:
        rc = lib.rewl_write_nonlinear(*args, first.size, values.shape[1], _p(first), _p(values))
    _check(lib, rc)
    return Path(directory) / f"{kind}_observables-{name}.txt"
