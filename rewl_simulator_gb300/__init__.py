"""GB300-native replica-exchange Wang-Landau (REWL) engine.

The hot path -- batched single-spin-flip Wang-Landau sweeps with replica
exchange between overlapping energy windows for the 2D Ising and 2D
Ashkin-Teller models -- runs as hand-written sm_103a CUDA kernels behind the C
ABI in include/rewl.h.  This package builds that library in-tree and exposes a
Python mirror of the ABI.
"""
from ._native import build as _build_native, load as load_library, LIB as LIBRARY_PATH
from .engine import (Batch, Engine, Instance, REWLError, Status, DISORDER_GAUSSIAN, DISORDER_UNIFORM,
                     FLAT_ALL_VISITED, FLAT_MAX_MIN_RATIO, FLAT_MIN_OVER_MEAN, MASK_STATIC, MASK_VISITED,
                     MODEL_ASHKIN_TELLER2D, MODEL_ISING2D, RNG_PHILOX, RNG_REPLAY, MATCH_DERIVATIVE, MATCH_REFERENCE,
                     concatenate_windows, generate_fields, instance_key)


def build(force: bool = False, verbose: bool = False):
    """Compile the CUDA engine for sm_103a (in-tree) and return the library path."""
    return _build_native(force=force, verbose=verbose)


__all__ = ["Batch", "Engine", "Instance", "REWLError", "Status", "build", "load_library", "LIBRARY_PATH",
           "MODEL_ISING2D", "MODEL_ASHKIN_TELLER2D", "FLAT_MIN_OVER_MEAN", "FLAT_MAX_MIN_RATIO", "FLAT_ALL_VISITED",
           "MASK_STATIC", "MASK_VISITED", "RNG_PHILOX", "RNG_REPLAY", "DISORDER_GAUSSIAN", "DISORDER_UNIFORM",
           "generate_fields", "concatenate_windows", "instance_key", "MATCH_DERIVATIVE", "MATCH_REFERENCE"]
