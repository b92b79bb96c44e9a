"""GB300-native WCSPH solver step, a drop-in for the RRSPH_OMP time loop.

The compute path is librrsph_cuda.so (hand-written sm_103a CUDA behind the C
ABI of include/rrsph_cuda.h); this package is the Python host over that ABI.
"""

from .capi import RrsphError, RrsphParams  # noqa: F401
from .solver import (  # noqa: F401
    Solver,
    default_params,
    derive,
    load_params,
    params_from_json,
    read_layer,
    write_layer,
)

__all__ = [
    "RrsphError",
    "RrsphParams",
    "Solver",
    "default_params",
    "derive",
    "load_params",
    "params_from_json",
    "read_layer",
    "write_layer",
]
