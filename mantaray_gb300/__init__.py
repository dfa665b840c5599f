"""mantaray_gb300: GB300-native (sm_103a) ray tracing of ocean surface
gravity waves, a drop-in for the hot path of mines-oceanography/mantaray.

The integration runs in libmantaray_gpu.so (hand-written CUDA kernels behind
a C ABI, include/mantaray_gpu.h).  There is no CPU fallback: importing the
tracing functions loads the library and fails loudly if it is missing.
"""

from ._native import MantarayError, MantarayIOError  # noqa: F401
from .core import (  # noqa: F401
    TraceResult,
    num_steps,
    ray_tracing,
    single_ray,
    trace,
    trace_device,
)
from .fields import Bathymetry, Current, read_netcdf3_variable  # noqa: F401

__all__ = [
    "Bathymetry",
    "Current",
    "MantarayError",
    "MantarayIOError",
    "TraceResult",
    "num_steps",
    "ray_tracing",
    "read_netcdf3_variable",
    "single_ray",
    "trace",
    "trace_device",
]
