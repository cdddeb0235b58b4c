"""sphexa_gb300: GB300-native (sm_103a) single-rank SPH hydro sweep.

The compute path is libsphgb.so (CUDA kernels behind the C ABI in include/sphgb.h); this
package holds its build script, the ctypes mirror of the ABI, the host-side mirror of the
reference's interface (sph.py) and the seeded synthetic workloads.
"""

from . import workloads  # noqa: F401

__all__ = ["workloads", "sph", "build"]


def build(verbose: bool = False):
    from .build import build as _b
    return _b(verbose=verbose)
