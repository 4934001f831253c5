"""GB300 (sm_103a) rVPM particle-field evaluation: the UJ_direct / SFS / RK3
hot path that FLOWUnsteady drives through FLOWVPM, as CUDA kernels behind a C
ABI (libvpmgpu.so, include/vpm_gpu.h) with a FLOWVPM-shaped Python host API."""
from . import _lib  # noqa: F401

__all__ = ["vpm", "batch", "_lib"]
