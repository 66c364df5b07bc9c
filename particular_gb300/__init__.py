"""particular_gb300: GB300-native (sm_103a) compute methods for particular's acceleration path.

The compute happens in libparticular_cuda.so (C ABI: include/particular_cuda.h);
this package is the host-side mirror of particular's API around it.
"""
from .gravity import Acceleration, AccelerationSoftened, GravitationalField, fields, positions
from .storage import Between, Ordered, Reordered, as_between
from . import cuda
from .cuda import CudaResources, cuda_barnes_hut, cuda_brute_force
from ._native import CudaError

__all__ = [
    "Acceleration", "AccelerationSoftened", "GravitationalField", "fields", "positions",
    "Between", "Ordered", "Reordered", "as_between", "cuda", "CudaResources",
    "cuda_brute_force", "cuda_barnes_hut", "CudaError",
]
