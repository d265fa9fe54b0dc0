"""MCAC per-step collision search and merge update on one GB300.

The native library (``_build/libmcacg.so``, C-ABI in include/mcacg.h) holds
the CUDA kernels for sm_103a and the C++ host layer; this package binds it
with ctypes and mirrors the reference's C++ interface (see ``api``).
"""
from .api import (CONTACT_DTYPE, AggregateContactInfo, AggregatList, Batch, PhysicalModel, Server,  # noqa: F401
                  calcul, device_count, init_state, resident_boxes, run_device, set_merge_grid_min,
                  synthetic_state)
from ._lib import StateBuffers  # noqa: F401
from .snapshot import Snapshot  # noqa: F401
