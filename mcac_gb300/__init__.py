"""MCAC per-step collision search and merge update on one GB300.

The native library (``_build/libmcacg.so``, C-ABI in include/mcacg.h) holds
the CUDA kernels for sm_103a and the C++ host layer; this package binds it
with ctypes and mirrors the reference's C++ interface (see ``api``).
"""
from .api import (AggregateContactInfo, AggregatList, Batch, PhysicalModel, Server, calcul, device_count,  # noqa: F401
                  init_state, run_device)
from .snapshot import Snapshot  # noqa: F401
