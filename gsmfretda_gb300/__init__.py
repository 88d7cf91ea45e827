"""gsmfretda_gb300 — GB300-native (sm_103a) photon-burst Monte-Carlo PDA.

The compute path is libgpda.so (hand-written CUDA + C++ host engine behind the
C ABI in include/gpda.h). This package holds its build script, the ctypes
binding, the reference-shaped host API (mc, gpuWorker/streamWorker flow) and
the seeded synthetic workloads.
"""
from ._lib import (GPDA_OK, MODE_OCCUPANCY, MODE_PHOTON, GpdaError, GpdaModel,  # noqa: F401
                   LIB_PATH, default_model, load)

__version__ = "0.1.0"
