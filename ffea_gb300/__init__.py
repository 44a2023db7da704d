"""ffea_gb300 -- FFEA's per-timestep blob update on GB300 (sm_103a).

The compute path is libffea_gb300.so (CUDA + C++ behind the C ABI of
include/ffea_gpu.h); this package holds its Python binding (``world``), the
host-side input handling (``params``, ``formats``, ``mesh``) and the build
recipe (``build``).
"""
from .params import SimulationParams, PRECISION_FP64, PRECISION_MIXED, SOLVER_MASS, SOLVER_NOMASS  # noqa: F401

__version__ = "0.1.0"
