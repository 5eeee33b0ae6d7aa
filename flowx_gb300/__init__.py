"""GB300-native (sm_103a) Position Based Fluids substep of Flow-X.

Hand-written CUDA kernels behind a C ABI (include/flowx.h, libflowx.so), with
a Python host mirror of the reference's solver/sph.py (``flowx_gb300.sph``).
"""

from .config import SolverConfig, push_constant_values, resolve_config  # noqa: F401

__all__ = ["SolverConfig", "push_constant_values", "resolve_config"]
