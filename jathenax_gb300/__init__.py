"""GB300-native (sm_103a) per-RK-stage isothermal hydro right-hand side.

A drop-in for the operator API of JathenAX (jathenax/__init__.py,
fluxes.py, hydro.py, forcing.py, run.py): the same functions and selectors,
running hand-written CUDA kernels from libjx.so through a C ABI.
"""

from .fluxes import flux_divergence, stress_face_fluxes
from .hydro import RK_STAGES, rk_stage

__all__ = ["RK_STAGES", "rk_stage", "stress_face_fluxes", "flux_divergence"]
