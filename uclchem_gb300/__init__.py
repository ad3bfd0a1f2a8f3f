"""uclchem_gb300: UCLCHEM's chemistry integration hot path on one GB300.

Batched rate coefficients, flux-form GETYDOT, analytic Jacobian and a
DVODE-logic BDF integrator with an FP64 or mixed-precision (FP32 LU) Newton
solve, behind the C ABI in include/uclchem_gb300.h.  Submodules: network
(MakeRates table compiler), params, model (uclchem.model-style front end),
build (in-tree nvcc build), _lib (ctypes binding).
"""
from . import network, params  # noqa: F401
