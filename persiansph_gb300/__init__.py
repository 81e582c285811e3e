"""persiansph-gb300: PersianSPH's per-step hot path on one GB300 (sm_103a).

The Domain API (persiansph_gb300.domain) mirrors SPH::Domain; Solve runs the
per-step loop through the C ABI (include/psph.h) on hand-written CUDA kernels
(persiansph_gb300/csrc). There is no CPU fallback: the solver raises if the
CUDA library is missing.
"""
from .domain import (Domain, Fatal, Morris, Multiplied_density, Qubic_Spline, Quintic, Quintic_Spline, Shao,
                     Squared_density, Takeda, Incompressible_Full)
from .particles import ParticleSet

__all__ = ["Domain", "Fatal", "ParticleSet", "Qubic_Spline", "Quintic", "Quintic_Spline", "Morris", "Shao",
           "Incompressible_Full", "Takeda", "Squared_density", "Multiplied_density"]
