"""cuco_gb300: GB300-native (sm_103a) PM + P3M gravity engine, a drop-in for the
force path of liulei/cuco.

The compute lives in libcuco_gb300.so (hand-written CUDA, C ABI in
include/cuco_gb300.h); this package loads it with ctypes and mirrors the
reference's interface (engine.Box).  There is no CPU fallback.
"""
from ._native import CucoError, load  # noqa: F401
from .engine import Box, BoxConfig, cosmo_factors, fixed_step_schedule, reference_split  # noqa: F401

__all__ = ["Box", "BoxConfig", "CucoError", "cosmo_factors", "fixed_step_schedule", "load",
           "reference_split"]
