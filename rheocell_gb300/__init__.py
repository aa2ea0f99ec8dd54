"""GB300-native engine for RheoCell's multi-phase-field time step.

The compute path is the CUDA library built from csrc/ (C ABI in
include/rheocell_gb300.h); this package holds its Python caller, the host-side
set-up that mirrors the reference's backend construction, and the seeded
synthetic workload generator.
"""
from . import abi, generator, host  # noqa: F401

__all__ = ["abi", "generator", "host", "engine", "build"]
