"""amps_gb300: GB300 (sm_103a) implementation of the AMPS particle / ECSIM hot path.

The compute lives in libamps_gpu.so (hand-written CUDA behind a C ABI,
include/amps_gpu.h); this package binds it and mirrors the reference call
surfaces (PIC::Mover, PIC::ParticleBuffer, ECSIM) for Python callers.
"""
from ._capi import AmpsGpuError, load  # noqa: F401
from .ecsim import (  # noqa: F401
    WORKLOADS,
    PRECOND_SHAPES,
    EcsimContext,
    PinnedArrays,
    PeriodicMesh,
    Species,
    Workload,
    block_origins,
    electron_proton_plasma,
    init_precond_weights,
    initial_fields,
    make_initial_condition,
    physical_positions,
    trace_dipole,
)

__all__ = [
    "AmpsGpuError", "load", "WORKLOADS", "EcsimContext", "PeriodicMesh", "Species", "Workload",
    "block_origins", "electron_proton_plasma", "initial_fields", "make_initial_condition",
    "PRECOND_SHAPES", "init_precond_weights", "PinnedArrays",
    "physical_positions", "trace_dipole",
]
