"""prestige_gb300: GB300-native (sm_103a) particle hot path of dineshadepu/prestige.

Layers
  include/prestige_gpu.h   the C ABI (extern "C"), the drop-in boundary
  csrc/                    CUDA kernels: neighbour search, SPH, DEM, batched step, adjoint
  _native / system         ctypes binding and the named-slice handle above it
  equations                the reference's #[equation] / EquationIR / fuse / codegen front end,
                           with a GPU executor for the fused gather
  workloads                seeded synthetic inputs
The CUDA library is required: nothing here falls back to the CPU.
"""
from . import build_lib  # noqa: F401
from ._native import PgError, load  # noqa: F401
from .system import ParticleSystem, config_dict, make_config  # noqa: F401

__all__ = ["ParticleSystem", "make_config", "config_dict", "PgError", "load", "build_lib"]
