"""ember_gb300 -- GB300 (sm_103a) implementation of Ember's split-step hot path.

The compute path is libember_gpu.so (hand-written FP64 CUDA kernels behind the
C ABI of include/ember_gpu.h); this package is the host-side mirror of the
reference's stage interfaces, for Python callers and tests:

  mechanism   Mechanism tables and the seeded synthetic mechanism
  source      GpuMechanism, integrate_production_terms (QSS / BDF), autotune,
              tuning, source_adjoint
  diffusion   integrate_diffusion_terms, TridiagonalIntegratorBatch,
              diffusion_adjoint
  transport   GpuTransport (thermo and "Approx" transport), synthetic fits
  split       FlameBatchSplitSolver (whole split steps of many flames)
  autograd    split_step_objectives (torch.autograd.Function)
  roofline    algorithmic work model of the kernels
"""
from ._lib import EmberGpuError, library_path  # noqa: F401
from . import _lib  # noqa: F401

__version__ = "0.1.0"


def device_count() -> int:
    return _lib.lib().ember_device_count()
