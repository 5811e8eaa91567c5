"""GB300 implementation of the SWM shallow-water time-stepping hot path.

The compute path is libswm_gb300.so (hand-written CUDA for sm_103a behind the
C ABI of include/swm_gpu.h); this package only binds it (``_lib``), mirrors
the reference's host-side configuration (``host``) and offers a Python model
object (``model.GpuModel``) with the SWM/tracer/SOR entry points.
"""
from ._lib import lib, check, SwmGpuError, PATHS  # noqa: F401
