"""odegpu: ODE 0.12's contact generation + dWorldQuickStep on GB300.

The compute path is libodegpu.so (hand-written CUDA for sm_103a behind a C ABI,
see include/odegpu.h and include/ode_gpu.h). This package is the Python face:
scene construction (``scene``), the batched stepping API (``batch``) and the
differentiable rollout (``adjoint``).
"""
from . import scene  # noqa: F401
from ._lib import lib, LibraryMissing, build  # noqa: F401
