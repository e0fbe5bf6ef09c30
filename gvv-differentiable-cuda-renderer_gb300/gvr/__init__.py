"""gvr -- a GB300-native differentiable mesh rasteriser with the operator
surface of the reference CudaRenderer TensorFlow op
(python/CudaRenderer.py), over a C ABI (include/gvr.h) backed by
hand-written sm_103a CUDA kernels (csrc/)."""
from . import scenes  # noqa: F401
from ._lib import ALBEDO, SHADING, GvrError, load  # noqa: F401
from .native_build import build  # noqa: F401


def __getattr__(name):
    # torch-dependent parts are imported lazily so the scene generator and the
    # build step work without touching torch
    if name in ("CudaRendererGpu", "RendererHandle", "RenderFunction", "get_handle", "render_forward",
                "render_backward"):
        from . import renderer
        return getattr(renderer, name)
    raise AttributeError(name)
