"""GB300-native (sm_103a) fit-and-render path of SAD (Soft Anisotropic Diagrams).

The compute lives in libsad_gb300.so (hand-written CUDA kernels behind the C ABI of
include/sad_gb300.h).  This package is the host-side mirror of the reference's Python
interface: `ops` / `torch.ops.sad` (tensor ops), `SADRenderFunction` / `SADRenderer` /
`CandidateUpdater` (autograd render and candidate search), and `Trainer` / `fit` (whole
fits on the device).
"""
from . import _lib, build  # noqa: F401

__version__ = "1.0.0"


def _lazy_torch():
    from . import modules, ops  # noqa: F401  (importing ops registers torch.ops.sad)
    return modules


def __getattr__(name):
    if name in ("SADRenderFunction", "SADRenderer", "CandidateUpdater"):
        return getattr(_lazy_torch(), name)
    if name in ("ops", "modules", "torch_ops"):
        import importlib
        mod = importlib.import_module(f".{name}", __name__)
        if name != "torch_ops":
            _lazy_torch()
        return mod
    if name in ("Trainer", "fit"):
        from . import trainer
        return getattr(trainer, name)
    raise AttributeError(name)


__all__ = ["SADRenderFunction", "SADRenderer", "CandidateUpdater", "Trainer", "fit", "ops"]
