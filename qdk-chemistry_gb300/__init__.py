"""GB300-native selected-CI / CASCI core with the interfaces of qdk-chemistry's MACIS path.

The compute path is ``libqdkgb.so`` (hand-written sm_103a CUDA kernels behind a
C ABI, declared in ``include/qdkgb.h``).  This Python package is the binding
side: ctypes calls into that library, the qdk-style ``MultiConfigurationCalculator``
mirror (``create("multi_configuration_calculator", "gb300_cas")``), the
``davidson_solver`` entry point and a ``torch.autograd.Function`` whose
backward returns the RDMs as integral gradients.
"""
from . import determinants, integrals  # noqa: F401

__all__ = ["determinants", "integrals"]


def __getattr__(name):
    # heavy submodules load the CUDA library lazily
    import importlib

    if name in ("capi", "calculators", "autograd", "build"):
        mod = importlib.import_module("." + name, __name__)
        globals()[name] = mod
        return mod
    raise AttributeError(name)
