"""GB300-native engine for the meteor-trail FDTD scattering path.

Drop-in for the time-stepping core of fatemedk/meteorscattering
(``source/meteor-2.1.cpp`` / ``source/meteor-fork.cpp``): it reads the same
run-directory inputs and writes the same outputs, with the time loop on one
GPU through hand-written sm_103a kernels behind the C ABI of
``include/mfdtd.h``.
"""
from . import rundir  # noqa: F401  (pure-Python file formats)

__all__ = ["rundir", "engine", "build"]


def __getattr__(name):
    if name in ("engine", "build"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
