"""GB300 engine for chiML's time-step loop.

The native library (``_build/libchiml_gb300.so``) exposes the C ABI declared in
``include/chiml_gpu.h``; :class:`Simulation` is a thin ctypes mirror of how
chiML's ``main.cpp`` drives ``parallelFDTDFieldReal``: construct from the JSON
input, step ``ceil(tLim/dt)`` times, then write the flux and detector files.
There is no CPU fallback: every entry point raises if the library is missing.
"""
from .api import (  # noqa: F401
    Batch,
    ChimlError,
    Simulation,
    Stats,
    load_library,
    PREC_FP64,
    PREC_SPLIT,
    COMPONENTS,
)
