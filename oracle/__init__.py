"""CPU FP64 oracle of chiML's time-step loop: test infrastructure only.

ctypes binding of oracle/_build/libchiml_oracle.so (built from chiml_oracle.cpp
by chiml_gb300/build.py). Used by tests, the smoke check and the CPU-baseline
leg of the benchmark; the product path never imports it.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libchiml_oracle.so")
REF_BIN = os.path.join(_HERE, "_ref", "chiml_ref")
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError("oracle library not built: " + LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        lib.chiml_oracle_create.argtypes = [ctypes.c_char_p]
        lib.chiml_oracle_create.restype = ctypes.c_void_p
        lib.chiml_oracle_last_error.restype = ctypes.c_char_p
        lib.chiml_oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.chiml_oracle_step.restype = ctypes.c_int
        lib.chiml_oracle_steps_total.argtypes = [ctypes.c_void_p]
        lib.chiml_oracle_steps_total.restype = ctypes.c_int
        lib.chiml_oracle_cells.argtypes = [ctypes.c_void_p]
        lib.chiml_oracle_cells.restype = ctypes.c_longlong
        lib.chiml_oracle_dims.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        lib.chiml_oracle_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.chiml_oracle_get_field.restype = ctypes.c_int
        lib.chiml_oracle_finalize.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        lib.chiml_oracle_finalize.restype = ctypes.c_int
        lib.chiml_oracle_destroy.argtypes = [ctypes.c_void_p]
        lib.chiml_oracle_run.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        lib.chiml_oracle_run.restype = ctypes.c_double
        lib.chiml_oracle_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


COMPONENTS = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5, "Dx": 6, "Dy": 7, "Dz": 8}


class OracleSim:
    def __init__(self, json_path):
        self._lib = load()
        self._h = self._lib.chiml_oracle_create(os.fsencode(json_path))
        if not self._h:
            raise RuntimeError(self._lib.chiml_oracle_last_error().decode())

    @property
    def steps_total(self):
        return self._lib.chiml_oracle_steps_total(self._h)

    def dims(self):
        d = (ctypes.c_int * 6)()
        self._lib.chiml_oracle_dims(self._h, d)
        return tuple(d)

    def step(self, n):
        return self._lib.chiml_oracle_step(self._h, int(n))

    def cells_physical(self):
        d = self.dims()
        return d[3] * d[4] * d[5]

    def field(self, name):
        lx, ly, lz = self.dims()[:3]
        out = np.empty(lx * ly * lz, dtype=np.float64)
        rc = self._lib.chiml_oracle_get_field(self._h, COMPONENTS[name], out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if rc != 0:
            raise KeyError(name)
        return out.reshape(ly, lz, lx)

    def finalize(self, out_dir):
        if self._lib.chiml_oracle_finalize(self._h, os.fsencode(out_dir)) != 0:
            raise RuntimeError(self._lib.chiml_oracle_last_error().decode())

    def close(self):
        if self._h:
            self._lib.chiml_oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def threads():
    return load().chiml_oracle_threads()


def run(json_path, out_dir, steps=-1):
    """Runs a whole simulation and writes its outputs; returns the step-loop wall seconds."""
    t = load().chiml_oracle_run(os.fsencode(json_path), os.fsencode(out_dir), int(steps))
    if t < 0:
        raise RuntimeError(load().chiml_oracle_last_error().decode())
    return t
