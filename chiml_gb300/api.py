"""ctypes binding of include/chiml_gpu.h."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libchiml_gb300.so")

PREC_FP64 = 0
PREC_SPLIT = 1
COMPONENTS = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5, "Dx": 6, "Dy": 7, "Dz": 8}
_STATUS = {
    0: "CHIML_OK",
    1: "CHIML_E_INPUT",
    2: "CHIML_E_UNSUPPORTED",
    3: "CHIML_E_CUDA",
    4: "CHIML_E_OOM",
    5: "CHIML_E_NUMERIC",
    6: "CHIML_E_TIMEOUT",
    7: "CHIML_E_STATE",
}


class ChimlError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (_STATUS.get(status, status), message))
        self.status = status


class _Options(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("device", ctypes.c_int),
        ("steps_per_graph", ctypes.c_int),
        ("out_dir", ctypes.c_char_p),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("cells", ctypes.c_int64),
        ("cells_physical", ctypes.c_int64),
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("steps_total", ctypes.c_int32),
        ("steps_done", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("bytes_per_cell_update", ctypes.c_double),
        ("device_bytes", ctypes.c_double),
        ("kernels_per_step", ctypes.c_int32),
        ("persistent", ctypes.c_int32),
        ("bytes_h_pass", ctypes.c_double),
        ("bytes_e_pass", ctypes.c_double),
        ("bytes_dft", ctypes.c_double),
        ("h2d_bytes", ctypes.c_double),
        ("d2h_bytes", ctypes.c_double),
        ("n_flux_regions", ctypes.c_int32),
        ("n_emitters", ctypes.c_int32),
        ("n_tfsf", ctypes.c_int32),
        ("reserved2", ctypes.c_int32),
        ("seconds_plan", ctypes.c_double),
        ("seconds_upload", ctypes.c_double),
        ("seconds_finalize", ctypes.c_double),
    ]


_lib = None

EXPORTED = [
    "chiml_create",
    "chiml_step",
    "chiml_sync",
    "chiml_finalize",
    "chiml_destroy",
    "chiml_last_error",
    "chiml_query",
    "chiml_get_field",
    "chiml_stream",
    "chiml_profile_steps",
    "chiml_get_box_noalloc",
    "chiml_batch_create",
    "chiml_batch_step",
    "chiml_batch_run",
    "chiml_batch_finalize",
    "chiml_batch_member",
    "chiml_batch_destroy",
    "chiml_barrier_selftest",
]

BOX_NOALLOC_MAX_CELLS = 1048576


def load_library(path=None):
    """Loads the engine library; raises FileNotFoundError when it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError("chiml_gb300 engine library not built: %s (run __graft_entry__.build())" % p)
    lib = ctypes.CDLL(p)
    lib.chiml_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(_Options), ctypes.POINTER(ctypes.c_void_p)]
    lib.chiml_create.restype = ctypes.c_int
    lib.chiml_step.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    lib.chiml_step.restype = ctypes.c_int
    lib.chiml_sync.argtypes = [ctypes.c_void_p]
    lib.chiml_sync.restype = ctypes.c_int
    lib.chiml_finalize.argtypes = [ctypes.c_void_p]
    lib.chiml_finalize.restype = ctypes.c_int
    lib.chiml_destroy.argtypes = [ctypes.c_void_p]
    lib.chiml_destroy.restype = None
    lib.chiml_last_error.argtypes = [ctypes.c_void_p]
    lib.chiml_last_error.restype = ctypes.c_char_p
    lib.chiml_query.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
    lib.chiml_query.restype = ctypes.c_int
    lib.chiml_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.chiml_get_field.restype = ctypes.c_int
    lib.chiml_stream.argtypes = [ctypes.c_void_p]
    lib.chiml_stream.restype = ctypes.c_void_p
    lib.chiml_profile_steps.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int)]
    lib.chiml_profile_steps.restype = ctypes.c_int
    lib.chiml_get_box_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int32),
                                          ctypes.POINTER(ctypes.c_double)]
    lib.chiml_get_box_noalloc.restype = ctypes.c_int
    lib.chiml_batch_create.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.POINTER(_Options),
                                       ctypes.POINTER(ctypes.c_void_p)]
    lib.chiml_batch_create.restype = ctypes.c_int
    lib.chiml_batch_step.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    lib.chiml_batch_step.restype = ctypes.c_int
    lib.chiml_batch_run.argtypes = [ctypes.c_void_p]
    lib.chiml_batch_run.restype = ctypes.c_int
    lib.chiml_batch_finalize.argtypes = [ctypes.c_void_p]
    lib.chiml_batch_finalize.restype = ctypes.c_int
    lib.chiml_batch_member.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.chiml_batch_member.restype = ctypes.c_void_p
    lib.chiml_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.chiml_batch_destroy.restype = None
    lib.chiml_barrier_selftest.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    lib.chiml_barrier_selftest.restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


def barrier_selftest(device=0, blocks=8, missing=0, limit_seconds=0.2):
    """Runs the persistent step's grid barrier alone (chiml_barrier_selftest); returns the
    status code: 0 when every block arrived, 6 (CHIML_E_TIMEOUT) when the wait gave up."""
    lib = load_library()
    st = lib.chiml_barrier_selftest(int(device), int(blocks), int(missing), float(limit_seconds))
    if st not in (0, 6):
        raise ChimlError(st, lib.chiml_last_error(None).decode())
    return st


class Simulation:
    """One simulation on one GPU, driven like chiML's main loop."""

    def __init__(self, json_path, precision="fp64", device=0, steps_per_graph=0, out_dir=None):
        self._lib = load_library()
        self._h = ctypes.c_void_p()
        prec = {"fp64": PREC_FP64, "split": PREC_SPLIT}[precision]
        self._out_dir = out_dir
        opt = _Options(prec, device, steps_per_graph, out_dir.encode() if out_dir else None)
        st = self._lib.chiml_create(os.fsencode(json_path), ctypes.byref(opt), ctypes.byref(self._h))
        if st != 0:
            raise ChimlError(st, self._lib.chiml_last_error(None).decode())

    def _check(self, st):
        if st != 0:
            raise ChimlError(st, self._lib.chiml_last_error(self._h).decode())

    def step(self, n=None):
        """Advances n steps (all remaining when n is None)."""
        if n is None:
            s = self.stats()
            n = s.steps_total - s.steps_done
        self._check(self._lib.chiml_step(self._h, int(n)))

    def sync(self):
        self._check(self._lib.chiml_sync(self._h))

    def finalize(self):
        self._check(self._lib.chiml_finalize(self._h))

    def stats(self):
        s = Stats()
        self._check(self._lib.chiml_query(self._h, ctypes.byref(s)))
        return s

    def field(self, name):
        """Returns a field as an FP64 array shaped (y, z, x) (chiML's local layout, halo included)."""
        s = self.stats()
        lx, ly = s.nx + 2, s.ny + 2
        lz = s.cells // (lx * ly)
        out = np.empty(s.cells, dtype=np.float64)
        self._check(self._lib.chiml_get_field(self._h, COMPONENTS[name], out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out.reshape(ly, lz, lx)

    def box_noalloc(self, name, origin, shape, out=None):
        """Reads the box at origin (x0, y0, z0) of shape (nx, ny, nz) of one field as an FP64 array
        shaped (ny, nz, nx), through the engine's fixed device array (no device allocation).
        A caller-provided `out` (C-contiguous float64, nx*ny*nz values) is filled and returned."""
        nx, ny, nz = (int(v) for v in shape)
        if out is None:
            out = np.empty(nx * ny * nz, dtype=np.float64)
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != nx * ny * nz:
            raise ValueError("out must be a C-contiguous float64 array of nx*ny*nz values")
        box = (ctypes.c_int32 * 6)(int(origin[0]), int(origin[1]), int(origin[2]), nx, ny, nz)
        self._check(self._lib.chiml_get_box_noalloc(self._h, COMPONENTS[name], box,
                                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out.reshape(ny, nz, nx)

    def profile_steps(self, n):
        """Runs n steps with per-kernel CUDA-event timing; returns {slot name: total ms}."""
        ms = (ctypes.c_double * 64)()
        ns = ctypes.c_int()
        self._check(self._lib.chiml_profile_steps(self._h, int(n), ms, 64, ctypes.byref(ns)))
        names = ["h_pass", "sources", "e_pass", "step_counter", "records"]
        st = self.stats()
        ndft, nem = st.n_flux_regions, st.n_emitters
        out = {}
        for k in range(ns.value):
            if k < len(names):
                out[names[k]] = ms[k]
            elif k < len(names) + 2 * ndft:
                q, r = divmod(k - len(names), 2)
                out["dft%d_%s" % (q, "sample" if r == 0 else "fold")] = ms[k]
            elif k < len(names) + 2 * ndft + nem:
                out["emitter%d" % (k - len(names) - 2 * ndft)] = ms[k]
            else:
                out["tfsf%d" % (k - len(names) - 2 * ndft - nem)] = ms[k]
        return out

    @property
    def stream(self):
        return self._lib.chiml_stream(self._h)

    def close(self):
        if self._h:
            self._lib.chiml_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Independent simulations stepped together (chiml_batch_*): a parameter sweep."""

    def __init__(self, json_paths, precision="fp64", device=0, steps_per_graph=20, out_dir=None):
        """Members write their outputs under out_dir, or beside their own input files when it is None."""
        self._lib = load_library()
        self._h = ctypes.c_void_p()
        prec = {"fp64": PREC_FP64, "split": PREC_SPLIT}[precision]
        opt = _Options(prec, device, steps_per_graph, out_dir.encode() if out_dir else None)
        arr = (ctypes.c_char_p * len(json_paths))(*[os.fsencode(p) for p in json_paths])
        st = self._lib.chiml_batch_create(arr, len(json_paths), ctypes.byref(opt), ctypes.byref(self._h))
        if st != 0:
            raise ChimlError(st, self._lib.chiml_last_error(None).decode())
        self.n = len(json_paths)

    def _check(self, st):
        if st != 0:
            why = "batch call failed"
            for i in range(self.n):
                h = self._lib.chiml_batch_member(self._h, i)
                msg = self._lib.chiml_last_error(ctypes.c_void_p(h)).decode()
                if msg:
                    why = "member %d: %s" % (i, msg)
            raise ChimlError(st, why)

    def step(self, n):
        """Advances every unfinished member by n steps (each stops at its last) and waits."""
        self._check(self._lib.chiml_batch_step(self._h, int(n)))

    def run(self):
        """Advances every member to its last step and waits."""
        self._check(self._lib.chiml_batch_run(self._h))

    def finalize(self):
        self._check(self._lib.chiml_batch_finalize(self._h))

    def member_stats(self, i):
        h = self._lib.chiml_batch_member(self._h, i)
        if not h:
            raise IndexError(i)
        s = Stats()
        st = self._lib.chiml_query(ctypes.c_void_p(h), ctypes.byref(s))
        if st != 0:
            raise ChimlError(st, "query failed")
        return s

    def close(self):
        if self._h:
            self._lib.chiml_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
