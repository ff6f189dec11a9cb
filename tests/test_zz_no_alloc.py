"""chiml_get_box_noalloc: the box read-back that allocates nothing, through the C ABI,
against chiml_get_field on the same handle.

Two calls in a row on one handle, with steps between them and a smaller second box,
so that the second call runs on an array that still holds the first call's values; and
the device's free memory, read through the driver, unchanged by a series of calls.
Collected last so that it runs both after the other GPU tests and alone.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative L2, the FP64 parity tolerance of the GPU tests


def _rel_l2(a, b):
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


def _slice(full, origin, shape):
    x0, y0, z0 = origin
    nx, ny, nz = shape
    return full[y0:y0 + ny, z0:z0 + nz, x0:x0 + nx]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_box_noalloc_matches_get_field(built_engine, tmp_path, precision):
    from chiml_gb300 import Simulation
    sim = Simulation(os.path.join(GOLDEN, "c2_small", "in.json"), precision=precision, out_dir=str(tmp_path))
    try:
        s = sim.stats()
        lx, ly = s.nx + 2, s.ny + 2
        lz = s.cells // (lx * ly)
        calls = [
            (7, "Ex", (0, 0, 0), (lx, ly, lz)),   # the whole component, halo included
            (5, "Hy", (3, 5, 2), (9, 4, 6)),      # a smaller, offset box of another component
        ]
        for nsteps, name, origin, shape in calls:
            sim.step(nsteps)
            ref = _slice(sim.field(name), origin, shape)
            out = np.full(shape[0] * shape[1] * shape[2], np.nan)
            got = sim.box_noalloc(name, origin, shape, out=out)
            assert got.shape == ref.shape
            assert np.isfinite(got).all()
            assert np.abs(ref).max() > 0
            assert _rel_l2(got, ref) <= TOL
    finally:
        sim.close()


def test_box_noalloc_rejects_bad_boxes(built_engine, tmp_path):
    """A 2-D TMz grid of 1032 x 1032 local cells: larger than the fixed array, no Ex field."""
    from chiml_gb300 import ChimlError, Simulation, configs
    from chiml_gb300.api import BOX_NOALLOC_MAX_CELLS
    cfg = configs.config1(n=1030, pml=10, steps=4, radius_cells=40, src_gap_cells=20, ndtc=1, nfreq=3)
    path = configs.write_json(cfg, str(tmp_path / "in.json"))
    sim = Simulation(path, precision="fp64", out_dir=str(tmp_path))
    try:
        s = sim.stats()
        lx, ly = s.nx + 2, s.ny + 2
        assert lx * ly > BOX_NOALLOC_MAX_CELLS
        sim.step(2)
        with pytest.raises(ChimlError, match="exceeds the limit of 1048576 cells"):
            sim.box_noalloc("Ez", (0, 0, 0), (lx, ly, 1))
        with pytest.raises(ChimlError, match="outside the local grid"):
            sim.box_noalloc("Ez", (1, 0, 0), (lx, 1, 1))
        with pytest.raises(ChimlError, match="field not present"):
            sim.box_noalloc("Ex", (0, 0, 0), (1, 1, 1))
        # the largest box that fits still reads correctly after the rejected calls
        rows = BOX_NOALLOC_MAX_CELLS // lx
        got = sim.box_noalloc("Ez", (0, 0, 0), (lx, rows, 1))
        ref = _slice(sim.field("Ez"), (0, 0, 0), (lx, rows, 1))
        assert _rel_l2(got, ref) <= TOL
    finally:
        sim.close()


def _device_free_bytes(device=0):
    """Free memory of the device as the driver reports it (cuMemGetInfo in the device's
    primary context, the context the engine's runtime calls use)."""
    cuda = ctypes.CDLL("libcuda.so.1")
    assert cuda.cuInit(0) == 0
    dev = ctypes.c_int()
    assert cuda.cuDeviceGet(ctypes.byref(dev), device) == 0
    ctx = ctypes.c_void_p()
    assert cuda.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev) == 0
    try:
        assert cuda.cuCtxPushCurrent_v2(ctx) == 0
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        rc = cuda.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total))
        cuda.cuCtxPopCurrent_v2(ctypes.byref(ctypes.c_void_p()))
        assert rc == 0
        return free.value
    finally:
        cuda.cuDevicePrimaryCtxRelease_v2(dev)


def test_box_noalloc_allocates_nothing(built_engine, tmp_path):
    """Free device memory after the handle is created and stepped equals free memory after
    several reads, the largest allowed box among them."""
    from chiml_gb300 import Simulation
    from chiml_gb300.api import BOX_NOALLOC_MAX_CELLS
    sim = Simulation(os.path.join(GOLDEN, "c2_small", "in.json"), precision="split", out_dir=str(tmp_path))
    try:
        s = sim.stats()
        lx, ly = s.nx + 2, s.ny + 2
        lz = s.cells // (lx * ly)
        sim.step(3)
        sim.sync()
        before = _device_free_bytes()
        rows = min(ly, BOX_NOALLOC_MAX_CELLS // (lx * lz))
        boxes = [("Ez", (0, 0, 0), (lx, rows, lz)), ("Hx", (1, 2, 3), (4, 5, 6)), ("Ey", (0, 0, 0), (lx, 1, lz))]
        got = [sim.box_noalloc(name, origin, shape) for name, origin, shape in boxes]
        after = _device_free_bytes()
        assert after == before, "free device memory changed by %d bytes" % (before - after)
        for (name, origin, shape), g in zip(boxes, got):
            assert _rel_l2(g, _slice(sim.field(name), origin, shape)) <= TOL
    finally:
        sim.close()
