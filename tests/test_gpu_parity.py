"""CUDA path against the reference outputs and the oracle (GPU required).

Every comparison goes through the C ABI (chiml_create / chiml_step /
chiml_finalize / chiml_get_field). FP64 runs are held to the parity bar,
relative L2 <= 1e-10 (summation order only); the FP32/FP64-split form to the
flux-spectrum target of 1e-4 and a field tolerance of 1e-4.
"""
import os
import shutil

import numpy as np
import pytest

from compare import compare_dirs, rel_l2
from conftest import GOLDEN, golden_cases, stage_inputs

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_SPLIT = 1e-4


def _run_gpu(case, out_dir, precision="fp64", graph=0):
    from chiml_gb300 import Simulation
    stage_inputs(case, out_dir)
    sim = Simulation(os.path.join(GOLDEN, case, "in.json"), precision=precision, steps_per_graph=graph, out_dir=str(out_dir))
    sim.step()
    sim.finalize()
    return sim


@pytest.mark.parametrize("case", golden_cases())
def test_fp64_matches_reference_outputs(case, built_engine, tmp_path):
    sim = _run_gpu(case, tmp_path)
    assert sim.stats().steps_done == sim.stats().steps_total
    compare_dirs(os.path.join(GOLDEN, case, "ref"), str(tmp_path), TOL_FP64)


@pytest.mark.parametrize("case", golden_cases())
def test_fp64_fields_match_oracle_midrun(case, built_engine, built_oracle):
    import oracle
    from chiml_gb300 import Simulation
    path = os.path.join(GOLDEN, case, "in.json")
    orc = oracle.OracleSim(path)
    sim = Simulation(path)
    n = orc.steps_total // 2
    orc.step(n)
    sim.step(n)
    checked = 0
    for name in ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz", "Dx", "Dy", "Dz"]:
        try:
            ref = orc.field(name)
        except KeyError:
            continue
        got = sim.field(name)
        assert got.shape == ref.shape
        e = rel_l2(ref, got)
        assert e <= TOL_FP64, "%s %s rel L2 %.3e" % (case, name, e)
        checked += 1
    assert checked >= 3


@pytest.mark.parametrize("case", ["c2_small", "qe_3d", "tfsf_oblique"])
def test_graph_replay_equals_eager_launches(case, built_engine, tmp_path):
    a = tmp_path / "eager"
    b = tmp_path / "graph"
    _run_gpu(case, a, graph=0)
    _run_gpu(case, b, graph=16)
    for d, _, files in os.walk(a):
        for f in files:
            pa = os.path.join(d, f)
            pb = os.path.join(b, os.path.relpath(pa, a))
            assert open(pa, "rb").read() == open(pb, "rb").read(), f


@pytest.mark.parametrize("graph,chunks", [(8, [5, 3, 17, 1]), (6, [7, 12])])
def test_graph_replays_from_any_step_equal_eager_launches(graph, chunks, built_engine, tmp_path):
    """Graphs whose length is a multiple of the DFT fold period hold only the fold launches
    of replays that start on the period: steps that leave the count off the period run
    eagerly until it is back on it. A graph of 6 steps (not a multiple of 4) carries every
    step's fold launch."""
    from chiml_gb300 import Simulation
    case = "c1_small"
    a = tmp_path / "eager"
    b = tmp_path / "graph"
    _run_gpu(case, a, graph=0)
    stage_inputs(case, b)
    sim = Simulation(os.path.join(GOLDEN, case, "in.json"), precision="fp64", steps_per_graph=graph, out_dir=str(b))
    try:
        for n in chunks:
            sim.step(n)
        sim.step()
        sim.finalize()
    finally:
        sim.close()
    for d, _, files in os.walk(a):
        for f in files:
            pa = os.path.join(d, f)
            pb = os.path.join(b, os.path.relpath(pa, a))
            assert open(pa, "rb").read() == open(pb, "rb").read(), f


@pytest.mark.parametrize("case", golden_cases())
def test_split_precision_within_tolerance(case, built_engine, tmp_path):
    _run_gpu(case, tmp_path, precision="split", graph=8)
    compare_dirs(os.path.join(GOLDEN, case, "ref"), str(tmp_path), TOL_SPLIT)
