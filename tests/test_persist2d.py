"""The persistent form of small 2-D grids (GPU required): one cooperative launch runs
several steps with grid barriers between the passes.

Gates: the barrier reports a wait that runs out (a missing arrival that nothing supplies)
as CHIML_E_TIMEOUT and leaves the device usable; eligible 2-D golden cases pick the form;
its outputs are byte-identical to the launch-per-kernel form's in FP64 and in the split
form, for step counts that do and do not end on a DFT fold."""
import filecmp
import os

import pytest

from conftest import GOLDEN, stage_inputs

pytestmark = pytest.mark.gpu

ELIGIBLE = ["c1_small", "shapes_2d", "src_oblique_2d"]


def _run(case, out_dir, precision, persistent, chunks=None):
    from chiml_gb300 import Simulation
    old = os.environ.get("CHIML_PERSIST2D")
    os.environ["CHIML_PERSIST2D"] = "1" if persistent else "0"
    try:
        stage_inputs(case, out_dir)
        sim = Simulation(os.path.join(GOLDEN, case, "in.json"), precision=precision, steps_per_graph=8, out_dir=str(out_dir))
    finally:
        if old is None:
            del os.environ["CHIML_PERSIST2D"]
        else:
            os.environ["CHIML_PERSIST2D"] = old
    try:
        used = sim.stats().persistent
        for n in chunks or []:
            sim.step(n)
        sim.step()
        sim.finalize()
    finally:
        sim.close()
    return used


def _same_tree(a, b):
    files = []
    for d, _, fs in os.walk(a):
        for f in fs:
            rel = os.path.relpath(os.path.join(d, f), a)
            if rel.endswith(".json"):
                continue
            files.append(rel)
    assert files
    for rel in files:
        assert filecmp.cmp(os.path.join(a, rel), os.path.join(b, rel), shallow=False), rel


def test_barrier_completes_and_times_out(built_engine):
    from chiml_gb300.api import barrier_selftest
    assert barrier_selftest(blocks=16, missing=0, limit_seconds=0.5) == 0
    assert barrier_selftest(blocks=16, missing=1, limit_seconds=0.2) == 6  # CHIML_E_TIMEOUT
    assert barrier_selftest(blocks=1, missing=3, limit_seconds=0.05) == 6
    # the device is usable afterwards
    assert barrier_selftest(blocks=4, missing=0, limit_seconds=0.5) == 0


@pytest.mark.parametrize("case", ELIGIBLE)
@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_persistent_outputs_equal_launch_per_kernel(case, precision, built_engine, tmp_path):
    used = _run(case, tmp_path / "p", precision, True, chunks=[5, 1, 2])
    assert used == 1, "the case should take the persistent form"
    assert _run(case, tmp_path / "k", precision, False, chunks=[5, 1, 2]) == 0
    _same_tree(str(tmp_path / "k"), str(tmp_path / "p"))


def test_ineligible_cases_keep_the_launch_form(built_engine, tmp_path):
    # emitters (qe_tm) and a TFSF surface (freq_2d) keep one launch per kernel
    for case in ("qe_tm", "freq_2d"):
        assert _run(case, tmp_path / case, "split", True) == 0
