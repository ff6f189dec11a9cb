"""The split form of the emitter update (FP32 fields; the Hermitian density update in FP32
with the state as float-float pairs) against the FP64 form, on the GPU.

Two gates: the emitter outputs (populations, polarisation) of every golden case with
emitters agree with the FP64 form's within TOL_EMIT, and over a run of 10^5 steps the
trace of the density matrices (the sum of the populations of every level) stays where it
started while the populations stay within TOL_LONG of the FP64 run. The fields are FP32 in
the split form, so part of the difference is the fields' own.
"""
import json
import os

import numpy as np
import pytest

from chiml_gb300.outfiles import read_output, relative_errors
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_EMIT = 1e-5    # relative L2 per data group of the emitter files, split vs FP64
TOL_TRACE = 1e-7   # relative drift of the summed populations over the long run (split: 1.2e-8)
TOL_LONG = 1e-5    # final populations, split vs FP64, after 10^5 steps

EMITTER_CASES = ["qe_tm", "qe_te", "qe_3d", "qe_dists_3d", "qe_dists_2d", "c5_small"]


def _run(path, precision, out_dir):
    from chiml_gb300 import Simulation
    sim = Simulation(path, precision=precision, steps_per_graph=16, out_dir=str(out_dir))
    try:
        sim.step()
        sim.finalize()
    finally:
        sim.close()


def _emitter_errors(ref_dir, out_dir):
    err = relative_errors(str(ref_dir), str(out_dir), detail=True)
    return {f: g for f, g in err.items() if "_level_" in f or "pol" in os.path.basename(f)}


@pytest.mark.parametrize("case", EMITTER_CASES)
def test_split_emitter_outputs_match_fp64(case, built_engine, tmp_path):
    path = os.path.join(GOLDEN, case, "in.json")
    _run(path, "fp64", tmp_path / "fp64")
    _run(path, "split", tmp_path / "split")
    err = _emitter_errors(tmp_path / "fp64", tmp_path / "split")
    print(case, {f: max(g.values()) for f, g in err.items()})
    assert err, "no emitter outputs"
    for f, groups in err.items():
        for g, e in groups.items():
            assert e <= TOL_EMIT, "%s %s [%s] relative L2 %.3e" % (case, f, g, e)


def test_split_emitter_long_run_keeps_trace(built_engine, tmp_path):
    """qe_3d (three levels, nine ensemble members, relaxation and dephasing) run for 10^5
    steps with its couplings at 0.3 of the golden case's: at full strength the explicit
    ABM4 step of the reference's own arithmetic (the oracle, FP64) diverges after ~3500
    steps; at 0.3 it stays finite for 10^5 steps, the populations are driven to 0.2-0.5 and
    the oracle's trace drifts by 2e-14."""
    cfg = json.load(open(os.path.join(GOLDEN, "qe_3d", "in.json")))
    dt = cfg["CompCell"]["dt"]
    cfg["CompCell"]["tLim"] = (100000 - 0.5) * dt
    emitter = cfg["ObjectList"][0]
    emitter["couplings"] = [0.3 * c for c in emitter["couplings"]]
    path = str(tmp_path / "in.json")
    with open(path, "w") as f:
        json.dump(cfg, f)
    _run(path, "fp64", tmp_path / "fp64")
    _run(path, "split", tmp_path / "split")
    levels = cfg["ObjectList"][0]["dtc_levs"]
    base = "out/qe_0_level_%d.dat"
    assert sorted(levels) == [0, 4, 8]  # every diagonal element of the three-level matrix
    traces = {}
    for prec in ("fp64", "split"):
        pops = [read_output(str(tmp_path / prec / (base % lv)))[2] for lv in levels]
        tr = sum(p[:, 1] for p in pops)  # real parts
        assert tr.shape[0] == 100000
        traces[prec] = tr
        drift = np.max(np.abs(tr - tr[0])) / abs(tr[0])
        print("%s: trace drift over 10^5 steps %.3e" % (prec, drift))
        assert drift <= TOL_TRACE, "%s trace drift %.3e" % (prec, drift)
    for lv in levels:
        a = read_output(str(tmp_path / "fp64" / (base % lv)))[2][:, 1:]
        b = read_output(str(tmp_path / "split" / (base % lv)))[2][:, 1:]
        e = np.linalg.norm(a - b) / np.linalg.norm(a)
        print("level %d: split vs FP64 populations relative L2 %.3e" % (lv, e))
        assert e <= TOL_LONG, "level %d populations relative L2 %.3e" % (lv, e)
