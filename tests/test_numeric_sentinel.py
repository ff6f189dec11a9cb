"""The NaN/Inf sentinel (GPU required): a detector or DFT point that samples a value that is
not finite turns the next chiml_sync / chiml_finalize into CHIML_E_NUMERIC.

The divergence is made by the input, not by a fault: a point source of amplitude 1e45
overflows FP32 at its first step in the split form (dt times the pulse there, ~3e41, is
above the FP32 range), while the FP64 form of the same input stays finite."""
import json
import os

import pytest

from chiml_gb300 import configs

pytestmark = pytest.mark.gpu


def _input(tmp_path, amp):
    cfg = configs.config1(n=48, pml=6, steps=60, radius_cells=5, src_gap_cells=6, ndtc=2, nfreq=4)
    src = cfg["SourceList"][0]
    src["PulseList"][0]["Field_Intensity"] = amp
    cfg["DetectorList"].append({"loc": list(src["loc"]), "size": [0.0, 0.0, 0.0], "type": "Ez",
                                "fname": "out/at_source", "dtc_class": "txt", "SI": False,
                                "Time_Interval": cfg["CompCell"]["dt"]})
    path = str(tmp_path / "in.json")
    with open(path, "w") as f:
        json.dump(cfg, f)
    return path


@pytest.mark.parametrize("graph", [0, 8])
def test_split_overflow_is_reported_as_numeric(built_engine, tmp_path, graph):
    from chiml_gb300 import Simulation
    from chiml_gb300.api import ChimlError
    sim = Simulation(_input(tmp_path, 1e45), precision="split", steps_per_graph=graph, out_dir=str(tmp_path / "out"))
    try:
        sim.step(16)
        with pytest.raises(ChimlError) as e:
            sim.sync()
        assert e.value.status == 5, str(e.value)
        with pytest.raises(ChimlError) as e:
            sim.finalize()
        assert e.value.status == 5
    finally:
        sim.close()


def test_finite_run_is_not_flagged(built_engine, tmp_path):
    from chiml_gb300 import Simulation
    for prec, amp in (("fp64", 1e45), ("split", 1.0)):
        sim = Simulation(_input(tmp_path, amp), precision=prec, steps_per_graph=8, out_dir=str(tmp_path / prec))
        try:
            sim.step()
            sim.sync()
            sim.finalize()
        finally:
            sim.close()
