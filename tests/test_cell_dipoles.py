"""Per-cell dipoles, an extension with no reference counterpart (an emitter object's z
operator turned per cell to a direction drawn on the sphere and scaled by a drawn factor,
from a seeded PCG32 stream).

Pins: the oracle with every cell's dipole along z and scale 1 reproduces the reference's
outputs (the extension reduces to the reference there); random directions and scales change
the outputs; the GPU's FP64 form matches the oracle within the parity bar and the split
form stays within its emitter tolerance (GPU tests)."""
import json
import os

import pytest

from compare import compare_dirs, relative_errors
from conftest import GOLDEN

TOL_FP64 = 1e-10
TOL_SPLIT_EMIT = 1e-5


def _case(tmp_path, name, **keys):
    cfg = json.load(open(os.path.join(GOLDEN, "qe_3d", "in.json")))
    cfg["ObjectList"][0].update(keys)
    p = str(tmp_path / (name + ".json"))
    with open(p, "w") as f:
        json.dump(cfg, f)
    return p


def test_z_dipoles_reduce_to_the_reference(built_oracle, tmp_path):
    import oracle
    p = _case(tmp_path, "z", dipole_orientation="z", dipole_scale_range=[1.0, 1.0])
    oracle.run(p, str(tmp_path / "z"))
    compare_dirs(os.path.join(GOLDEN, "qe_3d", "ref"), str(tmp_path / "z"), TOL_FP64)


def test_random_dipoles_change_the_outputs(built_oracle, tmp_path):
    import oracle
    p = _case(tmp_path, "r", dipole_orientation="random", dipole_seed=20261206, dipole_scale_range=[0.5, 1.5])
    oracle.run(p, str(tmp_path / "r"))
    err = relative_errors(os.path.join(GOLDEN, "qe_3d", "ref"), str(tmp_path / "r"), detail=True)
    pol = [e for f, g in err.items() if "pol" in f for e in g.values()]
    assert pol and max(pol) > 1e-2, err


def test_inputs_the_extension_rejects(built_engine, tmp_path):
    from chiml_gb300 import ChimlError, Simulation
    for keys, status in ((dict(dipole_orientation="sideways"), 1), (dict(dipole_scale_range=[2.0, 1.0]), 1)):
        p = _case(tmp_path, "bad", **keys)
        with pytest.raises(ChimlError) as e:
            Simulation(p)
        assert e.value.status == status, str(e.value)


def _gpu(path, out_dir, precision):
    from chiml_gb300 import Simulation
    sim = Simulation(path, precision=precision, steps_per_graph=8, out_dir=str(out_dir))
    try:
        sim.step()
        sim.finalize()
    finally:
        sim.close()


@pytest.mark.gpu
def test_gpu_random_dipoles_match_the_oracle(built_engine, built_oracle, tmp_path):
    import oracle
    p = _case(tmp_path, "r", dipole_orientation="random", dipole_seed=7, dipole_scale_range=[0.5, 1.5])
    oracle.run(p, str(tmp_path / "oracle"))
    _gpu(p, tmp_path / "fp64", "fp64")
    compare_dirs(str(tmp_path / "oracle"), str(tmp_path / "fp64"), TOL_FP64)
    _gpu(p, tmp_path / "split", "split")
    err = relative_errors(str(tmp_path / "fp64"), str(tmp_path / "split"), detail=True)
    for f, groups in err.items():
        if "_level_" in f or "pol" in f:
            for g, e in groups.items():
                assert e <= TOL_SPLIT_EMIT, (f, g, e)
