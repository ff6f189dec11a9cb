"""Host-side input handling: the reader's conversions and the rejection of unsupported features."""
import copy
import json
import os

import pytest

from chiml_gb300 import configs
from conftest import GOLDEN


def _create(built_engine, cfg, tmp_path):
    from chiml_gb300 import ChimlError, Simulation
    p = str(tmp_path / "in.json")
    configs.write_json(cfg, p)
    with pytest.raises(ChimlError) as ei:
        Simulation(p)
    return ei.value


def _base():
    return configs.config1(n=40, pml=6, steps=10, radius_cells=5, src_gap_cells=5, ndtc=1, nfreq=4)


@pytest.mark.parametrize("mutate,status", [
    (lambda c: c["CompCell"].__setitem__("PBC", True), 2),
    (lambda c: c["CompCell"].__setitem__("cplxFields", True), 2),
    # constant mu is taken inside the interior; an object of mu reaching the CPML is refused
    (lambda c: c["ObjectList"][0].update(mu=2.0, radius=0.65), 2),
    (lambda c: c["ObjectList"][0].__setitem__("mu", -1.0), 1),
    (lambda c: c["ObjectList"][0].__setitem__("material", "Unobtainium"), 1),
    (lambda c: c["ObjectList"][0].__setitem__("shape", "dodecahedron"), 1),
    (lambda c: c["ObjectList"][0].update(shape="cone", radSmall=0.2, radLarge=0.1, height=0.3), 1),
    (lambda c: c["DetectorList"][0].__setitem__("dtc_class", "bmp"), 2),
    (lambda c: c["DetectorList"][0].__setitem__("type", "Mx"), 2),
    (lambda c: c["CompCell"].__setitem__("dt", 1.0), 1),
    (lambda c: c["CompCell"].__setitem__("pol", "Q"), 1),
    (lambda c: c["ObjectList"][0].pop("Basis_Set"), 1),
    (lambda c: c.pop("FluxList"), 1),
    (lambda c: c["FluxList"][0].update(load=True), 1),
])
def test_rejections_are_reported_with_status(built_engine, tmp_path, mutate, status):
    cfg = copy.deepcopy(_base())
    mutate(cfg)
    err = _create(built_engine, cfg, tmp_path)
    assert err.status == status, str(err)


def _relpole(kind, **kw):
    p = {"gamma": 0.01, "omega": 1.0, "sigma_p": 1.0, "dipOrE": kind}
    p.update(kw)
    return p


@pytest.mark.parametrize("obj,status,msg", [
    # tanIso needs relative magnetic dipoles too; with the default isotropic ones the
    # reference's own check throws (parallelInputs.cpp:1290-1295)
    (dict(shape="sphere", radius=0.2, pols=[_relpole("normal", tanIso=True)]), 1, "isotropic in tangential"),
    # the reference's prism gradient reads past its vertex array
    (dict(shape="triangle_prism", base=0.3, height=0.2, length=0.3, pols=[_relpole("normal")]), 2, "triangular prism"),
    # the reference's TERS tip has no gradient and throws this message
    (dict(shape="ters_tip", rad_curve=0.1, base=0.3, length=0.3, pols=[_relpole("tangent")]), 1, "Gradient is not defined"),
])
def test_surface_relative_dipoles_that_cannot_run(built_engine, tmp_path, obj, status, msg):
    cfg = configs.config2(n=24, pml=4, steps=10, nell=0, nfreq=3, metal_radius_cells=0, tfsf=False)
    o = configs._obj(obj.pop("shape"), [0.0, 0.0, 0.0], material="custom", eps=2.0, pols=obj.pop("pols"), **obj)
    cfg["ObjectList"] = [o]
    err = _create(built_engine, cfg, tmp_path)
    assert err.status == status and msg in str(err), str(err)


def test_comments_are_stripped(built_oracle, tmp_path):
    import oracle
    src = open(os.path.join(GOLDEN, "c1_small", "in.json")).read().splitlines()
    src.insert(1, "   // a comment line")
    src[3] = src[3] + "   // trailing comment"
    p = tmp_path / "in.json"
    p.write_text("\n".join(src))
    sim = oracle.OracleSim(str(p))
    assert sim.steps_total == 300


def test_step_count_is_ceil_of_tlim_over_dt(built_oracle, tmp_path):
    import oracle
    cfg = _base()
    cfg["CompCell"]["tLim"] = 10.2 * cfg["CompCell"]["dt"]
    p = configs.write_json(cfg, str(tmp_path / "in.json"))
    assert oracle.OracleSim(p).steps_total == 11


def _reference_failures():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.exists(os.path.join(GOLDEN, d, "ref_error.txt")))


@pytest.mark.parametrize("case", _reference_failures())
def test_inputs_the_reference_cannot_run_are_rejected(built_engine, case):
    """The reference build stops on these inputs (its last message is in ref_error.txt): the
    engine rejects them at chiml_create instead of running them."""
    from chiml_gb300 import ChimlError, Simulation
    with pytest.raises(ChimlError) as ei:
        Simulation(os.path.join(GOLDEN, case, "in.json"))
    assert ei.value.status in (1, 2), str(ei.value)
