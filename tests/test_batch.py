"""The batched sweep (chiml_batch_*): independent simulations of uneven sizes (the sweep
of 2-D TMz emitter sheets, and mixed members) stepped together by packed launches.

Packing changes which launch runs a member's blocks, never what they compute: every
member of a batch must write the same files as the same input run alone (byte for
byte), and in FP64 the oracle's and the reference's files to the parity bar.
"""
import os

import pytest

from compare import compare_dirs

TOL_FP64 = 1e-10


def _small_sweep(n=4, steps=240):
    from chiml_gb300 import configs
    return configs.config4(n=n, sides=(40, 48, 56, 64), steps=steps, pml=8)


def _write_members(root, members):
    from chiml_gb300 import configs
    paths = []
    for name, cfg in members:
        d = os.path.join(str(root), name)
        os.makedirs(d, exist_ok=True)
        paths.append(configs.write_json(cfg, os.path.join(d, "in.json")))
    return paths


def _same_files(a, b):
    n = 0
    for d, _, files in os.walk(a):
        for f in files:
            if f == "in.json":
                continue
            pa = os.path.join(d, f)
            pb = os.path.join(b, os.path.relpath(pa, a))
            assert os.path.exists(pb), pb
            assert open(pa, "rb").read() == open(pb, "rb").read(), f
            n += 1
    assert n >= 4
    return n


def test_config4_sweep_covers_the_grid():
    from chiml_gb300 import configs
    members = configs.config4()
    assert len(members) == 96
    sides, dets, dens = set(), set(), set()
    for name, cfg in members:
        cc = cfg["CompCell"]
        side = int(round(cc["size"][0] / cc["stepSize"][0])) + 1
        assert cc["size"][0] == cc["size"][1] and cc["size"][2] == 0.0 and cc["pol"] == "Ez"
        assert side in range(192, 769, 64)
        sides.add(side)
        qe = cfg["ObjectList"][0]
        dets.add(round(qe["Energy_Levels"][1]["E_cen"][0] - 2.0, 9))
        dens.add(qe["mol_den"])
        assert int(round(qe["size"][0] / cc["stepSize"][0])) == 10
        assert cfg["PML"]["thickness"][0] == pytest.approx(16 * cc["stepSize"][0])
        relax = qe["RelaxationOperators"][0]
        assert relax["dephasing_rate"] == pytest.approx(1.0 / 30e-15)
        steps = cfg["CompCell"]["tLim"] / cc["dt"]
        assert abs(steps - 6000) < 1
    assert len(sides) >= 6
    assert min(dets) == pytest.approx(-0.1) and max(dets) == pytest.approx(0.1)
    assert min(dens) == pytest.approx(1e25) and max(dens) == pytest.approx(1e26)
    assert len(dets) * len(dens) == 96
    # the same seed draws the same sizes
    assert [c["CompCell"]["size"] for _, c in configs.config4()] == [c["CompCell"]["size"] for _, c in members]


@pytest.mark.gpu
def test_batch_fp64_matches_oracle(built_engine, built_oracle, tmp_path):
    import oracle
    from chiml_gb300 import Batch
    members = _small_sweep()
    paths = _write_members(tmp_path / "gpu", members)
    with Batch(paths, precision="fp64", steps_per_graph=16) as b:
        b.run()
        b.finalize()
        for i in range(len(paths)):
            st = b.member_stats(i)
            assert st.steps_done == st.steps_total > 0
            assert st.n_emitters == 1
    for (name, _), p in zip(members, paths):
        ref = tmp_path / "oracle" / name
        os.makedirs(ref)
        oracle.run(p, str(ref))
        res = compare_dirs(str(ref), os.path.dirname(p), TOL_FP64)
        assert any("qe" in k for k in res) and any("flux" in k for k in res)


@pytest.mark.gpu
def test_batch_split_equals_members_run_alone(built_engine, tmp_path):
    from chiml_gb300 import Batch, Simulation
    members = _small_sweep(n=6, steps=200)
    paths = _write_members(tmp_path / "batch", members)
    with Batch(paths, precision="split", steps_per_graph=16) as b:
        # partial advances reuse the packed launches; the rest runs as eager steps and graphs
        b.step(37)
        b.step(100)
        assert all(b.member_stats(i).steps_done == 137 for i in range(len(paths)))
        b.run()
        b.finalize()
    for name, cfg in members:
        alone = tmp_path / "alone" / name
        os.makedirs(alone)
        sim = Simulation(os.path.join(str(tmp_path / "batch"), name, "in.json"), precision="split",
                         steps_per_graph=16, out_dir=str(alone))
        sim.step()
        sim.finalize()
        _same_files(str(tmp_path / "batch" / name), str(alone))


@pytest.mark.gpu
@pytest.mark.parametrize("march", ["2", "32"])
def test_batch_march_depth_leaves_results_unchanged(built_engine, tmp_path, monkeypatch, march):
    """The packed 2-D passes with a fixed march depth (rows per warp; the autotuner's
    other choices) give the same bytes as the members run alone."""
    from chiml_gb300 import Batch, Simulation
    monkeypatch.setenv("CHIML_BATCH_MARCH", march)
    members = _small_sweep(n=3, steps=120)
    paths = _write_members(tmp_path / "batch", members)
    with Batch(paths, precision="split", steps_per_graph=16) as b:
        b.run()
        b.finalize()
    for name, cfg in members:
        alone = tmp_path / "alone" / name
        os.makedirs(alone)
        sim = Simulation(os.path.join(str(tmp_path / "batch"), name, "in.json"), precision="split",
                         steps_per_graph=16, out_dir=str(alone))
        sim.step()
        sim.finalize()
        _same_files(str(tmp_path / "batch" / name), str(alone))


@pytest.mark.gpu
def test_batch_of_golden_cases_matches_reference_outputs(built_engine, tmp_path):
    """Members of different dimensions, media, sources and step counts in one batch (3-D
    anisotropic and dispersive, 3-D and 2-D emitters, 2-D dielectric, 2-D and 3-D TFSF
    plane waves): the packed steps run in phases
    that stop each member at its own last step, and every member still meets the FP64
    parity bar against the reference's own outputs."""
    import shutil
    from conftest import GOLDEN, golden_cases
    from chiml_gb300 import Batch
    cases = [c for c in ["c2_aniso", "qe_3d", "qe_tm", "c1_small", "tfsf_2d_te", "tfsf_disp"] if c in golden_cases()]
    assert len(cases) >= 3
    paths = []
    for c in cases:
        d = tmp_path / c
        os.makedirs(d)
        shutil.copy(os.path.join(GOLDEN, c, "in.json"), d / "in.json")
        paths.append(str(d / "in.json"))
    with Batch(paths, precision="fp64", steps_per_graph=8) as b:
        totals = [b.member_stats(i).steps_total for i in range(len(paths))]
        assert len(set(totals)) > 1
        b.run()
        b.finalize()
    for c in cases:
        compare_dirs(os.path.join(GOLDEN, c, "ref"), str(tmp_path / c), TOL_FP64)


@pytest.mark.gpu
def test_batch_rejects_a_bad_member(built_engine, tmp_path):
    from chiml_gb300 import Batch, ChimlError
    members = _small_sweep(n=2, steps=10)
    paths = _write_members(tmp_path, members)
    bad = tmp_path / "bad.json"
    bad.write_text("{ not json")
    with pytest.raises(ChimlError) as ei:
        Batch([paths[0], str(bad), paths[1]])
    assert "batch member 1" in str(ei.value)
