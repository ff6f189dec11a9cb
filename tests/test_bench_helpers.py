"""bench.py's workload helpers (no GPU): the sizes each workload names and the c5 crop."""
import argparse
import os
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_workload_dimensions():
    assert bench._dims("c1", 400) == "400^2"
    assert bench._dims("c2", 256) == "256^3"
    assert bench._dims("c5", 640) == "640x640x320"
    cfg = bench._workload(64, 10, "c5")
    dx = cfg["CompCell"]["stepSize"][0]
    assert round(cfg["CompCell"]["size"][0] / dx) + 1 == 64 and round(cfg["CompCell"]["size"][2] / dx) + 1 == 32


def test_cpu_sample_config_uses_the_crop_for_c5(tmp_path):
    args = argparse.Namespace(workload="c5")
    path, what = bench._cpu_sample_config(args, str(tmp_path), "unused.json", 12)
    assert os.path.exists(path) and "160x160x80" in what
    args = argparse.Namespace(workload="c2")
    assert bench._cpu_sample_config(args, str(tmp_path), "in.json", 12) == ("in.json", "the full workload")
