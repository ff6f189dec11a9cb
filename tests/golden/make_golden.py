"""Regenerates the golden fixtures from the reference's own CPU build.

For every case in CASES this writes <case>/in.json (from chiml_gb300.configs),
runs the one-process build of the chiML sources (oracle/_ref/chiml_ref, made by
oracle/Makefile.ref) on it in a scratch directory, and copies every output file
it writes into <case>/ref/. Run it where the chiML sources are available:

    python tests/golden/make_golden.py
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from chiml_gb300 import configs  # noqa: E402


def _te_dispersive():
    """2-D TE (Ex, Ey, Hz): Drude-Lorentz disk, Ey point source, binary box detector, flux box."""
    cfg = configs.config1(n=72, pml=8, steps=260, radius_cells=9, src_gap_cells=10, ndtc=2, nfreq=9)
    cfg["CompCell"]["pol"] = "Hz"
    cfg["SourceList"][0]["pol"] = "Ey"
    cfg["ObjectList"] = [configs._obj("sphere", [0.0, 0.0, 0.0], radius=0.45, material="custom", eps=2.0,
                                      pols=configs.drude_lorentz_pols(4.0, [(1.0, 0.2, 0.0), (0.6, 0.3, 2.4)]))]
    for d in cfg["DetectorList"]:
        d["type"] = "Hz"
    cfg["DetectorList"].append({"loc": [0.5, 0.3, 0.0], "size": [0.2, 0.1, 0.0], "type": "Ey",
                                "fname": "out/te_box", "dtc_class": "bin", "SI": True, "Time_Interval": 2 * cfg["CompCell"]["dt"]})
    cfg["FluxList"] = [{"name": "out/te_flux", "loc": [0.0, 0.0, 0.0], "size": [1.6, 1.6, 0.0],
                        "lamL": 3.0, "lamR": 8.0, "nfreq": 9, "SI": True}]
    return cfg


def _tm_lorentz():
    """2-D TMz with a two-pole Lorentz disk and an E_pow box detector."""
    cfg = configs.config1(n=64, pml=8, steps=240, radius_cells=8, src_gap_cells=9, ndtc=3, nfreq=10)
    cfg["ObjectList"][0]["pols"] = configs.drude_lorentz_pols(6.0, [(0.5, 0.3, 2.0), (0.4, 0.5, 3.1)])
    cfg["ObjectList"][0]["eps"] = 1.5
    cfg["DetectorList"].append({"loc": [0.6, -0.2, 0.0], "size": [0.1, 0.15, 0.0], "type": "Ez",
                                "fname": "out/tm_box", "dtc_class": "bin", "SI": False, "Time_Interval": 3 * cfg["CompCell"]["dt"]})
    return cfg


CASES = {
    "c1_small": lambda: configs.config1(n=80, pml=10, steps=300, radius_cells=10, src_gap_cells=12, ndtc=4, nfreq=12),
    "c2_small": lambda: configs.config2(n=34, pml=6, steps=70, nell=3, nfreq=6, metal_radius_cells=20),
    "te_dispersive": _te_dispersive,
    "tm_lorentz": _tm_lorentz,
}


def main(names=None):
    ref = os.path.join(ROOT, "oracle", "_ref", "chiml_ref")
    if not os.path.exists(ref):
        raise SystemExit("build the reference first: make -f oracle/Makefile.ref")
    for name, make in CASES.items():
        if names and name not in names:
            continue
        case = os.path.join(HERE, name)
        shutil.rmtree(case, ignore_errors=True)
        os.makedirs(case)
        configs.write_json(make(), os.path.join(case, "in.json"))
        with tempfile.TemporaryDirectory() as tmp:
            shutil.copy(os.path.join(case, "in.json"), os.path.join(tmp, "in.json"))
            r = subprocess.run([ref, "in.json"], cwd=tmp, capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit("%s failed:\n%s%s" % (name, r.stdout, r.stderr))
            for d, _, files in os.walk(tmp):
                for f in files:
                    src = os.path.join(d, f)
                    rel = os.path.relpath(src, tmp)
                    if rel == "in.json" or f == "levelDist.dat":
                        continue
                    dst = os.path.join(case, "ref", rel)
                    os.makedirs(os.path.dirname(dst), exist_ok=True)
                    shutil.copy(src, dst)
        print(name, "ok")


if __name__ == "__main__":
    main(sys.argv[1:])
