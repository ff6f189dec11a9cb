"""The plan build puts the caller's OpenMP nesting settings back (no GPU).

The component build runs nested teams; it changes the OpenMP 3 nesting switch and the
max-active-levels count for its duration. Each check runs in a fresh process, so that the
settings it plants reach no other test, and builds a plan through the oracle library (which
shares the plan builder with the engine library).
"""
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, ROOT

_PROBE = r"""
import ctypes, sys
sys.path.insert(0, {root!r})
import oracle
lib = oracle.load()                       # loads the OpenMP runtime the plan builder uses
gomp = ctypes.CDLL("libgomp.so.1")
gomp.omp_set_nested({nested})
gomp.omp_set_max_active_levels({levels})
before = (gomp.omp_get_nested(), gomp.omp_get_max_active_levels())
sim = oracle.OracleSim({path!r})          # builds the plan (component build with nested teams)
sim.close()
after = (gomp.omp_get_nested(), gomp.omp_get_max_active_levels())
print(before, after)
sys.exit(0 if before == after else 1)
"""


@pytest.mark.parametrize("nested,levels", [(0, 1), (1, 3), (0, 4)])
def test_plan_build_restores_openmp_nesting(built_oracle, nested, levels):
    path = os.path.join(GOLDEN, "c2_small", "in.json")
    code = _PROBE.format(root=ROOT, nested=nested, levels=levels, path=path)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
