"""The oracle against the reference's own outputs (golden fixtures made by tests/golden/make_golden.py)."""
import os

import pytest

from conftest import GOLDEN, golden_cases, stage_inputs
from compare import compare_dirs

# FP64, same formulas; only the summation order differs from the reference build
TOL = 1e-10


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_matches_reference(case, built_oracle, tmp_path):
    import oracle
    stage_inputs(case, tmp_path)
    oracle.run(os.path.join(GOLDEN, case, "in.json"), str(tmp_path))
    res = compare_dirs(os.path.join(GOLDEN, case, "ref"), str(tmp_path), TOL)
    assert len(res) >= 2
