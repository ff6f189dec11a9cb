import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_oracle():
    from chiml_gb300 import build
    return build.build_oracle()


@pytest.fixture(scope="session")
def built_engine():
    from chiml_gb300 import build
    return build.build_engine()


def golden_cases():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.isdir(os.path.join(GOLDEN, d, "ref")))


def stage_inputs(case, out_dir):
    """Copies the files a golden case reads besides its input (its inputs/ directory: files a
    reference run of another input produced) into the run's output directory, which the
    engine and the oracle resolve relative names against."""
    import shutil
    src = os.path.join(GOLDEN, case, "inputs")
    if os.path.isdir(src):
        os.makedirs(str(out_dir), exist_ok=True)
        for f in os.listdir(src):
            shutil.copy(os.path.join(src, f), os.path.join(str(out_dir), f))
