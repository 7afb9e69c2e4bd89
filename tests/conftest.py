import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def built_lib():
    from asam_gb300.build import build_library, build_oracle

    build_oracle()
    return build_library()


@pytest.fixture(scope="session")
def built_oracle():
    from asam_gb300.build import build_oracle

    return build_oracle()
