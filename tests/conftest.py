import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the native kernels)")
    config.addinivalue_line("markers", "reference: needs the reference sources (compiled into oracle/_ref)")


def pytest_runtest_setup(item):
    if "gpu" in item.keywords:
        from glslppm_gb300 import native
        if native.device_count() == 0:
            # a GPU test must never pass silently on a machine without a GPU
            pytest.fail("GPU test selected but no CUDA device is visible")
    if "reference" in item.keywords:
        from oracle.build import reference_available
        if not reference_available():
            pytest.skip("reference sources not present on this machine")


@pytest.fixture(scope="session")
def native_lib():
    from glslppm_gb300 import native
    return native


@pytest.fixture(scope="session")
def cornell_c1_mesh():
    from glslppm_gb300 import scenes
    sc = scenes.cornell_box()
    return sc, sc.to_mesh()


@pytest.fixture(scope="session")
def cornell_metal():
    """The reference's default scene (cornell_metal.obj at scale 0.01, camera (0,0,13)) as the
    reference's host code loaded it -- from the committed fixture."""
    from tests.golden.fixtures import load_cornell_metal
    return load_cornell_metal()
