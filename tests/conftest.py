"""Test configuration: the ``gpu`` marker and the in-tree builds.

Tests marked ``gpu`` need a GB300 and call the CUDA library through its C ABI;
everything else runs on a CPU-only machine (oracle against the reference's
golden vectors, host logic, the C ABI's exports and argument checks, and the
multi-process paths over gloo).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (run with -m gpu)")
    # the reference's own host path (oracle/_ref) before collection: test
    # modules decide at import whether the live reference is there
    from oracle import build as obuild
    obuild.build_ref()


# Where the reference's sources sit on the machine that built this checkout
# (absent on the GPU machine, where the golden fixtures pin the oracle instead).
_REFERENCE_SOURCES = "/root/reference"
if "ST3D_REFERENCE_DIR" not in os.environ and os.path.isfile(
        os.path.join(_REFERENCE_SOURCES, "iterators.cpp")):
    os.environ["ST3D_REFERENCE_DIR"] = _REFERENCE_SOURCES


@pytest.fixture(scope="session", autouse=True)
def _native_builds():
    """Build libst3d.so and the oracle in-tree if they are missing or stale."""
    from stencil3d_gb300 import build as pbuild
    from oracle import build as obuild
    pbuild.build()
    obuild.build_oracle()
    yield
