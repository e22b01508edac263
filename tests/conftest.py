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


@pytest.fixture(scope="session", autouse=True)
def _native_builds():
    """Build libst3d.so and the oracle in-tree if they are missing or stale."""
    from stencil3d_gb300 import build as pbuild
    from oracle import build as obuild
    pbuild.build()
    obuild.build_oracle()
    yield
