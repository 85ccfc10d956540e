import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def port_built():
    """Builds the CPU checkers (oracle/_ref) once per session."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return True


# Where the reference's sources are mounted (its src/ and examples/); the
# STRUCTURED_REF environment variable overrides the default location.
REF_ROOT = os.environ.get("STRUCTURED_REF", "/root/reference")


@pytest.fixture(scope="session")
def ref_available():
    """The reference build exists only where its sources are mounted."""
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        return False
    r = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + REF_ROOT])
    return r.returncode == 0


@pytest.fixture(scope="session")
def gpu_lib():
    import torch  # noqa: F401  (device query only)
    from structured_gb300 import build
    build.build()
    from structured_gb300 import solver
    return solver.load_library()
