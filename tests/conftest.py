import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) GPU; runs the CUDA path")
    config.addinivalue_line("markers", "slow: larger volumes")
    # the CPU oracle and the CUDA library are build products; build them if a fresh checkout
    # runs the tests before build()
    if not os.path.exists(os.path.join(ROOT, "oracle", "libpnm_oracle.so")):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build.sh")], check=True)
    if not os.path.exists(os.path.join(ROOT, "peclet_pnm_gb300", "libpnm_gb300.so")):
        subprocess.run([sys.executable, os.path.join(ROOT, "peclet_pnm_gb300", "build.py")],
                       cwd=ROOT, check=True)


@pytest.fixture(scope="session")
def port():
    from oracle import Oracle

    return Oracle("port", threads=1)


@pytest.fixture(scope="session")
def gpu():
    """The package on a real device; fails (does not skip) if the CUDA path cannot run."""
    import peclet_pnm_gb300 as pnm

    ctx = pnm.Context(0)
    yield pnm, ctx
    ctx.close()
