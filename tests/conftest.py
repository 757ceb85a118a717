import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# batched solves of the test session keep their autotuner cache in a private
# temporary file, not in the user's cache directory
if "SIMALL_AUTOTUNE_CACHE" not in os.environ:
    import tempfile

    os.environ["SIMALL_AUTOTUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="simall_tests_"), "autotune.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build_oracle()
    return O


@pytest.fixture(scope="session")
def ref():
    """The reference's own code, compiled into oracle/_ref (only where the
    reference tree was available at build time)."""
    from oracle import oracle as O

    if not O.RefLib.available():
        pytest.skip("compiled reference oracle (oracle/_ref) not present")
    return O.RefLib()


@pytest.fixture(scope="session")
def sg():
    import simall_gb300

    simall_gb300.build.build()
    simall_gb300.load()
    return simall_gb300


@pytest.fixture(scope="session")
def ctx(sg):
    c = sg.Context(0)
    yield c
    c.close()
