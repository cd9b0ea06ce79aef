import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
# where the reference checkout lies on the machine that builds the oracle
# from it (absent elsewhere: the tests then use tests/golden)
os.environ.setdefault("RMN_REFERENCE_DIR", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def port():
    from oracle import bindings
    if not os.path.exists(bindings.PORT_SO):
        bindings.build(with_reference=False)
    return bindings.OracleLib("port")


@pytest.fixture(scope="session")
def ref():
    from oracle import bindings
    if not bindings.have_ref():
        if os.path.isdir(os.path.join(bindings.REFERENCE_DIR, "src")):
            bindings.build(with_reference=True)
        else:
            pytest.skip("the reference checkout is not on this machine; parity is carried by tests/golden")
    return bindings.OracleLib("ref")


@pytest.fixture(scope="session")
def ref_tex():
    from oracle import bindings
    if not bindings.have_ref_tex():
        if os.path.isdir(os.path.join(bindings.REFERENCE_DIR, "src")):
            bindings.build(with_reference=True)
        else:
            pytest.skip("the reference checkout is not on this machine; parity is carried by tests/golden")
    return bindings.OracleLib("ref_tex")
