import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and runs the CUDA engine")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def ref_oracle(oracle):
    from oracle import pyoracle
    if not pyoracle.RefOracle.available():
        pytest.skip("reference checkout not present: host build of the reference not available")
    return pyoracle.RefOracle()


@pytest.fixture(scope="session")
def mcfl_lib():
    from cudamcfl_gb300 import build, load
    build.build()
    return load()


@pytest.fixture(scope="session")
def multipliers(oracle):
    return oracle.multipliers(32769)


@pytest.fixture(scope="session")
def table32768(multipliers):
    return multipliers[1:].copy()


@pytest.fixture(scope="session")
def safeprimes_file(tmp_path_factory, oracle):
    p = tmp_path_factory.mktemp("sp") / "safeprimes_base32.txt"
    oracle.write_safeprimes(str(p), 32769)
    return str(p)


@pytest.fixture(scope="session")
def gpu_ctx(mcfl_lib):
    import cudamcfl_gb300 as m
    ctx = m.Context(math=m.MATH_EXACT)
    yield ctx
    ctx.close()
