import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__ as g

    g.build()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def gpu_ctx(built):
    from qclojure_gb300.state import Context

    ctx = Context(seed=1, arithmetic="exact")
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def gpu_ctx_df(built):
    from qclojure_gb300.state import Context

    ctx = Context(seed=1, arithmetic="double-float")
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def sim(built):
    from qclojure_gb300.backend import create_simulator

    s = create_simulator({"precision": "c128", "fusion": "tiled", "seed": 3, "arithmetic": "exact"})
    yield s
    s.close()


@pytest.fixture(scope="session")
def sim_df(built):
    from qclojure_gb300.backend import create_simulator

    s = create_simulator({"precision": "c128", "fusion": "tiled", "seed": 3, "arithmetic": "double-float"})
    yield s
    s.close()
