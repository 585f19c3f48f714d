import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the library's kernels")
    config.addinivalue_line("markers", "slow: full-size parity runs (minutes)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, LIB, build
    if not os.path.exists(LIB):
        build()
    return Oracle()


@pytest.fixture(scope="session")
def ref_oracle():
    """The reference itself compiled from its sources (only where they were available at build time)."""
    from oracle.oracle import Oracle, REF_LIB
    if not os.path.exists(REF_LIB):
        pytest.skip("oracle/_ref not built (reference sources absent)")
    return Oracle(reference=True)


@pytest.fixture(scope="session")
def gwn():
    import antipodal_gb300 as ag
    ag.library()
    return ag


@pytest.fixture()
def disp(gwn):
    # the mixed kernels run at every size here (by default they start at 2^20 pairs per call)
    d = gwn.CudaDispatcher(device=0, mixed_min_pairs=0)
    yield d
    d.close()
