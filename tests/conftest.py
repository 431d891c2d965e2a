import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libgbns.so")
    # temporary files of the tests stay inside the repository, in the git-ignored build folder
    if not config.option.basetemp:
        os.makedirs(os.path.join(ROOT, "_build"), exist_ok=True)   # pytest creates only the last level
        config.option.basetemp = os.path.join(ROOT, "_build", "pytest-tmp")


def corr_gauss(D, seed):
    """mu ~ N(0,1)^D, Sigma = A A^T / D + 0.1 I with A ~ N(0,1)^{DxD} (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    mu = rng.standard_normal(D)
    A = rng.standard_normal((D, D))
    return mu, A @ A.T / D + 0.1 * np.eye(D)


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from jaxns_gb300.build import build_library
    build_library()
    from jaxns_gb300 import _ffi
    return _ffi.load()
