import os
import sys

os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")   # one stream per concurrent solve in the serving tests

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "nunatak.jl_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libnunatak_gb300.so")


def _gpu_problem_class():
    import nunatak_gb300
    return nunatak_gb300.Problem


def _oracle_problem_class():
    import nunatak_oracle
    return nunatak_oracle.OracleProblem


@pytest.fixture(params=["oracle", pytest.param("gpu", marks=pytest.mark.gpu)])
def backend(request):
    """Problem class of the backend under test: the CPU oracle, or the GPU library (marked gpu)."""
    return _oracle_problem_class() if request.param == "oracle" else _gpu_problem_class()


@pytest.fixture
def oracle_cls():
    return _oracle_problem_class()


@pytest.fixture
def gpu_cls():
    return _gpu_problem_class()
