"""Shared test setup: import paths, the `gpu` marker, and built libraries."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "jagua-rs_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def jcde_mod():
    import jcde

    jcde.build()
    return jcde


@pytest.fixture(scope="session")
def strip_layout(oracle_mod):
    """The small strip layout (10 star items, 40 placed), generated with the oracle."""
    from jcde import workload as W

    return W.strip_layout(oracle_mod.OracleBackend)


@pytest.fixture(scope="session")
def star_layout(oracle_mod):
    """The large star-container layout (40 items, 300 placed, holes + zones), from the oracle."""
    from jcde import workload as W

    return W.star_container_layout(oracle_mod.OracleBackend)
