import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CONFIG_SMALL = os.path.join(ROOT, "pyprop_gb300", "configs", "hydrogen_velocity_small.ini")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libgbprop.so")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def small_problem_cpu():
    import pyprop_gb300 as pp
    conf = pp.Load(CONFIG_SMALL)
    prob = pp.Problem(conf, device="cpu")
    prob.SetupWavefunction()
    return prob


@pytest.fixture(scope="session")
def small_oracle(small_problem_cpu):
    from oracle import oracle as orc
    return orc.Operator.from_problem(small_problem_cpu)
