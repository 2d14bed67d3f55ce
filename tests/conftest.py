import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmmcgb.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle  # test infrastructure: the CPU checker
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def small_cube():
    from mmc_gb300 import meshgen
    return meshgen.homogeneous_cube(n=10)


@pytest.fixture(scope="session")
def small_inclusion():
    from mmc_gb300 import meshgen
    # 20^3 voxels at 3 mm, jittered, r=10 mm inclusion (a scaled-down copy of the 1.3M-tet workload)
    return meshgen.inclusion_cube(n=20, jitter=0.6, seed=7)


@pytest.fixture(scope="session")
def gpu_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mmc_gb300 import _native
    _native.load()  # raises if the library was not built: the GPU path must not fall back
    return True
