"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def pkg():
    import traditional_dic_gb300 as P
    from traditional_dic_gb300 import build
    build.build()
    return P


@pytest.fixture(scope="session")
def workload0():
    from traditional_dic_gb300 import synthetic
    return synthetic.workload(0)


@pytest.fixture(scope="session")
def gpu_ctx(pkg):
    from traditional_dic_gb300 import subset as S
    return S.default_context()


def small_speckle(shape=(96, 96), n=240, seed=7, u0=0.4, v0=-0.3, noise=0.5, dtype=np.uint8):
    from traditional_dic_gb300 import synthetic
    f = synthetic.Field("linear", dict(u0=u0, ux=0.002, uy=-0.001, v0=v0, vx=0.001, vy=0.003))
    return synthetic.speckle_pair(shape, n, f, noise, seed, dtype=dtype)
