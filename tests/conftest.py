import functools
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as entry  # noqa: E402

pkg = entry.load_package()
synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
import oracle  # noqa: E402  (the FP64 CPU oracle; test infrastructure)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available():
    try:
        return pkg.device_count() > 0
    except pkg.NativeLibraryMissing:
        return False


@pytest.fixture(scope="session", autouse=True)
def _built():
    # built by __graft_entry__.build(); build here when a fresh checkout runs the tests directly
    if not os.path.exists(pkg._native.LIB_PATH):
        entry.build()
    oracle.lib()


@pytest.fixture
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU test run without a CUDA device")


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


@functools.lru_cache(maxsize=None)
def workload(name, n_ant=None, nt=None, nch=None, seed=None):
    obs, cd = synth.build(synth.scaled_workload(name, n_ant=n_ant, nt=nt, nch=nch, seed=seed))
    return obs, cd


def constants(cd, **over):
    d = dict(cd)
    d.update(over)
    return pkg.GriddingConstants.from_dict(d), d


C_LIGHT = 299792458.0


def kat_constants(N=64, S=16, kernel=4, max_t=10, W=1, wstep=0.0, vis_count=1):
    """Constants with ImageSize = 1.0 exactly (cell = 1/N), so a uv coordinate in metres at
    frequency c is its pixel coordinate."""
    return dict(vis_count=vis_count, grid_size=N, subgrid_size=S, kernel_size=kernel, max_timesteps=max_t,
                scale_arcsec=1.0 / N, wlayer_count=W, wstep=wstep)
