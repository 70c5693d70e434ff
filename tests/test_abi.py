"""The C ABI: the library loads, exports every symbol include/p9idg.h declares, and the
host-only entry points behave as the reference's members do.  No compute runs here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available, kat_constants, oracle, pkg

HEADER = os.path.join(ROOT, "include", "p9idg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(p9idg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_surface():
    names = declared_functions()
    assert len(names) >= 30
    assert set(names) == set(pkg._native.SIGNATURES), set(names) ^ set(pkg._native.SIGNATURES)


def test_integration_binds_every_declared_symbol():
    """The P/Invoke declarations a C# maintainer adds cover the whole header."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    bound = set(re.findall(r"\bextern\s+\w+\s+(p9idg_[a-z0-9_]+)\s*\(", text))
    assert bound == set(declared_functions()), set(declared_functions()) ^ bound


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(pkg._native.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string():
    L = pkg._native.lib()
    assert b"sm_103a" in L.p9idg_version()
    assert L.p9idg_plan_set_mode(None, 0) == 1
    assert "null" in pkg._native.last_error()


def test_no_device_is_reported_not_faked():
    if gpu_available():
        pytest.skip("a GPU is present")
    cd = kat_constants()
    c = pkg.GriddingConstants.from_dict(cd)
    uvw = np.zeros((1, 2, 3))
    freq = np.array([299792458.0])
    part = pkg.Partitioner.CreatePartition(c, uvw, freq)
    with pytest.raises(pkg.P9IDGError) as e:
        pkg.IDG.GridW(c, part, np.ones((1, 2, 1), np.complex128), uvw, freq)
    assert e.value.code == 7  # P9IDG_NO_DEVICE: there is no CPU fallback
    with pytest.raises(pkg.P9IDGError):
        pkg.FFT.WStackIFFTFloat(np.zeros((1, 8, 8), np.complex128), 1)


@pytest.mark.parametrize("n", [4, 5, 8, 9])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_fft_shift_host(n, dtype):
    a = (np.arange(n * n) + 1j * np.arange(n * n)[::-1]).reshape(n, n)
    a = a.astype(dtype) if dtype == np.complex128 else a.real.astype(dtype)
    ref = oracle.shift(a)
    pkg.FFT.Shift(a)
    assert np.array_equal(a, ref)


def test_adder_range_error_matches_reference():
    """UPixel = N-S passes InRange but Adder.Add throws "invalid grid" (Adder.cs:30-50)."""
    cd = kat_constants()
    c = pkg.GriddingConstants.from_dict(cd)
    uvw = np.array([[[24.0, 0.0, 0.0]]])
    freq = np.array([299792458.0])
    part = pkg.Partitioner.CreatePartition(c, uvw, freq)
    assert part[0][0].UPixel == 48
    with pytest.raises(pkg.P9IDGError) as e:
        pkg.IDG.Grid(c, part, np.ones((1, 1, 1), np.complex128), uvw, freq)
    assert e.value.code == 4 and str(e.value) == "invalid grid"
    with pytest.raises(oracle.OracleError) as e2:
        subs = oracle.partition(cd, uvw, freq)
        oracle.idg_grid(cd, subs, np.ones((1, 1, 1), np.complex128), uvw, freq)
    assert e2.value.code == 4


def test_host_api_refuses_wrong_shapes():
    """Every array is sized from the plan in the C ABI, so the Python mirror refuses arrays of
    another shape instead of letting them be read or written out of bounds."""
    from conftest import constants, workload
    obs, cd = workload("small_256", n_ant=5, nt=20, nch=4)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    N = cd["grid_size"]
    with pytest.raises(ValueError):
        pkg.IDG.DeGridW(c, part, np.zeros((N // 2, N // 2), np.complex128), obs.uvw, obs.frequencies)
    with pytest.raises(ValueError):
        pkg.IDG.GridW(c, part, obs.vis[:, :10], obs.uvw, obs.frequencies)
    with pytest.raises(ValueError):
        pkg.IDG.CalculatePSF(c, part, obs.uvw, np.zeros((1, 1, 1), bool), obs.frequencies)
    with pytest.raises((ValueError, pkg.P9IDGError)):  # a plan for other uvw dimensions is refused too
        pkg.IDG.Grid(c, part, obs.vis, obs.uvw[:, :5], obs.frequencies)
