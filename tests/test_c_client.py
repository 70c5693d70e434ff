"""The C ABI driven by a plain C program (tests/c_abi_client.c), as a foreign-language shim
drives it: built with gcc against include/p9idg.h and the library, run on a small observation
through raw files.  Its partition must equal the oracle's bit for bit; on a GPU its w layers and
degridded visibilities must match the FP64 oracle and the model grid must come back shifted in
place (IDG.cs:44); without a GPU the first gridding call must return P9IDG_NO_DEVICE (exit 3)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, constants, gpu_available, oracle, pkg, rel_l2, workload

SRC = os.path.join(ROOT, "tests", "c_abi_client.c")


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("c_client") / "c_abi_client")
    lib = pkg._native.LIB_PATH
    subprocess.run([gcc, "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                    lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True, capture_output=True, text=True)
    return exe


def _run(client, tmp_path, mode):
    obs, cd = workload("small_256", n_ant=6, nt=120, nch=4)
    c, cd = constants(cd)
    N = cd["grid_size"]
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    np.ascontiguousarray(obs.uvw, np.float64).tofile(tmp_path / "uvw.bin")
    np.ascontiguousarray(obs.frequencies, np.float64).tofile(tmp_path / "freq.bin")
    np.ascontiguousarray(obs.vis, np.complex128).tofile(tmp_path / "vis.bin")
    np.ascontiguousarray(model, np.complex128).tofile(tmp_path / "grid.bin")
    nbl, nt, nch = obs.vis.shape
    args = [client, str(tmp_path), nbl, nt, nch, N, cd["subgrid_size"], cd["kernel_size"], cd["max_timesteps"],
            cd["wlayer_count"], repr(float(cd["wstep"])), repr(float(cd["scale_arcsec"])), cd["vis_count"], mode]
    r = subprocess.run([str(a) for a in args], capture_output=True, text=True, timeout=600)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    got = np.fromfile(tmp_path / "subgrids.bin", dtype=pkg.SUBGRID_DTYPE)
    assert np.array_equal(got.view(np.int32), subs.view(np.int32))
    return r, obs, cd, subs, model


def test_c_client_partition_and_no_device(client, tmp_path):
    if gpu_available():
        pytest.skip("a GPU is present (the GPU test runs the whole program)")
    r, *_ = _run(client, tmp_path, pkg.MODE_FP32)
    assert r.returncode == 3, r.stderr
    assert "no CUDA device" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("mode,tol", [(pkg.MODE_FP32, 1e-5), (pkg.MODE_TC_BF16X3, 1e-4)], ids=["fp32", "tc_bf16x3"])
def test_c_client_grids_and_degrids(need_gpu, client, tmp_path, mode, tol):
    r, obs, cd, subs, model = _run(client, tmp_path, mode)
    assert r.returncode == 0, r.stderr
    assert f"mode {mode}" in r.stdout
    N, W = cd["grid_size"], cd["wlayer_count"]
    layers = np.fromfile(tmp_path / "layers.bin", dtype=np.complex128).reshape(W, N, N)
    assert rel_l2(layers, oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < tol
    vis = np.fromfile(tmp_path / "vis_out.bin", dtype=np.complex128).reshape(obs.vis.shape)
    vref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(vis, vref) < tol
    shifted = np.fromfile(tmp_path / "grid_shifted.bin", dtype=np.complex128).reshape(N, N)
    assert np.array_equal(shifted, oracle.shift(model))
