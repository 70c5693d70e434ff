"""Host-array calls with the caller's arrays used in place (the kernels read and write host
memory directly where the device reaches it through the host's page tables) must equal the
staged path: same layers, same visibilities (uncovered samples exactly 0, whatever the output
array held), and the same in-place FFT.Shift of DeGrid's input grid."""
import numpy as np
import pytest

from conftest import constants, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
@pytest.mark.parametrize("wstack", [True, False], ids=["w", "nonw"])
def test_in_place_equals_staged(need_gpu, mode, wstack):
    obs, cd = workload("meerkat_3072", n_ant=10, nt=300, nch=16, seed=31)
    c, cd = constants(cd, grid_size=1024)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    grid_fn = pkg.IDG.GridW if wstack else pkg.IDG.Grid
    degrid_fn = pkg.IDG.DeGridW if wstack else pkg.IDG.DeGrid
    rng = np.random.default_rng(4)
    N = cd["grid_size"]
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    res = {}
    for access in (0, 1):
        part.plan.set_host_access(access)
        g = grid_fn(c, part, obs.vis, obs.uvw, obs.frequencies)
        grid_in = model.copy()
        out = np.full(obs.vis.shape, 7.0 + 7.0j)
        v = degrid_fn(c, part, grid_in, obs.uvw, obs.frequencies, out=out)
        res[access] = (g, v, grid_in)
    print("in place on this device:", part.plan.host_access())
    g0, v0, s0 = res[0]
    g1, v1, s1 = res[1]
    assert rel_l2(g1, g0) < 1e-6
    assert np.array_equal(v1, v0)
    assert np.array_equal(s1, s0)
    covered = np.zeros(obs.vis.shape[:2], bool)
    for s in part.plan.subgrids():
        covered[s["baseline_idx"], s["time_sample_start"]:s["time_sample_start"] + s["time_sample_count"]] = True
    assert (~covered).any(), "the workload should drop some samples (quirk P1)"
    assert np.all(v1[~covered] == 0)


def _layers_hit(part, N, S, W):
    """w layers AdderWStack.Add writes (AdderWStack.cs:38-51), from the plan's subgrids."""
    hit = set()
    for s in part.plan.subgrids():
        sx, sy, sw = int(s["u_pixel"]), int(s["v_pixel"]), int(s["w_lambda"])
        if sw < 0:
            sx, sy, sw = N - sx - S + 1, N - sy - S + 1, -sw - 1
        if 1 <= sx < N - S and 1 <= sy < N - S and sw < W:
            hit.add(sw)
    return hit


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
def test_grid_w_in_place_layer_groups_and_pinned_output(need_gpu, mode):
    """GridW in place grids the w layers other than the busiest first and writes them back while
    the busiest one grids; page-locked outputs are written by copy engines, pageable ones by
    kernels.  Every path must give the staged result, with unused layers exactly zero."""
    torch = pytest.importorskip("torch")
    obs, cd = workload("meerkat_3072", n_ant=10, nt=300, nch=16, seed=31)
    c, cd = constants(cd, grid_size=1024)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    N, S, W = cd["grid_size"], cd["subgrid_size"], cd["wlayer_count"]
    hit = _layers_hit(part, N, S, W)
    assert len(hit) >= 2, "the grouping needs subgrids in more than one layer"
    part.plan.set_host_access(0)
    ref = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    part.plan.set_host_access(1)
    for pinned in (True, False):
        if pinned:
            out = torch.empty((W, N, N), dtype=torch.complex128, pin_memory=True).numpy()
        else:
            out = np.empty((W, N, N), np.complex128)
        for _ in range(2):  # the second call reuses the plan's grouping and staging buffers
            out[...] = 5.0 - 3.0j
            got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies, out=out)
            assert np.shares_memory(got, out)
            assert rel_l2(out, ref) < 1e-6, (pinned, part.plan.host_access())
            for k in range(W):
                if k not in hit:
                    assert np.all(out[k] == 0), (pinned, k)


def test_grid_non_w_in_place_pinned_output(need_gpu):
    """Grid (one layer, no layer grouping) into page-locked and pageable outputs: copy-engine and
    kernel writeback both give the staged result."""
    torch = pytest.importorskip("torch")
    obs, cd = workload("meerkat_3072", n_ant=10, nt=300, nch=16, seed=31)
    c, cd = constants(cd, grid_size=1024)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(pkg.MODE_TC_BF16X3)
    N = cd["grid_size"]
    part.plan.set_host_access(0)
    ref = pkg.IDG.Grid(c, part, obs.vis, obs.uvw, obs.frequencies)
    part.plan.set_host_access(1)
    for pinned in (True, False):
        out = (torch.empty((N, N), dtype=torch.complex128, pin_memory=True).numpy() if pinned
               else np.empty((N, N), np.complex128))
        out[...] = 3.0 + 1.0j
        got = pkg.IDG.Grid(c, part, obs.vis, obs.uvw, obs.frequencies, out=out)
        assert np.shares_memory(got, out)
        assert rel_l2(out, ref) < 1e-6, pinned
