"""Batched multi-problem launches (one launch per kernel stage over several plans), their
CUDA-graph replay, per-problem completion latencies, and the autotuner.

A batch must produce, for every problem, what the problem's own plan produces through the
single-plan device entry points (same kernels and work items; only the FP32 atomics of
the adder may sum in another order)."""
import numpy as np
import pytest

from conftest import constants, pkg, rel_l2, synth

pytestmark = pytest.mark.gpu


def _problems(torch, mode, sizes=None):
    specs = [("small_256", dict(n_ant=8, nt=300, nch=8, seed=21), dict(grid_size=256)),
             ("meerkat_3072", dict(n_ant=9, nt=200, nch=12, seed=22), dict(grid_size=1024)),
             ("small_256", dict(n_ant=6, nt=500, nch=4, seed=23), dict(grid_size=384))]
    if sizes:  # per-problem subgrid size and kernel size
        specs = [(n, kw, dict(o, subgrid_size=S, kernel_size=k)) for (n, kw, o), (S, k) in zip(specs, sizes)]
    out = []
    for name, kw, over in specs:
        obs, cd = synth.build(synth.scaled_workload(name, **kw))
        c, cd = constants(cd, **over)
        part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
        part.plan.set_mode(mode)
        N, W = cd["grid_size"], cd["wlayer_count"]
        g = torch.Generator(device="cuda").manual_seed(len(out))
        bufs = dict(vis=torch.from_numpy(obs.vis.astype(np.complex64)).cuda(),
                    layers=torch.empty((W, N, N), dtype=torch.complex64, device="cuda"),
                    grid=torch.randn((N, N), dtype=torch.complex64, device="cuda", generator=g),
                    out=torch.empty(obs.vis.shape, dtype=torch.complex64, device="cuda"))
        out.append((part, cd, bufs, obs))
    return out


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3, pkg.MODE_TC_FP16X3],
                         ids=["fp32", "tc_bf16x3", "tc_fp16x3"])
def test_batch_matches_single_plans(need_gpu, mode):
    torch = pytest.importorskip("torch")
    probs = _problems(torch, mode)
    refs = []
    for part, cd, b, _ in probs:
        plan = part.plan
        lay = torch.empty_like(b["layers"])
        vo = torch.empty_like(b["out"])
        plan.grid_w_device(b["vis"].data_ptr(), lay.data_ptr())
        plan.degrid_w_device(b["grid"].data_ptr(), vo.data_ptr())
        plan.synchronize()
        refs.append((lay.cpu().numpy(), vo.cpu().numpy()))
    batch = pkg.Batch([p.plan for p, _, _, _ in probs], [b["vis"].data_ptr() for _, _, b, _ in probs],
                      [b["layers"].data_ptr() for _, _, b, _ in probs], [b["grid"].data_ptr() for _, _, b, _ in probs],
                      [b["out"].data_ptr() for _, _, b, _ in probs])
    for replay in (False, True):
        for _, _, b, _ in probs:
            b["layers"].fill_(7.0)
            b["out"].fill_(7.0)
        if replay:
            batch.capture_graph()
            for _, _, b, _ in probs:  # the capture ran the batch once: reset outputs before the replay
                b["layers"].fill_(7.0)
                b["out"].fill_(7.0)
        torch.cuda.synchronize()
        batch.run()
        batch.synchronize()
        for (part, cd, b, _), (lay, vo) in zip(probs, refs):
            assert rel_l2(b["layers"].cpu().numpy(), lay) < 1e-6
            assert rel_l2(b["out"].cpu().numpy(), vo) < 1e-6
        lat = batch.latencies_ms()
        assert np.all(lat > 0) and np.all(lat < 10_000)
    batch.destroy()


def test_small_first_schedule(need_gpu):
    """The SMALL_FIRST order gives the same results and finishes the smallest problem first."""
    torch = pytest.importorskip("torch")
    probs = _problems(torch, pkg.MODE_TC_BF16X3)
    batch = pkg.Batch([p.plan for p, _, _, _ in probs], [b["vis"].data_ptr() for _, _, b, _ in probs],
                      [b["layers"].data_ptr() for _, _, b, _ in probs], [b["grid"].data_ptr() for _, _, b, _ in probs],
                      [b["out"].data_ptr() for _, _, b, _ in probs])
    batch.run()
    batch.synchronize()
    ref = [(b["layers"].cpu().numpy(), b["out"].cpu().numpy()) for _, _, b, _ in probs]
    batch.set_schedule(pkg.Batch.SMALL_FIRST)
    batch.capture_graph()
    batch.run()
    batch.synchronize()
    for (_, _, b, _), (lay, vo) in zip(probs, ref):
        assert rel_l2(b["layers"].cpu().numpy(), lay) < 1e-6
        assert rel_l2(b["out"].cpu().numpy(), vo) < 1e-6
    sizes = [p.plan.info()["gridded_visibilities"] for p, _, _, _ in probs]
    lat = batch.latencies_ms()
    assert lat[int(np.argmin(sizes))] <= lat[int(np.argmax(sizes))]
    batch.destroy()


def test_batch_rejects_mixed_modes(need_gpu):
    torch = pytest.importorskip("torch")
    obs, cd = synth.build(synth.scaled_workload("small_256", n_ant=5, nt=50, nch=4))
    plans = []
    for mode in (pkg.MODE_FP32, pkg.MODE_TC_BF16X3):
        c, _ = constants(cd)
        plans.append(pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies).plan)
        plans[-1].set_mode(mode)
    buf = torch.empty(4, dtype=torch.complex64, device="cuda").data_ptr()
    with pytest.raises(pkg.P9IDGError) as e:
        pkg.Batch(plans, [buf] * 2, [buf] * 2, [buf] * 2, [buf] * 2)
    assert e.value.code == 8


def test_autotune_picks_a_valid_configuration(need_gpu):
    obs, cd = synth.build(synth.scaled_workload("meerkat_3072", n_ant=12, nt=400, nch=16))
    c, cd = constants(cd)
    t = pkg.autotune(c, obs.uvw, obs.frequencies, pkg.MODE_FP32, [24, 32, 48])
    assert t["subgrid_size"] in (24, 32, 48)
    assert t["gridder_max_vis"] in (512, 1024, 2048) and t["degridder_max_vis"] in (256, 512, 1024)
    assert 0 < t["seconds_per_gridded_vis"] < 1e-3 and 0 < t["gridded_fraction"] <= 1
    t2 = pkg.autotune(c, obs.uvw, obs.frequencies, pkg.MODE_TC_BF16X3, None)
    assert t2["subgrid_size"] in (24, 32) and t2["gridder_max_vis"] in (2048, 4096, 8192)
    # the chosen work-item sizes leave results unchanged
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    before = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    pkg.set_chunking(part.plan, t["gridder_max_vis"], t["degridder_max_vis"])
    after = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(after, before) < 1e-6


@pytest.mark.parametrize("mode,sizes,tol", [
    (pkg.MODE_FP32, [(16, 4), (48, 8), (24, 8)], 1e-5),
    (pkg.MODE_TC_BF16X3, [(16, 4), (32, 8), (24, 8)], 1e-4),
    (pkg.MODE_TC_FP16X3, [(24, 8), (8, 2), (32, 8)], 1e-4)], ids=["fp32", "tc_bf16x3", "tc_fp16x3"])
def test_batch_mixes_subgrid_sizes_against_the_oracle(need_gpu, mode, sizes, tol):
    """A batch whose problems use different subgrid sizes (one launch per kernel stage and size)
    reproduces every problem's GridW and DeGridW of the FP64 oracle, to the mode's bound."""
    import oracle

    torch = pytest.importorskip("torch")
    probs = _problems(torch, mode, sizes=sizes)
    batch = pkg.Batch([p.plan for p, _, _, _ in probs], [b["vis"].data_ptr() for _, _, b, _ in probs],
                      [b["layers"].data_ptr() for _, _, b, _ in probs],
                      [b["grid"].data_ptr() for _, _, b, _ in probs], [b["out"].data_ptr() for _, _, b, _ in probs])
    batch.capture_graph()
    batch.run()
    batch.synchronize()
    for part, cd, b, obs in probs:
        subs = oracle.partition(cd, obs.uvw, obs.frequencies)
        assert np.array_equal(part.plan.subgrids(), subs)
        ref = oracle.idg_grid_w(cd, subs, obs.vis.astype(np.complex64).astype(np.complex128), obs.uvw,
                                obs.frequencies)
        # the device API leaves the layers shifted (FFT.Shift folded into the adder), as GridW returns them
        assert part.plan.info()["mode"] == mode
        assert rel_l2(b["layers"].cpu().numpy(), ref) < tol
        grid = b["grid"].cpu().numpy().astype(np.complex128)
        vref, _ = oracle.idg_degrid(cd, subs, grid, obs.uvw, obs.frequencies, wstack=True)
        assert rel_l2(b["out"].cpu().numpy(), vref) < tol
    batch.destroy()
