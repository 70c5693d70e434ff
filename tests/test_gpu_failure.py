"""Failure paths, made to happen without faulting the GPU.

* Out of memory: p9idg_debug_fail_device_allocations makes the library's device allocations
  fail as cudaMalloc does when memory runs out.  Armed at every allocation point of a GridW /
  DeGridW call in turn, each call must return P9IDG_OUT_OF_MEMORY (or succeed once the point
  lies past the call's last allocation), the same plan must work once memory is back, and
  destroying the plans must give every byte back.
"""
import numpy as np
import pytest

from conftest import constants, oracle, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu
OOM = 5


def _arm(after):
    assert pkg._native.lib().p9idg_debug_fail_device_allocations(after) == 0


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
def test_out_of_memory_at_every_allocation_point(need_gpu, mode):
    torch = pytest.importorskip("torch")
    obs, cd = workload("small_256", n_ant=6, nt=120, nch=4)
    c, cd = constants(cd)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    vref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    try:
        for k in range(200):
            part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
            assert part.plan.set_mode(mode) == mode
            _arm(k)
            try:
                pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
                pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
                done = True
            except pkg.P9IDGError as e:
                assert e.code == OOM, (k, e.code, str(e))
                failures += 1
                done = False
            _arm(-1)
            # the same plan works once memory is available again
            assert rel_l2(pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies), ref) < 1e-4
            assert rel_l2(pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies), vref) < 1e-4
            part.plan.destroy()
            if done:
                break
        else:
            pytest.fail("the calls never ran to completion")
    finally:
        _arm(-1)
    assert failures >= 5  # the calls make several device allocations; each was made to fail once
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) <= 4 << 20  # every plan gave its memory back


MODES = [pytest.param(pkg.MODE_TC_BF16X3, id="bf16x3"), pytest.param(pkg.MODE_TC_FP16X3, id="fp16x3")]


@pytest.mark.parametrize("mode", MODES)
def test_tc_wait_runs_out_and_the_next_call_is_right(need_gpu, mode):
    """Bounded waits: with a 1 ms limit and the loader warp never delivering input stage 1 of each
    work item, the consumers' waits run out; every kernel gives up, frees its tensor memory once
    its issued MMAs have finished, and the call returns P9IDG_DEVICE_CHECK_FAILED.  Both loaders
    are covered: the TMA one (complex64 staging) and the cp.async one (complex128 host arrays
    read in place).  The next ordinary calls on the same plan match the FP64 oracle."""
    obs, cd = workload("small_256", n_ant=8, nt=300, nch=8)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    assert part.plan.set_mode(mode) == mode
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert int(subs["time_sample_count"].max()) * cd_nch(obs) > 2 * 128  # items with >= 2 stages / tiles
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    vref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    L = pkg._native.lib()
    for in_place in (True, False):
        part.plan.set_host_access(in_place)
        assert L.p9idg_debug_tc_wait(1_000_000, 1) == 0
        try:
            with pytest.raises(pkg.P9IDGError) as e:
                pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
            assert e.value.code == 9
            with pytest.raises(pkg.P9IDGError) as e:
                pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
            assert e.value.code == 9
        finally:
            assert L.p9idg_debug_tc_wait(0, -1) == 0
        assert rel_l2(pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies), ref) < 1e-4
        assert rel_l2(pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies), vref) < 1e-4


def cd_nch(obs):
    return obs.vis.shape[2]
