"""The tensor-core modes' w-term bounds (P9IDG_TC_MAX_W_TERM, P9IDG_TC_MAX_W_TERM2).

The tensor-core form writes the reference's phasor exp(i dw n(x, y)) (Gridder.cs:61-67,
143-145) as A(x) B(y) exp(i dw r(x, y)) and expands the last factor to first order (the term it
leaves out is at most (dw r)^2 / 2 per visibility and pixel) or, for |dw r| between TC_MAX_W_TERM
and TC_MAX_W_TERM2, to second order ((dw r)^3 / 6 left out).  A plan whose samples reach
|dw r| > TC_MAX_W_TERM2 keeps the FP32 kernels when a tensor-core mode is asked for.

The geometries here are wide fields (0.15 rad images) with the w coordinate scaled so that
max |dw| * max |r| lands just under or just over a limit.  CPU tests check the decision
(plan building and mode selection run on the host); GPU tests check the results against the
FP64 oracle: <= 1e-4 (the tensor-core bar) just under the limit, <= 1e-5 (the FP32 bar) for
the plan that fell back.
"""
import numpy as np
import pytest

from conftest import constants, oracle, pkg, rel_l2, synth, workload

TOL_TC = 1e-4
TOL_FP32 = 1e-5


def wide_field(eps):
    """A 256^2 wide-field observation (ImageSize 0.15 rad) whose w term is `eps` (None: as made)."""
    obs, cd = workload("small_256", n_ant=8, nt=300, nch=8)
    N = cd["grid_size"]
    uvw = obs.uvw.copy()
    uvw[..., :2] *= 0.05  # keeps every uv track inside the 256^2 grid at this cell size

    def consts(u):
        return constants(cd, scale_arcsec=float(np.float32(0.15 / N)), wstep=synth.wstep_for(u, obs.frequencies, 4),
                         wlayer_count=4)

    if eps is not None:
        c, _ = consts(uvw)
        part = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies)
        part.plan.set_mode(pkg.MODE_TC_BF16X3)
        uvw[..., 2] *= eps / part.plan.info()["tc_w_term"]
    c, d = consts(uvw)
    return obs, uvw, c, d


def test_w_term_decision():
    """Under TC_MAX_W_TERM the plan runs the first-order tensor-core form; between it and
    TC_MAX_W_TERM2 the second-order form; beyond, the FP32 kernels, with the reason in the
    last-error message.  FP32 asked for explicitly is kept as it is, and order 2 can be requested."""
    for eps, expect in ((0.9 * pkg.TC_MAX_W_TERM, 1), (1.1 * pkg.TC_MAX_W_TERM, 2),
                        (0.9 * pkg.TC_MAX_W_TERM2, 2), (1.1 * pkg.TC_MAX_W_TERM2, 0)):
        obs, uvw, c, d = wide_field(eps)
        part = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies)
        for mode in (pkg.MODE_TC_BF16X3, pkg.MODE_TC_FP16X3):
            got = part.plan.set_mode(mode)
            info = part.plan.info()
            assert info["requested_mode"] == mode
            assert info["tc_w_term"] == pytest.approx(eps, rel=1e-6)
            assert info["tc_order"] == expect
            if expect:
                assert got == mode
            else:
                assert got == pkg.MODE_FP32
                assert "FP32 kernels" in pkg._native.last_error()
        if expect == 1:
            part.plan.set_tc_order(2)
            assert part.plan.info()["tc_order"] == 2
            part.plan.set_tc_order(0)
            assert part.plan.info()["tc_order"] == 1
        assert part.plan.set_mode(pkg.MODE_FP32) == pkg.MODE_FP32
        assert part.plan.info()["requested_mode"] == pkg.MODE_FP32
        assert part.plan.info()["tc_order"] == 0


def test_w_term_of_the_3072_workload_is_far_below_the_limit():
    """The full 3072^2 geometry (2016 baselines x 2000 times x 16 channels): |dw r| ~ 3e-4, so
    the first-order term left out is ~5e-8 of a visibility's contribution."""
    uvw, freqs, cd = synth.build_geometry(synth.WORKLOADS["meerkat_3072"])
    c, _ = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, uvw, freqs)
    assert part.plan.set_mode(pkg.MODE_TC_BF16X3) == pkg.MODE_TC_BF16X3
    assert 0 < part.plan.info()["tc_w_term"] < 0.05 * pkg.TC_MAX_W_TERM


MODES = [pytest.param(pkg.MODE_TC_BF16X3, id="bf16x3"), pytest.param(pkg.MODE_TC_FP16X3, id="fp16x3")]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", MODES)
def test_tc_just_under_the_limit(need_gpu, mode):
    obs, uvw, c, d = wide_field(0.95 * pkg.TC_MAX_W_TERM)
    part = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies)
    assert part.plan.set_mode(mode) == mode
    subs = oracle.partition(d, uvw, obs.frequencies)
    got = pkg.IDG.GridW(c, part, obs.vis, uvw, obs.frequencies)
    ref = oracle.idg_grid_w(d, subs, obs.vis, uvw, obs.frequencies)
    assert rel_l2(got, ref) < TOL_TC
    rng = np.random.default_rng(7)
    N = d["grid_size"]
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    vis = pkg.IDG.DeGridW(c, part, model.copy(), uvw, obs.frequencies)
    vref, _ = oracle.idg_degrid(d, subs, model, uvw, obs.frequencies, wstack=True)
    assert rel_l2(vis, vref) < TOL_TC


def _grid_degrid_errors(mode, eps, order=0):
    obs, uvw, c, d = wide_field(eps)
    part = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies)
    assert part.plan.set_mode(mode) == mode
    part.plan.set_tc_order(order)
    subs = oracle.partition(d, uvw, obs.frequencies)
    got = pkg.IDG.GridW(c, part, obs.vis, uvw, obs.frequencies)
    ref = oracle.idg_grid_w(d, subs, obs.vis, uvw, obs.frequencies)
    rng = np.random.default_rng(7)
    N = d["grid_size"]
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    vis = pkg.IDG.DeGridW(c, part, model.copy(), uvw, obs.frequencies)
    vref, _ = oracle.idg_degrid(d, subs, model, uvw, obs.frequencies, wstack=True)
    return part.plan.info()["tc_order"], rel_l2(got, ref), rel_l2(vis, vref)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", MODES)
def test_tc_second_order_just_under_its_limit(need_gpu, mode):
    order, eg, ed = _grid_degrid_errors(mode, 0.95 * pkg.TC_MAX_W_TERM2)
    print(f"second-order form at 0.95 of its limit, mode {mode}: grid {eg:.2e}, degrid {ed:.2e}")
    assert order == 2 and eg < TOL_TC and ed < TOL_TC


@pytest.mark.gpu
@pytest.mark.parametrize("mode", MODES)
def test_tc_second_order_on_request_is_at_least_as_accurate(need_gpu, mode):
    """Asked for on a plan the first-order form covers, the second-order form leaves out less."""
    o1, g1, d1 = _grid_degrid_errors(mode, 0.95 * pkg.TC_MAX_W_TERM)
    o2, g2, d2 = _grid_degrid_errors(mode, 0.95 * pkg.TC_MAX_W_TERM, order=2)
    print(f"at 0.95 of the first-order limit, mode {mode}: first order {g1:.2e} / {d1:.2e}, "
          f"second order {g2:.2e} / {d2:.2e}")
    assert (o1, o2) == (1, 2)
    assert g2 < TOL_TC and d2 < TOL_TC
    assert g2 <= 1.05 * g1 and d2 <= 1.05 * d1


@pytest.mark.gpu
def test_tc_over_the_limit_runs_fp32(need_gpu):
    obs, uvw, c, d = wide_field(1.5 * pkg.TC_MAX_W_TERM2)
    part = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies)
    assert part.plan.set_mode(pkg.MODE_TC_BF16X3) == pkg.MODE_FP32
    subs = oracle.partition(d, uvw, obs.frequencies)
    got = pkg.IDG.GridW(c, part, obs.vis, uvw, obs.frequencies)
    assert rel_l2(got, oracle.idg_grid_w(d, subs, obs.vis, uvw, obs.frequencies)) < TOL_FP32


@pytest.mark.gpu
def test_tc_call_with_a_larger_w_is_refused(need_gpu):
    """The plan's own uvw passes the check; a call handing the same plan a uvw with 3x the w
    (beyond the limit) returns P9IDG_UNSUPPORTED from the coefficient kernel's check, and the
    plan's own uvw works again afterwards."""
    obs, uvw, c, d = wide_field(0.5 * pkg.TC_MAX_W_TERM)
    part = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies)
    assert part.plan.set_mode(pkg.MODE_TC_BF16X3) == pkg.MODE_TC_BF16X3
    big = uvw.copy()
    big[..., 2] *= 3.0
    with pytest.raises(pkg.P9IDGError) as e:
        pkg.IDG.GridW(c, part, obs.vis, big, obs.frequencies)
    assert e.value.code == 8
    subs = oracle.partition(d, uvw, obs.frequencies)
    got = pkg.IDG.GridW(c, part, obs.vis, uvw, obs.frequencies)
    assert rel_l2(got, oracle.idg_grid_w(d, subs, obs.vis, uvw, obs.frequencies)) < TOL_TC
