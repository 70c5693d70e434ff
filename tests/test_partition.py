"""Partitioner.CreatePartition: hand-derived known answers, oracle vs product planner.

The product planner runs on the host (no GPU), so these are CPU tests.  Subgrid lists
must be bit-identical: they decide which visibilities are gridded at all.
"""
import json
import os

import numpy as np
import pytest

from conftest import C_LIGHT, kat_constants, oracle, pkg, synth, workload

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "partition_kat.json")
ERRORS = {"CANNOT_PLACE": 2, "SUBGRID_OUT_OF_GRID": 3}


def _cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


def _case_inputs(case):
    uvw = np.array([[[float(v) for v in s] for s in bl] for bl in case["uvw"]], np.float64)
    if uvw.ndim != 3:
        uvw = uvw.reshape(len(case["uvw"]), 0, 3)
    freq = np.array(case["freq_over_c"], np.float64) * C_LIGHT
    cd = kat_constants(max_t=case["max_t"], W=case["W"], wstep=case["wstep"])
    return cd, uvw, freq


def _rows(arr):
    return [[int(r[k]) for k in arr.dtype.names] for r in arr]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_known_answers_oracle(case):
    cd, uvw, freq = _case_inputs(case)
    if "error" in case:
        with pytest.raises(oracle.OracleError) as e:
            oracle.partition(cd, uvw, freq)
        assert e.value.code == ERRORS[case["error"]]
    else:
        assert _rows(oracle.partition(cd, uvw, freq)) == case["expect"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_known_answers_product(case):
    cd, uvw, freq = _case_inputs(case)
    c = pkg.GriddingConstants.from_dict(cd)
    if "error" in case:
        with pytest.raises(pkg.P9IDGError) as e:
            pkg.Partitioner.CreatePartition(c, uvw, freq)
        assert e.value.code == ERRORS[case["error"]]
        if case["error"] == "CANNOT_PLACE":
            assert "could not place" in str(e.value)
    else:
        part = pkg.Partitioner.CreatePartition(c, uvw, freq)
        assert _rows(part.plan.subgrids()) == case["expect"]
        # List<List<Subgrid>> shape: one list per baseline
        assert len(part) == uvw.shape[0]
        flat = [[s.baselineIdx, s.timeSampleStart, s.timeSampleCount, s.UPixel, s.VPixel, s.WLambda]
                for lst in part for s in lst]
        assert flat == case["expect"]


@pytest.mark.parametrize("name,kw", [
    ("small_256", dict(n_ant=12, nt=600, nch=8)),
    ("meerkat_3072", dict(n_ant=16, nt=500, nch=16)),
    ("meerkat_3072", dict(n_ant=10, nt=300, nch=3)),
])
def test_product_planner_matches_oracle(name, kw):
    obs, cd = workload(name, **kw)
    c = pkg.GriddingConstants.from_dict(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    got = part.plan.subgrids()
    ref = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert len(got) == len(ref)
    assert np.array_equal(got.view(np.int32), ref.view(np.int32))


def test_product_planner_full_size_3072():
    """The full 2016-baseline x 2000-time x 16-channel track set (uvw only)."""
    w = synth.WORKLOADS["meerkat_3072"]
    o = w["obs"]
    rng = np.random.default_rng(o["seed"])
    ants = synth.antennas_log_radial(rng, o["n_ant"], o["array_diameter_m"])
    uvw = synth.earth_rotation_uvw(ants, -30.7215, -70.0, o["nt"], o["dump_s"])
    freq = np.linspace(o["f_lo"], o["f_hi"], o["nch"])
    cd = dict(vis_count=1, grid_size=o["grid_size"], subgrid_size=32, kernel_size=8, max_timesteps=1024,
              scale_arcsec=float(np.float32(synth.cell_rad(o["cell_arcsec"]))), wlayer_count=8,
              wstep=synth.wstep_for(uvw, freq, 8))
    part = pkg.Partitioner.CreatePartition(pkg.GriddingConstants.from_dict(cd), uvw, freq)
    got = part.plan.subgrids()
    ref = oracle.partition(cd, uvw, freq)
    assert np.array_equal(got.view(np.int32), ref.view(np.int32))
    info = part.plan.info()
    assert info["input_visibilities"] == 2016 * 2000 * 16
    assert info["gridded_visibilities"] == int(ref["time_sample_count"].sum()) * 16
    # quirk P1 drops long-baseline samples: report both counts
    assert info["gridded_visibilities"] < info["input_visibilities"]


def test_no_channels_is_invalid():
    cd = kat_constants()
    with pytest.raises(pkg.P9IDGError) as e:
        pkg.Partitioner.CreatePartition(pkg.GriddingConstants.from_dict(cd), np.zeros((1, 2, 3)), np.zeros(0))
    assert e.value.code == 1


def test_no_baselines():
    cd = kat_constants()
    part = pkg.Partitioner.CreatePartition(pkg.GriddingConstants.from_dict(cd), np.zeros((0, 5, 3)),
                                           np.array([C_LIGHT]))
    assert len(part) == 0 and len(part.plan.subgrids()) == 0


def test_plan_from_caller_subgrids_validates():
    cd = kat_constants()
    c = pkg.GriddingConstants.from_dict(cd)
    bad = np.array([(0, 3, 5, 24, 24, 0)], pkg.SUBGRID_DTYPE)  # samples 3..7 of a 4-sample track
    with pytest.raises(pkg.P9IDGError) as e:
        pkg.plan_from_subgrids(c, bad, np.zeros((1, 4, 3)), np.array([C_LIGHT]))
    assert e.value.code == 1
