"""Distinct plans on distinct host threads (the C ABI is thread-safe across plans and not
re-entrant on one plan): four threads, each driving its own plan (two precision modes, two
observations) through IDG.GridW / IDG.DeGridW several times at once, must each get exactly what
the same plan produces alone.  ctypes releases the GIL for the duration of every library call,
so the calls overlap on the host and their streams on the GPU."""
import threading

import numpy as np
import pytest

from conftest import constants, oracle, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu


def test_plans_on_concurrent_threads(need_gpu):
    jobs = []
    for k, (name, kw, mode) in enumerate([("small_256", dict(n_ant=8, nt=300, nch=8, seed=31), pkg.MODE_FP32),
                                          ("small_256", dict(n_ant=8, nt=300, nch=8, seed=31), pkg.MODE_TC_BF16X3),
                                          ("small_256", dict(n_ant=10, nt=200, nch=16, seed=32), pkg.MODE_FP32),
                                          ("small_256", dict(n_ant=10, nt=200, nch=16, seed=32),
                                           pkg.MODE_TC_BF16X3)]):
        obs, cd = workload(name, **kw)
        c, cd = constants(cd)
        part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
        assert part.plan.set_mode(mode) == mode
        rng = np.random.default_rng(k)
        N = cd["grid_size"]
        model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        alone = (pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies),
                 pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies))
        jobs.append((c, part, obs, model, alone, cd))
    errors = []

    def worker(job):
        c, part, obs, model, (lay0, vis0), _ = job
        try:
            for _ in range(4):
                lay = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
                vis = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
                # the adder's FP32 atomics may sum in another order; nothing else may differ
                if not (rel_l2(lay, lay0) < 1e-6 and np.array_equal(vis, vis0)):
                    errors.append((part.plan.info()["mode"], rel_l2(lay, lay0), rel_l2(vis, vis0)))
        except Exception as e:  # reported below, in the test's own thread
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(j,)) for j in jobs]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors
    # the results they reproduce are right, not only repeatable
    c, part, obs, _, (lay0, _), cd = jobs[0]
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert rel_l2(lay0, oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < 1e-5
