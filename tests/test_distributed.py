"""Baseline-sharded gridding with a grid reduce, as the reference's MPI driver does
(DistributedData.cs:94-96, MPIMajorCycle.cs:160-174), run as two gloo ranks on the CPU.

Each rank partitions and grids its own baseline block; the per-rank gridder here is the FP64
oracle (the collective logic is what is under test, and no GPU is needed).  The reduced grid
must equal the single-process grid of all baselines.  The second test runs the sharded path
`bench.py --gpus N` times: blocks balanced by gridded visibilities, the product's partitioner on
each block, the w layers summed on each rank and one N x N grid reduced, then the model grid
broadcast.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import __graft_entry__ as entry
    import oracle

    pkg = entry.load_package()
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
    dist_mod = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        obs, cd = synth.build(synth.scaled_workload("small_256", n_ant=9, nt=200, nch=4))
        c = pkg.GriddingConstants.from_dict(cd)
        red = dist_mod.GridReducer()

        def part_fn(c_, uvw, freq):
            return oracle.partition(cd, uvw, freq)

        def grid_fn(c_, subs, vis, uvw, freq):
            return oracle.idg_grid(cd, subs, vis, uvw, freq)

        total = dist_mod.distributed_grid(red, c, obs.uvw, obs.vis, obs.frequencies, grid_fn, root=0,
                                          partitioner=part_fn)
        img = red.broadcast(np.arange(6.0).reshape(2, 3) * (1 if rank == 0 else 0), root=0)
        both = red.sum_all(np.full((2, 2), rank + 1.0))
        if rank == 0:
            full = oracle.idg_grid(cd, oracle.partition(cd, obs.uvw, obs.frequencies), obs.vis, obs.uvw,
                                   obs.frequencies)
            err = np.linalg.norm(total - full) / np.linalg.norm(full)
            q.put(("ok", float(err), img.tolist(), both.tolist()))
    except Exception as e:  # report to the parent instead of hanging it
        q.put(("error", repr(e), None, None))
        raise
    finally:
        dist.destroy_process_group()


def test_baseline_blocks_match_reference_split():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as entry

    d = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
    assert [d.baseline_block(10, 3, r) for r in range(3)] == [(0, 3), (3, 6), (6, 10)]
    assert [d.baseline_block(435, 2, r) for r in range(2)] == [(0, 217), (217, 435)]
    with pytest.raises(ValueError):
        d.baseline_block(10, 2, 2)


def test_two_rank_grid_reduce_equals_single_process():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        status, err, img, both = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert status == "ok", err
    assert err < 1e-12
    assert img == [[0.0, 1.0, 2.0], [3.0, 4.0, 5.0]]
    assert both == [[3.0, 3.0], [3.0, 3.0]]
    assert all(p.exitcode == 0 for p in procs)


def _rank_main_layers(rank, world, port, q):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import __graft_entry__ as entry
    import oracle

    pkg = entry.load_package()
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
    dist_mod = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        obs, cd = synth.build(synth.scaled_workload("small_256", n_ant=9, nt=200, nch=4))
        c = pkg.GriddingConstants.from_dict(cd)
        nbl, nch = obs.uvw.shape[0], len(obs.frequencies)
        glob = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies).plan.subgrids()
        blocks = dist_mod.balanced_baseline_blocks(dist_mod.gridded_per_baseline(glob, nbl, nch), world)
        b, e = blocks[rank]
        uvw, vis = np.ascontiguousarray(obs.uvw[b:e]), np.ascontiguousarray(obs.vis[b:e])
        subs = pkg.Partitioner.CreatePartition(c, uvw, obs.frequencies).plan.subgrids()
        # the block's partition is the global partition's subgrids of these baselines
        mine = glob[(glob["baseline_idx"] >= b) & (glob["baseline_idx"] < e)].copy()
        mine["baseline_idx"] -= b
        same = bool(np.array_equal(subs, mine))
        red = dist_mod.GridReducer()
        layers = torch.from_numpy(oracle.idg_grid_w(cd, subs, vis, uvw, obs.frequencies).astype(np.complex64))
        grid = red.sum_layers_device_(layers).numpy().copy()
        model = torch.zeros((4, 4), dtype=torch.complex64)
        if rank == 0:
            model += torch.arange(16, dtype=torch.float32).reshape(4, 4) * (1 + 1j)
        red.broadcast_device_(model, root=0)
        if rank == 0:
            full = oracle.idg_grid_w(cd, glob, obs.vis, obs.uvw, obs.frequencies).sum(axis=0)
            err = float(np.linalg.norm(grid - full) / np.linalg.norm(full))
            q.put(("ok", err, blocks, same, model.numpy().tolist()))
        else:
            q.put(("rank1", None, blocks, same, model.numpy().tolist()))
    except Exception as ex:  # report to the parent instead of hanging it
        q.put(("error", repr(ex), None, None, None))
        raise
    finally:
        dist.destroy_process_group()


def test_balanced_blocks():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as entry

    d = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
    assert d.balanced_baseline_blocks([1] * 10, 3) == [(0, 3), (3, 7), (7, 10)]
    assert d.balanced_baseline_blocks([1, 1, 1, 1, 10, 1, 1, 1], 2) == [(0, 4), (4, 8)]
    assert d.balanced_baseline_blocks([0, 0, 5], 3) == [(0, 2), (2, 3), (3, 3)]
    w = np.random.default_rng(1).integers(0, 100, 500)
    bl = d.balanced_baseline_blocks(w, 8)
    assert bl[0][0] == 0 and bl[-1][1] == 500 and all(bl[i][1] == bl[i + 1][0] for i in range(7))
    loads = [w[a:b].sum() for a, b in bl]
    assert max(loads) - min(loads) <= 2 * w.max()
    with pytest.raises(ValueError):
        d.balanced_baseline_blocks([1, -1], 2)


def test_two_rank_sharded_grid_w_with_layer_sum_reduce():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main_layers, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = [q.get(timeout=240) for _ in range(2)]
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    errs = [r for r in res if r[0] == "error"]
    assert not errs, errs
    ok = [r for r in res if r[0] == "ok"][0]
    assert ok[1] < 1e-6  # complex64 layers summed across ranks vs the single-process FP64 layer sum
    assert all(r[3] for r in res)  # each block's partition = the global partition of its baselines
    blocks = ok[2]
    assert blocks[0][0] == 0 and blocks[0][1] == blocks[1][0] and 0 < blocks[0][1] < blocks[1][1]
    expect = (np.arange(16).reshape(4, 4) * (1 + 1j)).tolist()
    assert all(r[4] == expect for r in res)
    assert all(p.exitcode == 0 for p in procs)
