"""The NCCL form of the grid reduce, run as one rank on one GPU (the only multi-GPU form a
single-GPU machine can run): the w layers gridded on the device by the tensor-core kernels are
summed in place over an NCCL process group (complex64 as float pairs), host arrays are
reduced and broadcast through the GPU, and everything must come back unchanged with one rank.  The collective
logic across several ranks is covered by the two-rank gloo test."""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(port, q):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import __graft_entry__ as entry

    pkg = entry.load_package()
    synth = entry._load_module(entry.PKG_NAME + ".synth", os.path.join(entry.PKG_DIR, "synth.py"))
    dist_mod = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
    os.environ["NCCL_NVLS_ENABLE"] = "0"  # no NVLink multicast objects
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        obs, cd = synth.build(synth.scaled_workload("small_256", n_ant=9, nt=200, nch=4))
        c = pkg.GriddingConstants.from_dict(cd)
        part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
        part.plan.set_mode(pkg.MODE_TC_BF16X3)
        N, W = cd["grid_size"], cd["wlayer_count"]
        d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
        d_layers = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")
        part.plan.grid_w_device(d_vis.data_ptr(), d_layers.data_ptr())
        part.plan.synchronize()
        before = d_layers.cpu().numpy()
        red = dist_mod.GridReducer()
        red.sum_device_(d_layers)
        torch.cuda.synchronize()
        after = d_layers.cpu().numpy()
        host = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
        model = np.arange(12.0).reshape(3, 4)
        got = red.broadcast(model, root=0)
        # the host-array forms stage through the GPU for NCCL
        host_ok = (np.array_equal(red.sum_to_root(host, root=0), host) and
                   np.array_equal(red.sum_all(np.full((2, 2), 2.5)), np.full((2, 2), 2.5)))
        err = float(np.linalg.norm(after - host) / np.linalg.norm(host))
        q.put(("ok", bool(np.array_equal(after, before)), err, bool(np.array_equal(got, model) and host_ok)))
    except Exception as e:  # report to the parent instead of hanging it
        q.put(("error", repr(e), None, None))
        raise
    finally:
        dist.destroy_process_group()


def test_nccl_one_rank_device_reduce(need_gpu):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_rank_main, args=(_free_port(), q))
    p.start()
    try:
        status, unchanged, err, bcast = q.get(timeout=240)
    finally:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    assert status == "ok", unchanged
    assert unchanged  # one rank: the all-reduce leaves the device layers as they were
    assert err < 1e-6  # and they equal the host API's layers
    assert bcast
    assert p.exitcode == 0
