"""Data-parallel gridding over baselines: the reference's MPI layout on torch.distributed.

The reference shards the observation by contiguous baseline blocks
(Distributed-Reference/DistributedData.cs:94-96), grids each block locally
(MPIMajorCycle.cs:170, 208: IDG.Grid / IDG.GridPSF) and sums the N x N grids to rank 0
with Reduce(SequentialSum) (MPIMajorCycle.cs:173, 209, 221-232), broadcasting images
back (:106, 186-187, 215).  Here each rank partitions its own block (the partition is
per baseline, so the subgrids are those of the global plan for these baselines), grids
it on its GPU, and the grids (or w layers) are summed with one collective: NCCL on
device tensors, or gloo on host arrays.  Gridding is linear in the visibilities, so the
reduced grid equals the single-process grid up to summation order.
"""
from __future__ import annotations

import numpy as np


def baseline_block(nbl: int, world_size: int, rank: int) -> tuple[int, int]:
    """[begin, end) baselines of `rank`: equal blocks, the last rank takes the remainder
    (DistributedData.cs:94-96)."""
    if world_size <= 0 or not (0 <= rank < world_size):
        raise ValueError("invalid rank / world size")
    per = int(nbl / world_size)
    begin = rank * per
    end = (rank + 1) * per if rank + 1 < world_size else nbl
    return begin, end


def balanced_baseline_blocks(weights, world_size: int) -> list[tuple[int, int]]:
    """Contiguous [begin, end) baseline blocks, one per rank, with about equal total weight
    (e.g. gridded visibilities per baseline; the partitioner drops samples unevenly, so equal
    baseline counts would leave ranks with very different work).  Rank r's block ends at the
    baseline boundary whose running weight is closest to (r + 1) / world_size of the total; every
    block is contiguous, so each rank's partition is the global partition's subgrids of those
    baselines, in order."""
    w = np.asarray(weights, dtype=np.float64)
    if world_size <= 0:
        raise ValueError("invalid world size")
    if np.any(w < 0):
        raise ValueError("negative weight")
    nbl = len(w)
    cum = np.concatenate([[0.0], np.cumsum(w)])
    total = cum[-1]
    bounds = [0]
    for r in range(1, world_size):
        target = total * r / world_size
        b = int(np.searchsorted(cum, target, side="left"))
        if b > 0 and (b > nbl or target - cum[b - 1] <= cum[b] - target):
            b -= 1
        bounds.append(min(max(b, bounds[-1]), nbl))
    bounds.append(nbl)
    return [(bounds[r], bounds[r + 1]) for r in range(world_size)]


def gridded_per_baseline(subgrids, nbl: int, nch: int) -> np.ndarray:
    """Visibilities each baseline contributes to a plan's subgrids (time samples x channels)."""
    out = np.zeros(nbl, np.int64)
    np.add.at(out, np.asarray(subgrids["baseline_idx"], np.int64),
              np.asarray(subgrids["time_sample_count"], np.int64) * nch)
    return out


def local_block(arrays, nbl, world_size, rank):
    """Slices this rank's baselines out of [nbl, ...] arrays (uvw, visibilities, flags)."""
    b, e = baseline_block(nbl, world_size, rank)
    return [None if a is None else np.ascontiguousarray(a[b:e]) for a in arrays]


def _as_real_tensor(torch, arr):
    """A float64/float32 torch view of a complex numpy array (collectives sum real pairs)."""
    a = np.ascontiguousarray(arr)
    if np.iscomplexobj(a):
        a = a.view(np.float64 if a.dtype == np.complex128 else np.float32)
    return torch.from_numpy(a)


class GridReducer:
    """Sums grids across ranks (Reduce(SequentialSum) of MPIMajorCycle.cs:221-232)."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist

        self.torch = torch
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world_size = dist.get_world_size(group)
        # NCCL collectives take device tensors: host arrays go through the current GPU
        self.on_device = str(dist.get_backend(group)).lower() == "nccl"

    def _to_coll(self, t):
        return t.cuda() if self.on_device else t

    def _from_coll(self, t):
        return t.cpu() if self.on_device else t

    def sum_to_root(self, grid: np.ndarray, root: int = 0):
        """Host array (complex or real): the element-wise sum lands on `root` (None elsewhere)."""
        t = self._to_coll(_as_real_tensor(self.torch, grid).clone())
        self.dist.reduce(t, dst=root, op=self.dist.ReduceOp.SUM, group=self.group)
        if self.rank != root:
            return None
        out = self._from_coll(t).numpy()
        return out.view(grid.dtype).reshape(grid.shape) if np.iscomplexobj(grid) else out.reshape(grid.shape)

    def sum_all(self, grid: np.ndarray) -> np.ndarray:
        t = self._to_coll(_as_real_tensor(self.torch, grid).clone())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        out = self._from_coll(t).numpy()
        return out.view(grid.dtype).reshape(grid.shape) if np.iscomplexobj(grid) else out.reshape(grid.shape)

    def sum_device_(self, tensor):
        """In-place all-reduce of a device tensor (complex64 grids are summed as float pairs)."""
        t = self.torch.view_as_real(tensor) if tensor.is_complex() else tensor
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return tensor

    def sum_layers_device_(self, layers, root=None):
        """Dirty-image form of the grid reduce: WStackIFFTFloat applies no per-layer w correction
        (FFT.cs:188-215), so only the sum of the W layers matters.  Sums this rank's layers into
        layer 0 on the device, then reduces that one N x N grid across ranks (N^2 * 8 bytes for
        complex64, W times less than the layer stack): to every rank (root None) or to `root`.
        Returns layer 0 (the summed grid on the ranks that receive it)."""
        grid = layers[0]
        for w in range(1, layers.shape[0]):
            grid.add_(layers[w])
        t = self.torch.view_as_real(grid) if grid.is_complex() else grid
        if root is None:
            self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        else:
            self.dist.reduce(t, dst=root, op=self.dist.ReduceOp.SUM, group=self.group)
        return grid

    def broadcast_device_(self, tensor, root: int = 0):
        """In-place broadcast of a device (or, with gloo, host) tensor from `root`: the model grid
        every rank degrids (MPIMajorCycle.cs:106)."""
        t = self.torch.view_as_real(tensor) if tensor.is_complex() else tensor
        self.dist.broadcast(t, src=root, group=self.group)
        return tensor

    def broadcast(self, arr, root: int = 0):
        """Host array from `root` to every rank (MPIMajorCycle.cs:106, 186-187, 215)."""
        t = self._to_coll(_as_real_tensor(self.torch, arr).clone())
        self.dist.broadcast(t, src=root, group=self.group)
        out = self._from_coll(t).numpy()
        return out.view(arr.dtype).reshape(arr.shape) if np.iscomplexobj(arr) else out.reshape(arr.shape)


def distributed_grid(reducer: GridReducer, c, uvw_all, vis_all, frequencies, gridder, root: int = 0,
                     partitioner=None):
    """ForwardCalculateB's gridding half (MPIMajorCycle.cs:160-174): partition and grid this
    rank's baseline block with `gridder(c, partition, vis, uvw, freq)`, then sum to `root`.

    `partitioner(c, uvw, freq)` defaults to Partitioner.CreatePartition of this package."""
    uvw, vis = local_block([uvw_all, vis_all], uvw_all.shape[0], reducer.world_size, reducer.rank)
    if partitioner is None:
        from .idg import Partitioner
        partitioner = Partitioner.CreatePartition
    part = partitioner(c, uvw, frequencies)
    local = gridder(c, part, vis, uvw, frequencies)
    return reducer.sum_to_root(np.ascontiguousarray(local), root)
