"""Multi-GPU sharding of a basis build (one process per GPU).

Coarse cells are independent (the reference builds each rank's cells with no
exchange, source/Q/q_global.cc:50-86), so a batch is split into contiguous
cell ranges balanced by fine DoF x RHS, each rank builds its range on its own
GPU, and nothing crosses ranks during the build. The one collective is the
gather of the small per-cell Galerkin blocks (64 + 8 doubles per Q1 cell,
324 + 18 per Ned_RT, 400 + 20 per Q_Ned, 49 + 7 per RT_DQ cell) for the
global coarse assembly, which every rank
then holds in full. Timing of a sharded step is the maximum over ranks.

The helpers take the per-rank builder and the process group as arguments so
that the same code runs over NCCL with the GPU library and over gloo on CPU:
the tensors they exchange live on the current CUDA device when the group's
backend is NCCL (which accepts CUDA tensors only) and on the host otherwise.
"""
from __future__ import annotations

import numpy as np


def cell_work(cells, kind):
    """Fine DoF x RHS of every cell (the measures of the benchmark's workloads):
    Q1 8 (n+1)^3, Ned_RT 18 (N_edge + N_face), Q_Ned 20 (N_vertex + N_edge),
    RT_DQ 6 (N_face + N_cell)."""
    n = 1 << np.asarray(cells["depth"]).astype(np.int64)
    n_edge, n_face = 3 * n * (n + 1) ** 2, 3 * n * n * (n + 1)
    if kind == "q1":
        return (n + 1) ** 3 * 8
    if kind == "nedrt":
        return (n_edge + n_face) * 18
    if kind == "qned":
        return ((n + 1) ** 3 + n_edge) * 20
    if kind == "rtdq":
        return (n_face + n ** 3) * 6
    raise ValueError(f"unknown pairing {kind!r}")


def partition(work, world, rank):
    """Contiguous cell range [lo, hi) of `rank`: boundaries at the cumulative
    work quantiles r / world (every cell in exactly one range, ranges in rank
    order, possibly empty when cells are fewer than ranks)."""
    w = np.asarray(work, dtype=np.float64)
    cum = np.concatenate([[0.0], np.cumsum(w)])
    b = [int(np.searchsorted(cum, cum[-1] * r / world, side="left")) for r in range(world + 1)]
    b[0], b[-1] = 0, len(w)
    for r in range(1, world + 1):
        b[r] = max(b[r], b[r - 1])
    return b[rank], b[rank + 1]


def fine_offsets(cells):
    """Offsets of every cell's n^3 fine-cell values in the concatenated arrays."""
    n = 1 << np.asarray(cells["depth"]).astype(np.int64)
    return np.concatenate([[0], np.cumsum(n ** 3)])


def exchange_device(dist, group=None):
    """Device of the tensors a collective of `group` exchanges: the current
    CUDA device for the NCCL backend, the host for every other backend."""
    import torch
    if str(dist.get_backend(group)).lower() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def gather_blocks(local, dist, group=None):
    """All-gather per-rank arrays of per-cell blocks (leading axis = cells of
    the rank's range, in rank order) into the full array on every rank."""
    import torch
    world = dist.get_world_size(group)
    dev = exchange_device(dist, group)
    t = torch.from_numpy(np.ascontiguousarray(local)).to(dev)
    counts = torch.tensor([t.shape[0]], dtype=torch.int64, device=dev)
    all_counts = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(all_counts, counts, group=group)
    cmax = int(max(int(c.item()) for c in all_counts))
    pad = torch.zeros((cmax,) + tuple(t.shape[1:]), dtype=t.dtype, device=dev)
    pad[: t.shape[0]] = t
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return np.concatenate([p[: int(c.item())].cpu().numpy() for p, c in zip(parts, all_counts)])


def max_over_ranks(x, dist=None, group=None):
    """Maximum of a per-rank scalar (the time of a sharded step)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=exchange_device(dist, group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def weak_scaling_value(work_local, seconds_local, dist=None, group=None):
    """Whole-job throughput of a weak-scaling step in which every rank builds
    its own batch of independent cells: the work of all ranks divided by the
    slowest rank's time (no data-path collective; only these two scalars are
    reduced)."""
    if dist is None:
        return float(work_local) / float(seconds_local)
    import torch
    w = torch.tensor([float(work_local)], dtype=torch.float64, device=exchange_device(dist, group))
    dist.all_reduce(w, op=dist.ReduceOp.SUM, group=group)
    return float(w.item()) / max_over_ranks(seconds_local, dist, group)


def build_sharded(build, cells, fine_arrays, kind, world, rank, dist=None, group=None):
    """Build this rank's share of `cells` with `build(cells_slice, arrays_slice)
    -> (KH, FH)` and return the full (KH, FH) of the batch on every rank.
    `fine_arrays` are per-fine-cell arrays (first axis concatenated over cells
    in batch order); each is sliced to the rank's cells."""
    lo, hi = partition(cell_work(cells, kind), world, rank)
    off = fine_offsets(cells)
    sl = [None if a is None else a[off[lo]:off[hi]] for a in fine_arrays]
    KH, FH = build(cells[lo:hi], sl)
    if dist is None or world == 1:
        return KH, FH
    return gather_blocks(KH, dist, group), gather_blocks(FH, dist, group)
