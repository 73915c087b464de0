"""Batch sharding across processes (one GPU per process).

A batch of model x segment pairs (the batched registration workload) has no
data dependence between pairs, so it is split by pairs with no collective on
the data path: each rank recognises its own slice with rtr_recognize_batch
and rank 0 gathers every pair's (pose, score, status) on the host.

The split is longest-processing-time first by point count (segment points
plus model voxels, the terms every stage's cost grows with): pairs in
descending size, each to the rank with the least assigned so far (ties to
the lower rank, then the lower pair index), so every rank's share is within
one pair of the mean.  The gather moves 16 doubles, one float and two ints
per pair over a host process group (gloo), whatever backend the job's GPU
work uses.
"""
from __future__ import annotations

import heapq

import numpy as np

# per pair: pose (16 doubles), score, instances, status, pair index
_ROW = 16 + 4


def lpt_partition(sizes, world_size: int) -> list[list[int]]:
    """Pair indices per rank, each rank's list ascending."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    sizes = [int(s) for s in sizes]
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    heap = [(0, r) for r in range(world_size)]
    heapq.heapify(heap)
    parts: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + sizes[i], r))
    return [sorted(p) for p in parts]


def pair_sizes(models, scenes) -> list[int]:
    """Cost proxy per pair: segment points + model voxels."""
    return [int(s.shape[0]) + int(m.n_voxels) for m, s in zip(models, scenes)]


def pack_results(parsed: list[dict], indices: list[int]) -> np.ndarray:
    """[k, 20] float64 rows: best instance pose (identity when none), its
    score, the instance count, the status and the pair index."""
    out = np.zeros((len(parsed), _ROW), np.float64)
    for r, (res, i) in enumerate(zip(parsed, indices)):
        inst = res["instances"]
        out[r, :16] = (inst[0]["pose"] if inst else np.eye(4)).reshape(16)
        out[r, 16] = inst[0]["score"] if inst else 0.0
        out[r, 17] = len(inst)
        out[r, 18] = res["status"]
        out[r, 19] = i
    return out


def gather_rows(rows: np.ndarray, n_pairs: int, group=None, dst: int = 0):
    """Every rank's packed rows to rank `dst`, in pair order: [n_pairs, 20]
    on dst, None elsewhere.  A single process returns its own rows sorted."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        full = np.zeros((n_pairs, _ROW), np.float64)
        full[rows[:, 19].astype(np.int64)] = rows
        return full
    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    # fixed-size exchange: pad every rank's rows to the largest count
    n_local = torch.tensor([rows.shape[0]], dtype=torch.int64)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(ws)]
    dist.all_gather(counts, n_local, group=group)
    cap = int(max(c.item() for c in counts))
    buf = torch.full((cap, _ROW), -1.0, dtype=torch.float64)
    buf[: rows.shape[0]] = torch.from_numpy(rows)
    got = [torch.zeros((cap, _ROW), dtype=torch.float64) for _ in range(ws)] if rank == dst else None
    dist.gather(buf, got, dst=dst, group=group)
    if rank != dst:
        return None
    full = np.zeros((n_pairs, _ROW), np.float64)
    for r, t in enumerate(got):
        a = t.numpy()[: int(counts[r].item())]
        full[a[:, 19].astype(np.int64)] = a
    return full


def recognize_batch_sharded(ctx, models, scenes, params, mlp=None, keep: float = 1.0, group=None,
                            recognize_fn=None):
    """This rank's share of the batch through rtr_recognize_batch, gathered on
    rank 0: returns ([n_pairs, 20] rows on rank 0 / None elsewhere, this
    rank's pair indices).  recognize_fn(ctx, models, scenes, params, mlp, keep)
    -> list of parsed results stands in for the GPU call in host-only tests."""
    import torch.distributed as dist
    dist_on = dist.is_available() and dist.is_initialized()
    ws = dist.get_world_size(group) if dist_on else 1
    rank = dist.get_rank(group) if dist_on else 0
    mine = lpt_partition(pair_sizes(models, scenes), ws)[rank]
    sub_m = [models[i] for i in mine]
    sub_s = [scenes[i] for i in mine]
    if recognize_fn is None:
        from . import parse_recog_result, recognize_batch
        parsed = []
        if mine:
            res = recognize_batch(ctx, sub_m, sub_s, params, mlp=mlp, keep=keep).cpu().numpy()
            parsed = [parse_recog_result(bytes(r)) for r in res[: len(mine)]]
    else:
        parsed = recognize_fn(ctx, sub_m, sub_s, params, mlp, keep)
    rows = pack_results(parsed, mine) if mine else np.zeros((0, _ROW), np.float64)
    return gather_rows(rows, len(scenes), group=group), mine
