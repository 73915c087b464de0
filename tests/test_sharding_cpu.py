"""Batch sharding on CPU: the longest-processing-time split of pairs by point
count, and two gloo ranks that each recognise their share (the GPU step is
replaced by a deterministic host function of the pair) and gather every
pair's (pose, score, status) on rank 0, which must equal one process doing
the whole batch."""
import os
import socket
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from realtime_robot_gb300 import sharding as SH  # noqa: E402


class _Model:
    def __init__(self, n_voxels):
        self.n_voxels = n_voxels


def _batch(seed=0, n=64):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(2000), np.log(60000), n)).astype(int)
    models = [_Model(int(v)) for v in rng.integers(3000, 12000, n)]
    scenes = [np.zeros((int(s), 4), np.float32) for s in sizes]
    return models, scenes


def _fake_recognize(ctx, models, scenes, params, mlp, keep):
    """Stands in for rtr_recognize_batch: a result that depends only on the
    pair (so a pair gives the same result on whichever rank runs it)."""
    out = []
    for m, s in zip(models, scenes):
        k = s.shape[0] * 7 + m.n_voxels
        pose = np.eye(4)
        pose[:3, 3] = [k * 1e-6, -k * 2e-6, 0.5]
        found = k % 3 != 0
        out.append({"instances": [{"pose": pose, "score": (k % 1000) / 1000.0}] if found else [],
                    "status": 0 if found else 4})
    return out


def test_lpt_partition_balanced_and_complete():
    models, scenes = _batch(1)
    sizes = SH.pair_sizes(models, scenes)
    for ws in (1, 2, 3, 8):
        parts = SH.lpt_partition(sizes, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        # LPT: every rank within one pair of every other
        assert max(loads) - min(loads) <= max(sizes)
        assert parts == SH.lpt_partition(sizes, ws)  # deterministic
    # a rank can receive nothing when there are fewer pairs than ranks
    assert SH.lpt_partition([5, 3], 4)[2:] == [[], []]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as tdist
    from realtime_robot_gb300 import sharding as S
    tdist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        models, scenes = _batch(2)
        rows, mine = S.recognize_batch_sharded(None, models, scenes, None, recognize_fn=_fake_recognize)
        q.put((rank, mine, None if rows is None else rows.tolist()))
    finally:
        tdist.destroy_process_group()


def test_two_gloo_ranks_gather_equals_single_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(2):
        rank, mine, rows = q.get(timeout=120)
        got[rank] = (mine, rows)
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    models, scenes = _batch(2)
    single, mine_all = SH.recognize_batch_sharded(None, models, scenes, None, recognize_fn=_fake_recognize)
    assert mine_all == list(range(64))
    # the ranks' shares partition the batch; rank 1 gets no gather result
    assert sorted(got[0][0] + got[1][0]) == list(range(64)) and got[1][1] is None
    np.testing.assert_array_equal(np.array(got[0][1]), single)
    assert np.array_equal(single[:, 19], np.arange(64))
