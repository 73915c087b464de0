"""bench.py's N > 1 host logic on CPU: two gloo ranks, each timing its own
replica; the whole-job value is every rank's units over the slowest rank's
time, and the reference arm runs on rank 0 only."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as tdist
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        slow = bench.max_over_ranks(1.0 + rank, True)
        value = bench.replica_throughput(10, 1.0 + rank, ws, True)
        q.put((rank, slow, value))
    finally:
        tdist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slow, value in got:
        assert slow == 2.0
        assert value == pytest.approx(10 * 2 / 2.0)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus = 2, 3, 2

    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_line_keeps_the_contract_and_loads_no_gpu_library():
    """Rank 0 of the reference arm prints one JSON line with the contract's
    keys, times whole oracle recognitions of the room, and maps only the
    oracle's libraries (none of the GPU path's)."""
    import json
    import subprocess
    code = (
        "import sys, json; sys.path.insert(0, %r); import bench\n"
        "class A: steps, warmup, gpus = 1, 0, 1\n"
        "bench.run_reference(A())\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'so': sorted({l.split()[-1] for l in maps.splitlines() if l.endswith('.so')})}))\n"
    ) % str(ROOT)
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env,
                       cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    line, so = lines[0], lines[1]["so"]
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "recognitions/s"
    assert line["cpu_baseline"]["kind"] == "port" and "full" in line["cpu_baseline"]["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["counts"]["n_voxels"] > 200000 and line["counts"]["n_keypoints"] > 100000
    mine = [s for s in so if str(ROOT) in s]
    assert mine and all("/oracle/" in s for s in mine), mine
