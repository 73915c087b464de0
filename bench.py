"""Benchmark of the GB300 registration hot path (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline workload (config 1): single-scene recognition of the 20,000-point
box chair in a 300,000-point ray-cast room (5 x 5 x 3 m, floor + 2 walls,
3 chairs + 1 desk at seeded poses, camera at (0, -2.5, 1.5), 3 mm noise):
1 cm voxel filter, k=10 normals, 2 cm uniform keypoints, SHOT-352 at 4 cm,
1-NN matching, geometric-consistency grouping (1 cm, 5), hypothesis
verification and 30-iteration ICP refinement (2 cm).  The model is prepared
once (outside the timed region); one step = one rtr_recognize of the scene.
Metric: scene recognitions per second.  The same line carries config 0
(20k <-> 20k chair ICP, 5 cm, 50 iterations) as ICP iterations per second.

The path does not shard (one scene is one unit): with N GPUs every rank runs
its own replica and `value` sums the units of all ranks over the slowest
rank's time.  `--impl reference` times the CPU restatement of the path
(oracle/, all host threads): whole recognitions of the same room, with its
inputs made by oracle/libsynth.so (no library of the GPU path is loaded).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_PTS = 20000
ITERS = 50
MAX_DIST = 0.05
SEED = 2024
ROOM_SEED = 1
CAM = (0.0, -2.5, 1.5)
FLUSH_BYTES = 256 << 20  # > 129 MB L2
METRIC = "scene recognitions/s (config 1: 300k-pt room, 20k-pt chair model, plain form)"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return (float(d["hbm_gbs"]), float(d["bf16_tflops"]),
                "measured (MEASURED_PEAKS.json: hbm_gbs copy, bf16_tflops burst)")
    return 6800.0, 1900.0, "fallback (6.8 TB/s, 1.9 PFLOP/s)"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def _profiled_traffic(scope: str):
    """DRAM bytes (read + write) per launch of the kernel behind `scope`, from
    the committed ncu summary of the bench workload, or None."""
    f = ROOT / "profiles" / f"{scope}_room300k.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, dist: bool, device="cpu") -> float:
    """The slowest rank's value (all-reduce MAX), or x on one process."""
    if not dist:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, seconds_local: float, ws: int, dist: bool, device="cpu") -> float:
    """Whole-job throughput of ws independent replicas: every rank's units
    over the slowest rank's time (weak scaling, no data-path collective)."""
    return units_per_rank * ws / max_over_ranks(seconds_local, dist, device)


def _room(gen=None):
    """The config-1 room, the chair model and the three chairs' true poses,
    from `gen` (the package's generator, or oracle.synth: the same source
    built host-only, for the reference arm)."""
    if gen is None:
        import realtime_robot_gb300 as gen
    scene, shapes, poses = gen.synth_room(ROOM_SEED)
    model = gen.synth_shape(gen.CHAIR, N_PTS, SEED)
    chairs = [poses[i] for i in range(len(shapes)) if shapes[i] == 0]
    return scene, model, chairs


def _icp_pair(gen=None):
    if gen is None:
        import realtime_robot_gb300 as gen
    return gen.config0_pair(SEED, N_PTS)


def _grid_cells(tgt: np.ndarray, h: float) -> int:
    ext = tgt[:, :3].max(0).astype(np.float64) - tgt[:, :3].min(0)
    return int(np.prod(np.floor(ext / h) + 1))


def _nearest_errors(instances, chairs):
    import oracle as O
    out = []
    for inst in instances:
        e = min((O.pose_error(inst["pose"], g) for g in chairs), key=lambda x: x[0])
        out.append([round(e[0], 4), round(float(np.degrees(e[1])), 3), round(float(inst["score"]), 3)])
    return out


def _chairs_found(instances, chairs) -> int:
    """Chairs with an instance within 1 cm / 1 degree of the generator's pose."""
    import oracle as O
    found = 0
    for g in chairs:
        found += any(O.pose_error(inst["pose"], g)[0] <= 0.01 and O.pose_error(inst["pose"], g)[1] <= np.radians(1.0)
                     for inst in instances)
    return found


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (C restatement, OpenMP, all host threads)
# ---------------------------------------------------------------------------
def cpu_recognition(scene, model, steps: int = 1, warmup: int = 0) -> dict:
    """The whole oracle pipeline on the whole config-1 scene, per step: voxel
    filter, normals, keypoints, SHOT, exact 1-NN of every scene keypoint,
    grouping of every correspondence (256-cluster cap, as on the GPU),
    hypothesis scores, 16 ICP refinements, final scores.  The model is
    prepared once beforehand, as on the GPU."""
    import oracle as O
    from oracle import pipeline as OP
    p = OP.params(viewpoint=CAM)
    m = OP.prepare_model(model, p)
    for _ in range(warmup):
        OP.recognize(m, scene, p)
    times, stage = [], {}
    r = None
    for _ in range(steps):
        t0 = time.perf_counter()
        r = OP.recognize(m, scene, p, timing=stage)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    return {"value": len(times) / total, "unit": "recognitions/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"full: {len(times)} whole recognitions of the config-1 scene by the C oracle (every scene "
                      "keypoint matched, every correspondence grouped), model prepared beforehand",
            "stage_s": {k: round(v / len(times), 3) for k, v in stage.items()},
            "counts": {k: r[k] for k in ("n_voxels", "n_keypoints", "n_correspondences", "n_clusters")},
            "instances": len(r["instances"])}


def cpu_icp_sample(src, tgt, budget_s: float = 10.0) -> dict:
    import oracle as O
    t0 = time.perf_counter()
    runs = 0
    while True:
        O.icp(src, tgt, ITERS, MAX_DIST)
        runs += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": runs * ITERS / dt, "unit": "iters/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{runs} full config-0 registrations of the C oracle (exact grid 1-NN + FP64 fit)"}


def run_reference(args):
    """The reference arm: the CPU restatement of the path (oracle/, all host
    threads) timed on the same workload, W untimed and K timed steps, each a
    whole recognition of the config-1 room.  Its inputs come from
    oracle/libsynth.so, so no library of the GPU path is loaded."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from oracle import synth as S
    scene, model, chairs = _room(S)
    c = cpu_recognition(scene, model, steps=args.steps, warmup=args.warmup)
    v = c["value"]
    src, tgt, _ = _icp_pair(S)
    icp = cpu_icp_sample(src, tgt, 5.0)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "recognitions/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": "config1_room300k_chair20k", "room_seed": ROOM_SEED,
                                            "model_points": N_PTS, "scene_points": int(scene.shape[0])},
            "cpu_baseline": {k: c[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "stage_s": c["stage_s"], "counts": c["counts"],
            "e2e": {"value": v, "unit": "recognitions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "icp": {"metric": "ICP iters/s (config 0)", "value": icp["value"], "unit": "iters/s",
                    "sample": icp["sample"]}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    import realtime_robot_gb300 as R

    ws, rank, local = _dist()
    dist = ws > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = R.Context(local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    hbm_peak, bf16_peak, peak_src = _peaks()

    # ------------------------------ config 1 ------------------------------
    scene, model, chairs = _room()
    prm = R.recog_default_params(viewpoint=CAM)
    m = R.Model(ctx, torch.from_numpy(model).to(dev), prm)
    s_d = torch.from_numpy(scene).to(dev)
    res = torch.zeros(R.C.sizeof(R.RecogResult), dtype=torch.uint8, device=dev)

    def step():
        R.recognize(ctx, m, s_d, prm, result=res, stream=stream.cuda_stream)

    def timed_steps(n):
        """n steps, L2 flushed before each, CUDA events around each on the
        launching stream; returns the per-step ms."""
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for i in range(n):
            flush.zero_()
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    # Warm-up: the first call sizes the scratch arena, the second identical
    # call captures the recognition's launches into a CUDA graph (the
    # context's "auto_graph"), the timed calls replay it.
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    ctx.check()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    l0 = R.launch_count()
    step_ms = timed_steps(args.steps)
    launches = R.launch_count() - l0
    if dist:
        tdist.barrier()
    clocks = sampler.stop()
    ctx.check()
    total_ms = max_over_ranks(sum(step_ms), dist, dev)
    value = replica_throughput(args.steps, total_ms / 1e3, ws, False)
    r = R.parse_recog_result(res)
    # the same steps with every kernel launched by the host (no graph replay)
    ctx.set_tuning("auto_graph", 0)
    step()
    direct_ms = sum(timed_steps(args.steps)) / args.steps
    # stage times: the same steps once more, profiled (profiling runs them
    # direct, each stage bracketed by events)
    ctx.set_profiling(True)
    ctx.profile(clear=True)
    timed_steps(args.steps)
    prof = ctx.profile(clear=True)
    ctx.set_profiling(False)
    ctx.set_tuning("auto_graph", 1)
    ctx.check()
    stage_ms = {}
    for nm, ms in prof:
        stage_ms[nm] = stage_ms.get(nm, 0.0) + ms / args.steps

    # roofline of the dominant kernel (kernel-level profiling scopes; the
    # algorithmic work of each is stated beside it)
    Ks, Km, C = r["n_keypoints"], m.n_keypoints, r["n_correspondences"]
    gcs = ctx.gc_stats()
    M_ref = min(r["n_clusters"], prm.refine_top)
    kern = {
        # one FP32-equivalent GEMM: 2 * scene keypoints * model keypoints * 352
        "match_gemm": ("tensor", 2.0 * Ks * Km * 352, "k_match_tc (tcgen05 BF16 hi/lo split, FP32 accumulate, top-8)",
                       "three BF16 MMAs per K step; two 96 KB TMA stages per CTA"),
        # the unique bytes the walk must move: both endpoints (32 B) of every
        # correspondence; everything else (C x sets consistency checks over
        # those endpoints, the pass masks, the sets) lives in L2
        "gc_walk": ("hbm", 32.0 * C, "k_gc_coop (cooperative grouping walk)",
                    f"barrier- and latency-bound: {gcs['sets']} consensus sets over {C} correspondences in "
                    f"{gcs['rounds']} rounds of four grid-wide phases (seed tests pruned to the chunks within "
                    f"each seed's reach; stale sets recomputed in place); the 32 B x C endpoints stay in L2"),
        # per hypothesis and iteration: each model voxel (16 B) and its matched scene point (16 B)
        "icp_refine": ("hbm", 32.0 * M_ref * prm.icp_iterations * m.n_voxels, "k_icp (multi-problem refinement)",
                       "latency- and barrier-bound: per iteration a 27-cell 1-NN per source point (own cell, "
                       "then only the neighbours within reach; grid and voxels stay in L2), a per-hypothesis "
                       "barrier and the FP64 pose solve"),
    }
    kern = {k: v for k, v in kern.items() if k in stage_ms}
    top = max(kern, key=lambda k: stage_ms[k])
    bound, work, kname, knote = kern[top]
    kms = stage_ms[top]
    if bound == "tensor":
        ach = work / (kms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": bf16_peak, "unit": "TFLOP/s", "frac": ach / bf16_peak,
                "traffic": _profiled_traffic(top), "kernel": kname, "kernel_ms": kms,
                "algorithmic_flops_per_launch": work, "peak_source": peak_src, "note": knote}
    else:
        ach = work / (kms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                "traffic": _profiled_traffic(top), "kernel": kname, "kernel_ms": kms,
                "algorithmic_bytes_per_launch": work, "peak_source": peak_src, "note": knote}
    roof["kernel_ms_by_scope"] = {k: round(stage_ms[k], 3) for k in kern}

    # end to end through the C ABI's host entry: rtr_recognize_host copies the
    # pinned host scene in, recognises, copies the result out and checks the
    # status word (synchronising), once per step
    h_scene = torch.from_numpy(scene).pin_memory()
    h_rr = R.RecogResult()
    n_scene = int(scene.shape[0])

    def host_step():
        R.check(R.lib().rtr_recognize_host(ctx.h, m.h, h_scene.data_ptr(), n_scene, R.C.byref(prm), R.C.byref(h_rr)))

    for _ in range(3):  # arena sizing, then the graph's capture
        host_step()
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e_s = max_over_ranks(time.perf_counter() - e0, dist, dev)
    e2e = {"value": replica_throughput(args.steps, e_s, ws, False), "unit": "recognitions/s",
           "h2d_bytes_per_step": int(scene.nbytes), "d2h_bytes_per_step": int(R.C.sizeof(R.RecogResult)),
           "path": "rtr_recognize_host (C ABI): pinned host scene in, rtr_recog_result out, wall clock; "
                   "the call replays its CUDA graph after the second identical call"}

    # ------------------------------ config 0 ------------------------------
    src, tgt, T = _icp_pair()
    s0 = torch.from_numpy(src).to(dev)
    t0 = torch.from_numpy(tgt).to(dev)
    ires = torch.zeros(256, dtype=torch.uint8, device=dev)

    def icp_step():
        ctx.icp(s0, t0, ITERS, MAX_DIST, result=ires, stream=stream.cuda_stream)

    for _ in range(3):
        icp_step()
    torch.cuda.synchronize()
    ctx.set_profiling(True)
    ctx.profile(clear=True)
    iev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        iev[i][0].record(stream)
        icp_step()
        iev[i][1].record(stream)
    torch.cuda.synchronize()
    iprof = ctx.profile(clear=True)
    ctx.set_profiling(False)
    icp_ms = sum(a.elapsed_time(b) for a, b in iev)
    kms = [ms for nm, ms in iprof if nm == "icp_kernel"]
    kavg = sum(kms) / max(1, len(kms))
    cells = _grid_cells(tgt, 0.5 * MAX_DIST)
    icp_bytes = ITERS * (16 * N_PTS + 16 * N_PTS + 8 * cells)
    icp_ach = icp_bytes / (kavg * 1e-3) / 1e9
    import oracle as O
    ir = ctx.parse_icp_result(ires)
    icp = {"metric": "ICP iters/s (config 0: 20k<->20k chair, 5 cm, 50 it)",
           "value": ITERS * args.steps * ws / (icp_ms / 1e3), "unit": "iters/s",
           "ms_per_registration": icp_ms / args.steps,
           "roofline": {"bound": "hbm", "achieved": icp_ach, "peak": hbm_peak,
                        "unit": "GB/s", "frac": icp_ach / hbm_peak, "traffic": None,
                        "kernel": "k_icp (persistent)", "kernel_ms": kavg,
                        "algorithmic_bytes_per_launch": icp_bytes},
           "pose_error_vs_truth": list(O.pose_error(ir["pose"], T))}

    batch = streaming = learned_room = ref_route = None
    if not args.no_extra:
        mlp, batch = batch_block(ctx, R, args.steps)
        learned_room = learned_room_block(ctx, R, m, s_d, prm, mlp, args.steps, stream, flush, r)
        streaming = stream_block(ctx, R, mlp)
        ref_route = ref_route_block(ctx, R, args.steps, rank == 0 and ws == 1 and not args.no_cpu_baseline)

    line = {
        "metric": METRIC, "value": value, "unit": "recognitions/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "config1_room300k_chair20k", "room_seed": ROOM_SEED, "model_points": N_PTS,
                   "scene_points": int(scene.shape[0]), "parallelism": f"replicas{ws}",
                   "l2": "flushed between steps (256 MiB write)",
                   "launch": "rtr_recognize replaying the context's CUDA graph of its launches (auto_graph)"},
        "direct_launch": {"value": replica_throughput(args.steps, direct_ms * args.steps / 1e3, ws, False),
                          "unit": "recognitions/s", "ms_per_step": direct_ms,
                          "note": "the same recognition with each kernel launched by the host (auto_graph 0)"},
        "roofline": roof,
        "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()},
        "counts": {k: r[k] for k in ("n_voxels", "n_keypoints", "n_correspondences", "n_clusters")},
        "model_keypoints": Km,
        "instances_err_to_nearest_chair_m_deg_score": _nearest_errors(r["instances"], chairs),
        "chairs_within_1cm_1deg": f"{_chairs_found(r['instances'], chairs)} of {len(chairs)}",
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "icp": icp,
        "batch": batch,
        "learned_room": learned_room,
        "streaming": streaming,
        "reference_route": ref_route,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_recognition(scene, model, steps=1, warmup=0)
        line["icp"]["cpu_baseline"] = cpu_icp_sample(src, tgt, 5.0)
    if rank == 0:
        print(json.dumps(line), flush=True)
    m.close()
    ctx.close()
    if dist:
        tdist.destroy_process_group()
    return 0


def batch_block(ctx, R, steps: int):
    """Config 2: 64 model x segment pairs (chairs, desks, sofas; 2k-60k points,
    <= 30 deg, +-0.3 m, 2 mm noise, 0-40 % crop) through rtr_recognize_batch
    and as a replayed CUDA graph (rtr_batch_graph_*), plain and learned (MLP
    trained here on the GPU, top 25 % of keypoints), against the same pairs
    one rtr_recognize call at a time."""
    import torch
    from realtime_robot_gb300 import learned as L
    prm = R.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    mods, scenes, npts, nmodel = [], [], 0, 0
    for seed in range(3000, 3064):
        # source and target sizes both log-uniform in [2k, 60k]
        shape, model, seg, _ = L.make_pair(seed, n_model=None)
        mods.append(R.Model(ctx, torch.from_numpy(model).cuda(), prm))
        scenes.append(torch.from_numpy(seg).cuda())
        npts += seg.shape[0]
        nmodel += model.shape[0]
    models = {i: m for i, m in enumerate(mods)}
    t0 = time.perf_counter()
    # labels at the plain pipeline's final pose; credible keypoints repeated
    # to a tenth of the rows
    X, y = L.build_dataset(ctx, range(4000, 4160), prm, label_pose="plain")
    Xb, yb = L.balance(X, y, 0.1)
    mlp, losses = L.train(ctx, Xb, yb, epochs=20, batch=4096, lr=1e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0

    def seq():
        for m, s in zip(mods, scenes):
            R.recognize(ctx, m, s, prm)
        torch.cuda.synchronize()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps

    reps = max(1, min(steps, 5))
    t_seq = timed(seq, reps)
    workers, group = R.batch_autotune(ctx, mods[:16], scenes[:16], prm)
    tuned = R.batch_tuning(ctx)
    t_plain = timed(lambda: R.recognize_batch(ctx, mods, scenes, prm), reps)
    t_learned = timed(lambda: R.recognize_batch(ctx, mods, scenes, prm, mlp=mlp, keep=0.25), reps)
    # the same batches captured once into CUDA graphs and replayed
    gp = R.BatchGraph(ctx, mods, scenes, prm)
    gl = R.BatchGraph(ctx, mods, scenes, prm, mlp=mlp, keep=0.25)
    t_gplain = timed(lambda: gp.launch(), reps)
    t_glearned = timed(lambda: gl.launch(), reps)
    gp.close()
    gl.close()
    for k in ("batch_workers", "icp_group", "scene_grid_mm", "normals_grid_mm"):
        ctx.set_tuning(k, 0)
    res_p = [R.parse_recog_result(bytes(r)) for r in R.recognize_batch(ctx, mods, scenes, prm).cpu().numpy()]

    def agreement(net, keep):
        """(pairs agreeing with plain, of them pairs where plain found one)"""
        res = [R.parse_recog_result(bytes(r)) for r in
               R.recognize_batch(ctx, mods, scenes, prm, mlp=net, keep=keep).cpu().numpy()]
        agree = found = 0
        for a, b in zip(res_p, res):
            if a["instances"] and b["instances"]:
                dt, dr = L.pose_diff(a["instances"][0]["pose"], b["instances"][0]["pose"])
                found += int(dt <= 0.01 and dr <= 1.0)
                agree += int(dt <= 0.01 and dr <= 1.0)
            else:
                agree += int(not a["instances"] and not b["instances"])
        return agree, found

    agree, found_agree = agreement(mlp, 0.25)
    untrained = R.Mlp(ctx, seed=99)
    gain = {"plain_found": sum(1 for a in res_p if a["instances"]),
            "trained_keep0.25": found_agree, "random_keep0.25": agreement(untrained, 0.25)[1],
            "trained_keep0.5": agreement(mlp, 0.5)[1], "random_keep0.5": agreement(untrained, 0.5)[1]}
    untrained.close()
    for m in models.values():
        m.close()
    n = len(scenes)
    return mlp, {"metric": "pairs/s (config 2: 64 model x segment pairs, 2k-60k points)", "unit": "pairs/s",
            "pairs": n, "points": npts,
            "sequential_plain": n / t_seq, "batched_plain": n / t_plain, "batched_learned": n / t_learned,
            "graph_plain": n / t_gplain, "graph_learned": n / t_glearned,
            # a pair whose learned pose disagrees with the plain one is re-run plain
            "graph_learned_with_fallback": n / (t_glearned + (n - agree) / n * t_gplain),
            "learned_graph_over_plain_sequential": t_seq / t_glearned,
            "autotuned": tuned,
            "graph_learned_with_fallback_over_sequential_plain": (n / (t_glearned + (n - agree) / n * t_gplain)) /
                                                                  (n / t_seq),
            "target_learned_over_plain": 5.0,
            "sizes": "source and target log-uniform in [2k, 60k]", "model_points": nmodel,
            "learned": {"keep": 0.25, "labels": "plain pipeline's final pose, 1 cm inliers",
                        "train_rows": int(X.shape[0]), "positives": int(y.sum().item()),
                        "positive_rate": float(y.mean()), "train_rows_balanced": int(Xb.shape[0]),
                        "train_s_incl_harvest": train_s, "final_loss": float(losses[-1]),
                        "pairs_agreeing_with_plain_1cm_1deg": agree, "fallbacks": n - agree,
                        "found_pairs_agreeing_trained_vs_random": gain}}


def learned_room_block(ctx, R, m, s_d, prm, mlp, steps, stream, flush, plain) -> dict:
    """The headline room recognised in the learned form (the MLP trained in
    the batch block keeps the 25 % most credible scene keypoints), timed like
    `value`, and compared with the plain result."""
    import torch
    res = torch.zeros(R.C.sizeof(R.RecogResult), dtype=torch.uint8, device=s_d.device)

    def step():
        R.recognize_learned(ctx, m, mlp, s_d, keep=0.25, params=prm, result=res, stream=stream.cuda_stream)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    # stage times of the same recognition, profiled (each stage bracketed by
    # events, kernels launched by the host)
    ctx.set_profiling(True)
    ctx.profile(clear=True)
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    stage_ms = {}
    for nm, t in ctx.profile(clear=True):
        stage_ms[nm] = stage_ms.get(nm, 0.0) + t / 3
    ctx.set_profiling(False)
    gcs = ctx.gc_stats()
    rl = R.parse_recog_result(res)
    same = len(rl["instances"]) == len(plain["instances"]) and all(
        np.abs(a["pose"][:3, 3] - b["pose"][:3, 3]).max() <= 0.01 for a, b in zip(rl["instances"], plain["instances"]))
    return {"metric": "scene recognitions/s, learned form (keep 0.25), config 1", "value": 1e3 / ms,
            "unit": "recognitions/s", "ms_per_step": ms, "n_keypoints_matched": rl["n_keypoints"],
            "n_correspondences": rl["n_correspondences"], "n_clusters": rl["n_clusters"],
            "instances": len(rl["instances"]), "agrees_with_plain_1cm": bool(same),
            "stage_ms": {k: round(v, 3) for k, v in stage_ms.items()},
            "grouping_walk": {"seeds_walked": gcs["walk_end"], "rounds": gcs["rounds"]}}


def ref_route_block(ctx, R, steps: int, cpu: bool) -> dict:
    """The reference's own descriptor route (occupancy grids, TDF fields,
    36-yaw get_Distance over every model x scan keypoint pair, the gated
    all-pairs loop, Ransac) on main's own inputs: chair1.pcd (1,818 points)
    and T0_m8111.pcd (3,218 points), keypoints by uniform sampling at 5 cm.
    Each step runs the whole route from the device clouds (every call
    synchronises); get_Distance is also timed alone with CUDA events."""
    import torch
    d = np.load(Path(__file__).resolve().parent / "tests" / "golden" / "main_clouds.npz")
    model, scan = d["chair1"], d["T0_m8111"]
    dm, ds = torch.from_numpy(model).cuda(), torch.from_numpy(scan).cuda()
    dkm = dm[ctx.uniform_sample(dm, 0.05).long()].contiguous()
    dks = ds[ctx.uniform_sample(ds, 0.05).long()].contiguous()
    nm, ns = dkm.shape[0], dks.shape[0]

    def route():
        mn, mo, mi = ctx.ref_occupancy(dm, dkm)
        sn, _, _ = ctx.ref_occupancy(ds, dks)
        tdf = ctx.ref_tdf(dm, dkm, mo, mi)
        sc, T = ctx.ref_distance(dm, dkm, mo, mi, tdf, dks)
        pi = ctx.ref_correspond(dkm, mn, dks, sn, sc)
        Tb, inl, best = ctx.ref_ransac(dkm, dks, pi, sc, T) if pi.shape[0] else (None, 0, -1)
        return (mn, mo, mi, tdf), pi, inl

    for _ in range(2):
        route()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        occ, pi, inl = route()
    route_ms = (time.perf_counter() - t0) * 1e3 / steps
    mn, mo, mi, tdf = occ
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist_ms = []
    for _ in range(steps):
        a.record()
        ctx.ref_distance(dm, dkm, mo, mi, tdf, dks)
        b.record()
        torch.cuda.synchronize()
        dist_ms.append(a.elapsed_time(b))
    dms = float(np.median(dist_ms))
    out = {"metric": "get_Distance pairs/s and route ms (main's clouds: chair1.pcd x T0_m8111.pcd, 5 cm keypoints)",
           "model_keypoints": nm, "scan_keypoints": ns, "pairs": nm * ns,
           "value": nm * ns / (dms * 1e-3), "unit": "pairs/s", "get_distance_ms": dms, "route_ms": route_ms,
           "kept_pairs": int(pi.shape[0]), "ransac_inliers": int(inl),
           "occupancy_points_max": int((mo[1:] - mo[:-1]).max().item())}
    if cpu:
        # the oracle (oracle/refmatch.c, all host threads) on the first model
        # keypoints' pairs, a bounded sample of the same workload
        import oracle as O
        km, ks = dkm.cpu().numpy(), dks.cpu().numpy()
        rmo, rmi = mo.cpu().numpy(), mi.cpu().numpy()
        rtdf = tdf.cpu().numpy()
        take = max(1, min(nm, 24))
        pm = np.repeat(np.arange(take, dtype=np.int32), ns)
        ps = np.tile(np.arange(ns, dtype=np.int32), take)
        t0 = time.perf_counter()
        O.ref_distance(model, km, rmo, rmi, rtdf, ks, pm, ps)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": pm.shape[0] / cs, "unit": "pairs/s", "cores": O.num_threads(),
                               "kind": "port", "sample": f"get_Distance of the first {take} model keypoints x all "
                               f"{ns} scan keypoints ({pm.shape[0]} pairs)"}
    out["cpp_kept_api"] = cpp_route_figure()
    return out


def cpp_route_figure():
    """main's route through the kept C++ API, one keypoint and one pair per
    call as main makes them (`realtime_robot_demo ref`: a 3,000-point chair
    and a moved resampling of it, 20 x 15 keypoints, 300 get_Distance calls),
    timed by the demo's own wall clock; the best of three runs."""
    import re
    import subprocess
    demo = Path(__file__).resolve().parent / "realtime_robot_gb300" / "realtime_robot_demo"
    if not demo.exists():
        return {"unavailable": "realtime_robot_demo not built"}
    best = None
    for _ in range(3):
        r = subprocess.run([str(demo), "ref", "1"], capture_output=True, text=True, timeout=300)
        m = re.search(r"timing keypoints (\d+) keypoint_s ([0-9.]+) pairs (\d+) pair_s ([0-9.]+)", r.stdout)
        if r.returncode != 0 or not m:
            return {"unavailable": f"demo exited {r.returncode}"}
        k, ks, p, ps = int(m.group(1)), float(m.group(2)), int(m.group(3)), float(m.group(4))
        if best is None or ps < best[3]:
            best = (k, ks, p, ps)
    k, ks, p, ps = best
    return {"metric": "get_Distance pairs/s through the kept C++ API (one pair per call)", "value": p / ps,
            "unit": "pairs/s", "pairs": p, "pair_loop_s": ps, "keypoints": k, "keypoint_members_s": ks,
            "per_pair_ms": 1e3 * ps / p, "per_keypoint_ms": 1e3 * ks / k}


def stream_block(ctx, R, mlp) -> dict:
    """Config 4: 300 organised 640x480 depth frames at 30 Hz (fx=fy=525) of the
    room with 6 chairs, 2 desks and 1 sofa along a smooth seeded path (0.5 m/s,
    <= 20 deg/s), depth noise 1.5 mm * z^2, ray-cast on the GPU before timing.
    Per frame: back-projection, frame-to-frame ICP odometry, batched learned
    recognition of the three model classes, fusion into a 5 mm voxel-hash
    map.  Latency is per frame, end to end on the host clock."""
    import torch
    from realtime_robot_gb300 import streaming as S
    p = R.room_default_params()
    p.n_chairs, p.n_desks, p.n_sofas = 6, 2, 1
    boxes, _, _ = R.synth_room_boxes(11, p)
    traj = R.synth_trajectory(11, 300, 30.0)
    frames = ctx.synth_depth_frames(boxes, traj, 640, 480, S.FX, S.FY, S.CX, S.CY, 0.0015, seed=11)
    torch.cuda.synchronize()
    prm = R.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    models = [R.Model(ctx, torch.from_numpy(R.synth_shape(sh, 20000, 1000 + sh)).cuda(), prm)
              for sh in (R.CHAIR, R.DESK, R.SOFA)]
    pipe = S.StreamPipeline(ctx, models, mlp=mlp, keep=0.25, params=prm)
    pipe.run(frames[:10], traj[0], traj[:10])  # warm-up (scratch growth)
    pipe.map.clear()
    out = pipe.run(frames, traj[0], traj)
    pipe.close()
    for m in models:
        m.close()
    out.update({"metric": "frames/s and per-frame latency (config 4: 300 depth frames 640x480)",
                "width": 640, "height": 480, "map_voxel_m": 0.005, "recognition": ("learned (keep 0.25)" if mlp is not None else "plain") + ", 3 classes",
                "odometry": "2 cm frame vs previous full-resolution frame, 30 iterations, 2 cm gate, constant-velocity start"})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batch and streaming blocks (profiling runs)")
    ap.add_argument("--only-ref-route", action="store_true",
                    help="run only the reference descriptor route block and print its JSON (profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.only_ref_route:
        import realtime_robot_gb300 as R
        ctx = R.Context(0)
        print(json.dumps(ref_route_block(ctx, R, args.steps, not args.no_cpu_baseline)), flush=True)
        ctx.close()
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
