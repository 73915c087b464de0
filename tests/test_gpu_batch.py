"""rtr_recognize_batch: every pair's result equals the single-pair call's,
for the plain and the learned form; the autotuner picks a valid setting.

Batch workers each get a share of the GPU for the cooperative kernels, so an
ICP problem may be split over fewer blocks than in a single call; its FP32
block sums then round differently.  Counts must match exactly, poses within
1e-5 (the ICP tolerance against the FP64 oracle) and scores within 1e-3."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(ctx, rtr):
    import torch
    from realtime_robot_gb300 import learned as L
    prm = rtr.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    models, scenes = {}, []
    mods = []
    for seed in range(200, 210):
        shape, model, seg, _ = L.make_pair(seed, n_seg=None)
        if shape not in models:
            models[shape] = rtr.Model(ctx, torch.from_numpy(model).cuda(), prm)
        mods.append(models[shape])
        scenes.append(torch.from_numpy(seg).cuda())
    return prm, mods, scenes


def _rows(res):
    return [bytes(r) for r in res.cpu().numpy()]


def _same(rtr, a: bytes, b: bytes):
    ra, rb = rtr.parse_recog_result(a), rtr.parse_recog_result(b)
    for k in ("n_voxels", "n_keypoints", "n_correspondences", "n_clusters", "status"):
        assert ra[k] == rb[k], k
    assert len(ra["instances"]) == len(rb["instances"])
    for x, y in zip(ra["instances"], rb["instances"]):
        assert x["hypothesis"] == y["hypothesis"] and x["cluster_size"] == y["cluster_size"]
        np.testing.assert_allclose(x["pose"], y["pose"], atol=1e-5)
        assert abs(x["score"] - y["score"]) <= 1e-3


def test_batch_equals_single_calls(ctx, rtr, batch):
    prm, mods, scenes = batch
    ctx.set_tuning("batch_workers", 3)
    got = _rows(rtr.recognize_batch(ctx, mods, scenes, prm))
    for i, (m, s) in enumerate(zip(mods, scenes)):
        ref = rtr.recognize(ctx, m, s, prm).cpu().numpy().tobytes()
        _same(rtr, got[i], ref)
    ctx.set_tuning("batch_workers", 0)


def test_batch_learned_equals_single_calls(ctx, rtr, batch):
    prm, mods, scenes = batch
    mlp = rtr.Mlp(ctx, seed=5)
    got = _rows(rtr.recognize_batch(ctx, mods, scenes, prm, mlp=mlp, keep=0.5))
    for i, (m, s) in enumerate(zip(mods, scenes)):
        ref = rtr.recognize_learned(ctx, m, mlp, s, keep=0.5, params=prm).cpu().numpy().tobytes()
        _same(rtr, got[i], ref)


def test_batch_autotune(ctx, rtr, batch):
    prm, mods, scenes = batch
    ref = [bytes(r) for r in rtr.recognize_batch(ctx, mods[:4], scenes[:4], prm).cpu().numpy()]
    w, g = rtr.batch_autotune(ctx, mods[:4], scenes[:4], prm)
    t = rtr.batch_tuning(ctx)
    assert w in (1, 2, 4, 8) and g in (2, 4, 8)
    assert t["batch_workers"] == w and t["icp_group"] == g
    assert t["scene_grid_mm"] in (0, 20, 40, 60) and t["normals_grid_mm"] in (0, 20, 30, 80)
    # the tuned grids change speed, not results (ICP block sums aside)
    got = [bytes(r) for r in rtr.recognize_batch(ctx, mods[:4], scenes[:4], prm).cpu().numpy()]
    for a, b in zip(got, ref):
        _same(rtr, a, b)
    for k in ("batch_workers", "icp_group", "scene_grid_mm", "normals_grid_mm"):
        ctx.set_tuning(k, 0)


def test_batch_empty(ctx, rtr, batch):
    prm, _, _ = batch
    rtr.recognize_batch(ctx, [], [], prm)


def test_batch_graph_replays_the_batch(ctx, rtr, batch):
    import torch
    prm, mods, scenes = batch
    ctx.set_tuning("batch_workers", 4)
    ref = _rows(rtr.recognize_batch(ctx, mods, scenes, prm))
    g = rtr.BatchGraph(ctx, mods, scenes, prm)
    for _ in range(2):
        g.results.zero_()
        g.launch()
        torch.cuda.synchronize()
        got = _rows(g.results)
        for a, b in zip(got, ref):
            assert a == b  # same workers, same blocks: identical
    g.close()
    ctx.set_tuning("batch_workers", 0)


def test_batch_graph_refuses_to_run_after_scratch_moved(rtr, batch):
    # a fresh context: the plain graph is made on its scratch; growing the
    # arena afterwards (as a larger call would) reallocates it, so the graph's
    # launch must be refused on the host (no kernel runs)
    import torch
    prm, mods, scenes = batch
    c2 = rtr.Context(0)
    c2.set_tuning("batch_workers", 2)
    g = rtr.BatchGraph(c2, mods[:4], scenes[:4], prm)
    g.launch()
    torch.cuda.synchronize()
    c2.reserve(2 * c2.scratch_bytes() + (1 << 20))
    with pytest.raises(rtr.RtrError) as e:
        g.launch()
    assert e.value.status == 1 and "recreate" in str(e.value)
    g.close()
    # made again after the growth, it runs
    g = rtr.BatchGraph(c2, mods[:4], scenes[:4], prm)
    g.launch()
    torch.cuda.synchronize()
    g.close()
    c2.close()


def test_single_recognition_captured_in_a_graph(ctx, rtr, batch):
    import torch
    prm, mods, scenes = batch
    m, s = mods[0], scenes[0]
    ref = rtr.recognize(ctx, m, s, prm).cpu().numpy().tobytes()
    st = torch.cuda.Stream()
    res = torch.zeros(C.sizeof(rtr.RecogResult), dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(st):
        rtr.recognize(ctx, m, s, prm, result=res, stream=st.cuda_stream)  # sizes the scratch
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st, capture_error_mode="thread_local"):
        rtr.recognize(ctx, m, s, prm, result=res, stream=st.cuda_stream)
    res.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert res.cpu().numpy().tobytes() == ref


@pytest.mark.parametrize("workers", [1, 3])
def test_multi_model_one_scene_equals_single_calls(ctx, rtr, batch, workers):
    # rtr_recognize_multi: the scene's stages once, every model on it; one
    # worker runs the models in turn on the caller's stream (bit-identical),
    # several share the GPU (ICP block sums may round differently)
    prm, mods, scenes = batch
    uniq = list({id(m): m for m in mods}.values())
    scene = scenes[0]
    ctx.set_tuning("batch_workers", workers)
    got = _rows(rtr.recognize_multi(ctx, uniq, scene, prm))
    ctx.set_tuning("batch_workers", 0)
    for i, m in enumerate(uniq):
        ref = rtr.recognize(ctx, m, scene, prm).cpu().numpy().tobytes()
        if workers == 1:
            assert got[i] == ref
        else:
            _same(rtr, got[i], ref)


def test_multi_model_learned_equals_single_calls(ctx, rtr, batch):
    prm, mods, scenes = batch
    uniq = list({id(m): m for m in mods}.values())
    mlp = rtr.Mlp(ctx, seed=9)
    for scene in scenes[:3]:
        got = _rows(rtr.recognize_multi(ctx, uniq, scene, prm, mlp=mlp, keep=0.5))
        for i, m in enumerate(uniq):
            ref = rtr.recognize_learned(ctx, m, mlp, scene, keep=0.5, params=prm).cpu().numpy().tobytes()
            _same(rtr, got[i], ref)


def test_multi_model_edge_cases(ctx, rtr, batch):
    import torch
    prm, mods, _ = batch
    rtr.recognize_multi(ctx, [], torch.zeros((0, 4), device="cuda"), prm)
    res = rtr.recognize_multi(ctx, mods[:2], torch.zeros((0, 4), device="cuda"), prm)
    for r in _rows(res):
        d = rtr.parse_recog_result(r)
        assert d["n_voxels"] == 0 and d["instances"] == []
