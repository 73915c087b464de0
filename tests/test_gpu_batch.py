"""rtr_recognize_batch: every pair's result equals the single-pair call's,
for the plain and the learned form; the autotuner picks a valid setting."""
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


def test_batch_equals_single_calls(ctx, rtr, batch):
    prm, mods, scenes = batch
    ctx.set_tuning("batch_workers", 3)
    got = _rows(rtr.recognize_batch(ctx, mods, scenes, prm))
    for i, (m, s) in enumerate(zip(mods, scenes)):
        ref = rtr.recognize(ctx, m, s, prm).cpu().numpy().tobytes()
        assert got[i] == ref, i
    ctx.set_tuning("batch_workers", 0)


def test_batch_learned_equals_single_calls(ctx, rtr, batch):
    prm, mods, scenes = batch
    mlp = rtr.Mlp(ctx, seed=5)
    got = _rows(rtr.recognize_batch(ctx, mods, scenes, prm, mlp=mlp, keep=0.5))
    for i, (m, s) in enumerate(zip(mods, scenes)):
        ref = rtr.recognize_learned(ctx, m, mlp, s, keep=0.5, params=prm).cpu().numpy().tobytes()
        assert got[i] == ref, i


def test_batch_autotune(ctx, rtr, batch):
    prm, mods, scenes = batch
    w, g = rtr.batch_autotune(ctx, mods[:4], scenes[:4], prm)
    assert w in (1, 2, 4, 8) and g in (4, 8)
    ctx.set_tuning("batch_workers", 0)
    ctx.set_tuning("icp_group", 0)


def test_batch_empty(ctx, rtr, batch):
    prm, _, _ = batch
    rtr.recognize_batch(ctx, [], [], prm)
