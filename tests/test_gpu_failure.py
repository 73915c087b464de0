"""Failure detection in the forms that fault no GPU.

- Bounded device waits: with a wait budget too small for any wait to be met,
  the ICP grid barrier and the matcher's mbarrier pipeline return
  RTR_ERR_TIMEOUT through the context's status word (the matcher first waits
  for its own copies and MMAs already in flight, then frees its TMEM), and
  the same context gives exact results once the budget is restored.
- Bad inputs made on the host: points with NaN / inf coordinates are dropped
  by the voxel filter as PCL's VoxelGrid drops them (the oracle the same),
  so a scene with such points is recognised exactly as the scene without
  them; a scene of nothing but such points, and an empty scene, find nothing
  (status RTR_ERR_NOT_FOUND, no pose); ICP with such points in either cloud
  never matches them and returns a finite pose, the oracle's correspondences.
- An allocation failure injected through the context's scratch limit
  returns RTR_ERR_OOM and leaves the context usable.
"""
import numpy as np
import pytest

import oracle as O
from oracle import pipeline as OP

pytestmark = pytest.mark.gpu


def _dev(a, dt=np.float32):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()


def _pair(R, seed=1):
    model = R.synth_shape(R.CHAIR, 20000, 2024)
    T = R.synth_rigid(100 + seed, 30.0, 0.3)
    seg = R.synth_transform_noise(R.synth_crop(R.synth_shape(R.CHAIR, 20000, 500 + seed), 0.4, seed), T,
                                  0.002, 9 + seed)
    return model, seg, T


def _poison(pts, frac, seed):
    """pts with rows of NaN / +inf / -inf coordinates inserted at random places."""
    rng = np.random.default_rng(seed)
    k = max(3, int(frac * pts.shape[0]))
    bad = np.zeros((k, 4), np.float32)
    bad[:, :3] = rng.uniform(-1, 1, (k, 3))
    kinds = [np.nan, np.inf, -np.inf]
    for i in range(k):
        bad[i, i % 3] = kinds[i % 3]
    pos = np.sort(rng.integers(0, pts.shape[0] + 1, k))
    return np.insert(pts, pos, bad, axis=0)


def test_icp_wait_budget_runs_out_then_recovers(rtr):
    src, tgt, T = rtr.config0_pair(2024, 8000)
    c = rtr.Context(0)
    try:
        s, t = _dev(src), _dev(tgt)
        c.set_wait_budget_ms(1e-6)
        res, _, _ = c.icp(s, t, 30, 0.05)
        with pytest.raises(rtr.RtrError, match="RTR_ERR_TIMEOUT"):
            c.check()
        r = c.parse_icp_result(res)
        assert np.all(np.isfinite(r["pose"]))
        c.set_wait_budget_ms(2000.0)
        res, tp, tc = c.icp(s, t, 30, 0.05, trace=True)
        c.check()
        corr, _, _ = O.icp_replay(src, tgt, 0.05, tp.cpu().numpy())
        assert np.array_equal(corr, tc.cpu().numpy())
        r = c.parse_icp_result(res)
        assert r["status"] == 0 and r["iterations"] == 30
    finally:
        c.close()


def test_match_wait_budget_runs_out_then_recovers(rtr):
    rng = np.random.default_rng(3)
    q = rng.random((3000, 352), dtype=np.float32)
    db = rng.random((5000, 352), dtype=np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    db /= np.linalg.norm(db, axis=1, keepdims=True)
    c = rtr.Context(0)
    try:
        dq, ddb = _dev(q), _dev(db)
        c.set_wait_budget_ms(1e-6)
        c.match(dq, ddb)
        with pytest.raises(rtr.RtrError, match="RTR_ERR_TIMEOUT"):
            c.check()
        c.set_wait_budget_ms(2000.0)
        idx, d2 = c.match(dq, ddb)
        c.check()
        ri, rd = O.match(q, db)
        assert np.array_equal(idx.cpu().numpy(), ri) and np.array_equal(d2.cpu().numpy(), rd)
    finally:
        c.close()


def test_voxel_filter_drops_nonfinite_points_like_the_oracle(ctx, rtr):
    import torch
    model, seg, _ = _pair(rtr)
    bad = _poison(seg, 0.02, 5)
    v = ctx.voxel_downsample(_dev(bad), 0.01)
    rv = O.voxel_downsample(bad, 0.01)
    assert np.array_equal(v.cpu().numpy(), rv)
    assert np.array_equal(rv, O.voxel_downsample(seg, 0.01))  # the same voxels as without them
    k = ctx.uniform_sample(_dev(bad), 0.02)
    assert np.array_equal(k.cpu().numpy(), O.uniform_sample(bad, 0.02))
    allbad = np.full((500, 4), np.nan, np.float32)
    assert ctx.voxel_downsample(_dev(allbad), 0.01).shape[0] == 0
    assert O.voxel_downsample(allbad, 0.01).shape[0] == 0
    torch.cuda.synchronize()


def test_recognize_ignores_nonfinite_points_and_finds_nothing_in_empty_scenes(ctx, rtr):
    import torch
    model, seg, T = _pair(rtr)
    prm = rtr.recog_default_params(scene_outward=1)
    m = rtr.Model(ctx, _dev(model), prm)
    try:
        clean = rtr.recognize(ctx, m, _dev(seg), prm).cpu().numpy().tobytes()
        bad = _poison(seg, 0.02, 6)
        got = rtr.recognize(ctx, m, _dev(bad), prm).cpu().numpy().tobytes()
        assert got == clean
        r = rtr.parse_recog_result(got)
        assert r["instances"] and O.pose_error(r["instances"][0]["pose"], T)[0] < 0.01
        for scene in (np.zeros((0, 4), np.float32), np.full((800, 4), np.nan, np.float32)):
            r = rtr.parse_recog_result(rtr.recognize(ctx, m, _dev(scene), prm))
            assert r["instances"] == [] and r["status"] == 4 and r["n_voxels"] == 0
        # the batch entry: clean, poisoned, empty and all-NaN pairs side by side
        scenes = [_dev(seg), _dev(bad), torch.zeros((0, 4), dtype=torch.float32, device="cuda"),
                  _dev(np.full((800, 4), np.nan, np.float32))]
        out = rtr.recognize_batch(ctx, [m] * 4, scenes, prm).cpu().numpy()
        res = [rtr.parse_recog_result(bytes(o)) for o in out]
        for x in res[:2]:
            assert x["instances"] and O.pose_error(x["instances"][0]["pose"], T)[0] < 0.01
            assert x["n_voxels"] == rtr.parse_recog_result(clean)["n_voxels"]
        for x in res[2:]:
            assert x["instances"] == [] and x["status"] == 4
        ctx.check()
    finally:
        m.close()


def test_icp_never_matches_nonfinite_points(ctx, rtr):
    src, tgt, T = rtr.config0_pair(2024, 6000)
    bsrc, btgt = _poison(src, 0.01, 7), _poison(tgt, 0.01, 8)
    res, tp, tc = ctx.icp(_dev(bsrc), _dev(btgt), 50, 0.05, trace=True)
    ctx.check()
    r = ctx.parse_icp_result(res)
    assert r["status"] == 0 and np.all(np.isfinite(r["pose"]))
    corr, opose, _ = O.icp_replay(bsrc, btgt, 0.05, tp.cpu().numpy())
    gc = tc.cpu().numpy()
    assert np.array_equal(corr, gc)
    nonfinite_src = ~np.isfinite(bsrc[:, :3]).all(1)
    nonfinite_tgt = np.nonzero(~np.isfinite(btgt[:, :3]).all(1))[0]
    assert np.all(gc[:, nonfinite_src] == -1) and not np.isin(gc, nonfinite_tgt).any()
    dt, dr = O.pose_error(r["pose"], T)
    assert dt < 0.01 and dr < np.radians(1.0)
    # unbounded: an infinite source point is at infinite d^2 from everything
    # and still matches nothing
    res, tp, tc = ctx.icp(_dev(bsrc), _dev(btgt), 50, 0.0, trace=True)
    r = ctx.parse_icp_result(res)
    assert np.all(np.isfinite(r["pose"]))
    gc = tc.cpu().numpy()
    assert np.all(gc[:, nonfinite_src] == -1) and not np.isin(gc, nonfinite_tgt).any()
    corr, _, _ = O.icp_replay(bsrc, btgt, 0.0, tp.cpu().numpy())
    assert np.array_equal(corr, gc)


def test_scratch_limit_returns_oom_and_context_stays_usable(rtr):
    model, seg, T = _pair(rtr)
    c = rtr.Context(0)
    try:
        prm = rtr.recog_default_params(scene_outward=1)
        # a fresh context under a 1 MiB budget: its first scratch is refused
        c.set_tuning("scratch_limit_mb", 1)
        with pytest.raises(rtr.RtrError, match="RTR_ERR_OOM"):
            rtr.Model(c, _dev(model), prm)
        src, tgt, _ = rtr.config0_pair(2024, 20000)
        with pytest.raises(rtr.RtrError, match="RTR_ERR_OOM"):
            c.icp(_dev(src), _dev(tgt), 10, 0.05)
        c.set_tuning("scratch_limit_mb", 0)
        m = rtr.Model(c, _dev(model), prm)
        r = rtr.parse_recog_result(rtr.recognize(c, m, _dev(seg), prm))
        assert r["instances"] and O.pose_error(r["instances"][0]["pose"], T)[0] < 0.01
        c.check()
        m.close()
    finally:
        c.close()
