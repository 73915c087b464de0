"""GPU parity of geometric-consistency grouping against the sequential oracle:
identical clusters (as sets, in the same order), sizes, and FP64 poses."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _dev(a, dt=np.float32):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()


def _check(ctx, mk, sk, cm, cs, cd, gc=0.01, th=5, maxc=64):
    mem, sizes, poses = ctx.gc_group(_dev(mk), _dev(sk), _dev(cm, np.int32), _dev(cs, np.int32), _dev(cd),
                                     gc, th, maxc, 128)
    mem, sizes, poses = mem.cpu().numpy(), sizes.cpu().numpy(), poses.cpu().numpy()
    clus, rposes, rsizes = O.gc_group(mk, sk, cm, cs, cd, gc, th, maxc)
    assert len(sizes) == len(rsizes), (len(sizes), len(rsizes))
    assert np.array_equal(sizes, rsizes)
    for c in range(len(sizes)):
        got = set(mem[c][: sizes[c]].tolist())
        ref = set(np.nonzero(clus == c)[0].tolist())
        assert got == ref, c
        dt, dr = O.pose_error(poses[c], rposes[c])
        assert dt < 1e-7 and dr < 1e-7, (c, dt, dr)
    return len(sizes)


def test_gc_planted_clusters(ctx):
    rng = np.random.default_rng(0)
    nm, ns = 400, 3000
    mk = np.zeros((nm, 4), np.float32)
    mk[:, :3] = rng.uniform(-0.3, 0.3, (nm, 3))
    sk = np.zeros((ns, 4), np.float32)
    sk[:, :3] = rng.uniform(-2, 2, (ns, 3))
    # plant two rigidly consistent clusters
    import realtime_robot_gb300 as R
    cm, cs = [], []
    for t in range(2):
        T = R.synth_rigid(t + 5, 90.0, 1.5)
        pick = rng.choice(nm, 20, replace=False)
        pts = O.transform_f32(T, mk[pick])
        idx = rng.choice(ns, 20, replace=False)
        sk[idx] = pts + np.float32(0.001) * rng.standard_normal((20, 4)).astype(np.float32) * [1, 1, 1, 0]
        cm += list(pick)
        cs += list(idx)
    n_rand = 1500
    cm += list(rng.integers(0, nm, n_rand))
    cs += list(rng.integers(0, ns, n_rand))
    cm, cs = np.array(cm, np.int32), np.array(cs, np.int32)
    cd = rng.uniform(0, 0.3, len(cm)).astype(np.float32)
    cd[:40] *= 0.1
    assert _check(ctx, mk, sk, cm, cs, cd) >= 2


def test_gc_real_correspondences(ctx, rtr):
    model = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    T = rtr.synth_rigid(5, 30.0, 0.3)
    seg = rtr.synth_transform_noise(rtr.synth_shape(rtr.CHAIR, 20000, 77), T, 0.002, 9)
    mv = O.voxel_downsample(model, 0.01)
    mn = O.orient_outward(mv, O.normals(mv, 10, (0, 0, 0)))
    sv = O.voxel_downsample(seg, 0.01)
    sn = O.orient_outward(sv, O.normals(sv, 10, (0, 0, 0)))
    mk = O.uniform_sample(mv, 0.01)
    sk = O.uniform_sample(sv, 0.02)
    md, _ = O.shot352(mv, mn, mk, 0.04)
    sd, _ = O.shot352(sv, sn, sk, 0.04)
    idx, d2 = O.match(sd, md)
    m = d2 < 0.25
    cs = np.nonzero(m)[0].astype(np.int32)
    n = _check(ctx, mv[mk], sv[sk], idx[m], cs, d2[m], 0.01, 5, 128)
    assert n > 10


def test_gc_no_correspondences(ctx):
    import torch
    e4 = torch.zeros((1, 4), dtype=torch.float32, device="cuda")
    ei = torch.zeros(0, dtype=torch.int32, device="cuda")
    ef = torch.zeros(0, dtype=torch.float32, device="cuda")
    mem, sizes, poses = ctx.gc_group(e4, e4, ei, ei, ef)
    assert len(sizes) == 0


def _random_scene(seed, nm, ns, C, spread=2.0):
    rng = np.random.default_rng(seed)
    mk = np.zeros((nm, 4), np.float32)
    mk[:, :3] = rng.uniform(-0.3, 0.3, (nm, 3))
    sk = np.zeros((ns, 4), np.float32)
    sk[:, :3] = rng.uniform(-spread, spread, (ns, 3))
    cm = rng.integers(0, nm, C).astype(np.int32)
    cs = rng.integers(0, ns, C).astype(np.int32)
    cd = rng.uniform(0, 0.3, C).astype(np.float32)
    cd[rng.choice(C, C // 10, replace=False)] = cd[0]  # many equal distances: ties keep input order
    return mk, sk, cm, cs, cd


@pytest.mark.parametrize("maxc", [1, 7, 256])
def test_gc_many_clusters_walk_stops_at_cap(ctx, maxc):
    # random correspondences in a small scene: nearly every seed forms a
    # cluster, so the walk commits densely, loses members to earlier commits
    # (recomputed sets) and stops at max_clusters
    mk, sk, cm, cs, cd = _random_scene(3, 600, 4000, 20000, 0.5)
    n = _check(ctx, mk, sk, cm, cs, cd, 0.01, 3, maxc)
    assert n == maxc


def test_gc_walk_reaches_the_end(ctx):
    # few clusters form: the walk runs past many windows to the last seed
    mk, sk, cm, cs, cd = _random_scene(4, 300, 3000, 9000, 3.0)
    _check(ctx, mk, sk, cm, cs, cd, 0.005, 4, 256)


def test_gc_wait_budget_runs_out_then_recovers(rtr):
    # a grid-barrier wait with no budget left returns RTR_ERR_TIMEOUT and the
    # context stays usable; the same call with the normal budget is exact
    mk, sk, cm, cs, cd = _random_scene(5, 600, 4000, 20000, 0.5)
    c = rtr.Context(0)
    try:
        args = (_dev(mk), _dev(sk), _dev(cm, np.int32), _dev(cs, np.int32), _dev(cd), 0.01, 3, 64, 128)
        c.set_wait_budget_ms(1e-6)
        with pytest.raises(rtr.RtrError, match="RTR_ERR_TIMEOUT"):
            c.gc_group(*args)
        with pytest.raises(rtr.RtrError, match="RTR_ERR_TIMEOUT"):
            c.check()  # the device status word saw it too (and is cleared by reading)
        c.set_wait_budget_ms(2000.0)
        c.check()
        _check(c, mk, sk, cm, cs, cd, 0.01, 3, 64)
    finally:
        c.close()


@pytest.mark.parametrize("case", ["dense", "far"])
def test_gc_without_pass_lists_same_clusters_more_rounds(rtr, case):
    """The walk recomputes a set that lost a member in place, from the pass
    list its admission kept; with no lists kept (the gc_pass_lists knob) every
    such set ends the round and the next round recomputes it.  Both give the
    oracle's clusters; the in-place form needs fewer rounds."""
    if case == "dense":
        mk, sk, cm, cs, cd = _random_scene(3, 600, 4000, 20000, 0.5)
        gc, th, maxc = 0.01, 3, 256
    else:
        mk, sk, cm, cs, cd = _random_scene(4, 300, 3000, 9000, 3.0)
        gc, th, maxc = 0.005, 4, 256
    c = rtr.Context(0)
    try:
        rounds = {}
        for off in (0, 1):
            c.set_tuning("gc_pass_lists", off)
            assert c.get_tuning("gc_pass_lists") == off
            _check(c, mk, sk, cm, cs, cd, gc, th, maxc)
            rounds[off] = c.gc_stats()["rounds"]
        assert rounds[0] <= rounds[1]
        if case == "dense":
            assert rounds[0] < rounds[1]
    finally:
        c.close()


def test_gc_nonfinite_scene_endpoints(ctx):
    """Scene keypoints with a NaN or infinite coordinate: the seed tests never
    skip the chunks that hold them (the consistency test of a NaN distance
    passes, as in the oracle), so the clusters stay the oracle's."""
    mk, sk, cm, cs, cd = _random_scene(6, 400, 3000, 12000, 0.6)
    used = np.unique(cs)
    rng = np.random.default_rng(6)
    bad = rng.choice(used, 6, replace=False)
    sk[bad[:3], 0] = np.nan
    sk[bad[3:], 1] = np.inf
    mem, sizes, _ = ctx.gc_group(_dev(mk), _dev(sk), _dev(cm, np.int32), _dev(cs, np.int32), _dev(cd),
                                 0.01, 3, 64, 128)
    mem, sizes = mem.cpu().numpy(), sizes.cpu().numpy()
    clus, _, rsizes = O.gc_group(mk, sk, cm, cs, cd, 0.01, 3, 64)
    assert np.array_equal(sizes, rsizes) and len(sizes) > 0
    for k in range(len(sizes)):
        assert set(mem[k][: sizes[k]].tolist()) == set(np.nonzero(clus == k)[0].tolist()), k
