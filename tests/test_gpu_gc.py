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
