"""The reference's own descriptor route on the GPU (rtr_ref_*: getOccupiedGrid,
get_TSDF, get_Distance, the gated all-pairs loop, Ransac) against the CPU
oracle (oracle/refmatch.c), bit for bit: integer outputs equal, float scores
and transforms equal, NaN where the oracle has NaN."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _route(ctx, model, scan, km, ks):
    """Every stage on the GPU and in the oracle; asserts equality, returns
    the oracle's (scores, transforms)."""
    dm, ds, dkm, dks = _dev(model), _dev(scan), _dev(km), _dev(ks)
    mn, mo, mi = ctx.ref_occupancy(dm, dkm)
    sn, so, si = ctx.ref_occupancy(ds, dks)
    rmn, rmo, rmi = O.ref_occupancy(model, km)
    rsn, rso, rsi = O.ref_occupancy(scan, ks)
    assert np.array_equal(mn.cpu().numpy(), rmn) and np.array_equal(mo.cpu().numpy(), rmo)
    assert np.array_equal(mi.cpu().numpy(), rmi)
    assert np.array_equal(sn.cpu().numpy(), rsn) and np.array_equal(so.cpu().numpy(), rso)
    assert np.array_equal(si.cpu().numpy(), rsi)
    tdf = ctx.ref_tdf(dm, dkm, mo, mi)
    rtdf = O.ref_tdf(model, km, rmo, rmi)
    assert np.array_equal(tdf.cpu().numpy(), rtdf)
    sc, T = ctx.ref_distance(dm, dkm, mo, mi, tdf, dks)
    rsc, rT = O.ref_distance(model, km, rmo, rmi, rtdf, ks)
    g = sc.cpu().numpy()
    assert np.array_equal(np.isnan(g), np.isnan(rsc))
    ok = ~np.isnan(rsc)
    bad = np.nonzero(g[ok] != rsc[ok])[0]
    assert bad.size == 0, (bad[:5], g[ok][bad[:5]], rsc[ok][bad[:5]])
    assert np.array_equal(T.cpu().numpy(), rT, equal_nan=True)
    pi = ctx.ref_correspond(dkm, mn, dks, sn, sc)
    rpi = O.ref_correspond(km, rmn, ks, rsn, rsc)
    assert np.array_equal(pi.cpu().numpy(), rpi)
    if rpi.size:
        Tb, inl, best = ctx.ref_ransac(dkm, dks, pi, sc, T)
        rTb, rinl, rbest = O.ref_ransac(km, ks, rpi, rsc, rT)
        assert (inl, best) == (rinl, rbest) and np.array_equal(Tb, rTb)
    return rsc, rT, rpi


def test_route_on_the_reference_clouds(ctx):
    """main's inputs (chair1.pcd model, T0_m8111.pcd scan), keypoints every
    5 cm: 340 x 573 pairs, every stage equal to the oracle."""
    d = np.load(GOLDEN / "main_clouds.npz")
    model, scan = d["chair1"], d["T0_m8111"]
    km = model[O.uniform_sample(model, 0.05)]
    ks = scan[O.uniform_sample(scan, 0.05)]
    sc, _, pi = _route(ctx, model, scan, km, ks)
    assert np.isfinite(sc).all() and pi.size > 0


def test_route_on_a_synthetic_chair(ctx, rtr):
    """A 20k-point chair (occupancy clouds of up to ~2.5k points: the
    512-thread pair kernel) against a cropped, turned copy."""
    model = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    th = np.radians(20.0)
    T = np.eye(4)
    T[:3, :3] = [[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]]
    T[:3, 3] = [0.05, -0.03, 0.0]
    scan = rtr.synth_transform_noise(rtr.synth_crop(rtr.synth_shape(rtr.CHAIR, 20000, 501), 0.3, 1), T, 0.002, 10)
    km = model[O.uniform_sample(model, 0.1)]
    ks = scan[O.uniform_sample(scan, 0.1)]
    _route(ctx, model, scan, km, ks)


def test_dense_occupancy_and_explicit_pairs(ctx, rtr):
    """60k points on the chair: occupancy clouds above 4096 points (the
    1024-thread pair kernel), the index buffer regrown past its first
    capacity; explicit pair lists equal the all-pairs result."""
    model = rtr.synth_shape(rtr.CHAIR, 60000, 11)
    scan = rtr.synth_shape(rtr.CHAIR, 30000, 12)
    rng = np.random.default_rng(5)
    km = model[rng.choice(model.shape[0], 24, replace=False)]
    ks = scan[rng.choice(scan.shape[0], 5, replace=False)]
    dm, dkm, dks = _dev(model), _dev(km), _dev(ks)
    mn, mo, mi = ctx.ref_occupancy(dm, dkm)
    rmn, rmo, rmi = O.ref_occupancy(model, km)
    assert np.array_equal(mo.cpu().numpy(), rmo) and np.array_equal(mi.cpu().numpy(), rmi)
    assert np.diff(rmo).max() > 4096 and rmo[-1] > (1 << 16)
    tdf = ctx.ref_tdf(dm, dkm, mo, mi)
    rtdf = O.ref_tdf(model, km, rmo, rmi)
    assert np.array_equal(tdf.cpu().numpy(), rtdf)
    pm = np.array([20, 5, 13, 13, 7, 2], np.int32)  # 20: the largest occupancy cloud (5,589 points)
    ps = np.array([4, 0, 2, 1, 1, 3], np.int32)
    sc, T = ctx.ref_distance(dm, dkm, mo, mi, tdf, dks, _dev(pm), _dev(ps))
    rsc, rT = O.ref_distance(model, km, rmo, rmi, rtdf, ks, pm, ps)
    assert np.array_equal(sc.cpu().numpy(), rsc) and np.array_equal(T.cpu().numpy(), rT)


def test_edge_cases(ctx, rtr):
    """A keypoint with an empty box (Number 0, field all 900, score 0 as in
    the reference), a non-finite scan keypoint (NaN, identity), a scan
    keypoint 40 m away (the octree grows 8 levels)."""
    model = rtr.synth_shape(rtr.CHAIR, 4000, 3)
    km = np.concatenate([model[:3], np.array([[30.0, 30.0, 30.0, 0.0]], np.float32)])
    ks = np.array([[0.1, 0.2, 0.4, 0], [np.nan, 0.0, 0.3, 0], [40.0, -3.0, 1.0, 0], [0.0, 0.0, 0.0, 0]],
                  np.float32)
    dm, dkm, dks = _dev(model), _dev(km), _dev(ks)
    mn, mo, mi = ctx.ref_occupancy(dm, dkm)
    assert mn.cpu().numpy()[3] == 0
    tdf = ctx.ref_tdf(dm, dkm, mo, mi)
    assert np.all(tdf.cpu().numpy()[3] == 900.0)
    sc, T = ctx.ref_distance(dm, dkm, mo, mi, tdf, dks)
    rmn, rmo, rmi = O.ref_occupancy(model, km)
    rsc, rT = O.ref_distance(model, km, rmo, rmi, O.ref_tdf(model, km, rmo, rmi), ks)
    g = sc.cpu().numpy()
    assert np.array_equal(np.isnan(g), np.isnan(rsc)) and np.isnan(g[1::4]).all()
    assert np.array_equal(g[~np.isnan(g)], rsc[~np.isnan(rsc)])
    # the scan keypoint at z = 0 scales by kz / 0: inf and NaN entries, equal too
    assert np.array_equal(T.cpu().numpy(), rT, equal_nan=True)
    assert np.array_equal(T.cpu().numpy()[1], np.eye(4, dtype=np.float32))


def test_bad_arguments_are_refused(ctx, rtr):
    model = _dev(rtr.synth_shape(rtr.CHAIR, 2000, 3))
    keys = model[:4].contiguous()
    with pytest.raises(rtr.RtrError):
        ctx.ref_occupancy(model, keys, 0.01, 0.5)  # 100 leaves across: beyond the 32^3 bitmap
    _, mo, mi = ctx.ref_occupancy(model, keys)
    with pytest.raises(rtr.RtrError):
        ctx.ref_tdf(model, keys, mo, mi, 0.01, 0.2)  # dim 40 > 30
    tdf = ctx.ref_tdf(model, keys, mo, mi)
    import torch
    bad_m = torch.tensor([0, 7], dtype=torch.int32, device="cuda")
    bad_s = torch.tensor([0, 0], dtype=torch.int32, device="cuda")
    with pytest.raises(rtr.RtrError):
        ctx.ref_distance(model, keys, mo, mi, tdf, keys, bad_m, bad_s)  # model index 7 of 4
    ctx.check()
