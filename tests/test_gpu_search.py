"""GPU parity: exact 1-NN / k-NN through the C ABI vs the CPU oracle.
Indices and squared distances must be bit-exact (ties -> lowest index)."""
import numpy as np
import pytest

import oracle as O

from pathlib import Path

GOLDEN = Path(__file__).resolve().parent / "golden"

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _rand(rng, n, scale=1.0):
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(-scale, scale, (n, 3))
    return p


@pytest.mark.parametrize("max_dist", [0.0, 0.01, 0.05, 0.3])
def test_knn1_bit_exact_random(ctx, max_dist):
    rng = np.random.default_rng(10)
    t = _rand(rng, 20000, 0.5)
    q = _rand(rng, 15000, 0.6)
    idx, d2 = ctx.knn1(_dev(q), _dev(t), max_dist)
    ri, rd = O.nn1(q, t, max_dist, "brute")
    assert np.array_equal(idx.cpu().numpy(), ri)
    got = d2.cpu().numpy()
    ok = ri >= 0
    assert np.array_equal(got[ok], rd[ok]) and np.all(np.isinf(got[~ok]))


def test_knn1_ties_go_to_lowest_index(ctx):
    rng = np.random.default_rng(11)
    t = _rand(rng, 2000)
    t[1000:1100] = t[7]       # 101 copies of point 7
    t[1500] = t[1200]          # a later duplicate
    q = np.concatenate([t[[7, 1050, 1200, 1500]], _rand(rng, 100)])
    idx, _ = ctx.knn1(_dev(q), _dev(t), 0.0)
    idx = idx.cpu().numpy()
    assert list(idx[:4]) == [7, 7, 1200, 1200]
    ri, _ = O.nn1(q, t, 0.0, "brute")
    assert np.array_equal(idx, ri)


def test_knn1_surface_clouds_config0(ctx, rtr):
    src, tgt, T = rtr.config0_pair(5)
    q = O.transform_f32(T, src)
    for md in (0.05, 0.0):
        idx, d2 = ctx.knn1(_dev(q), _dev(tgt), md)
        ri, rd = O.nn1(q, tgt, md, "grid")
        assert np.array_equal(idx.cpu().numpy(), ri)


def test_knn1_edge_cases(ctx):
    rng = np.random.default_rng(12)
    t = _rand(rng, 1)
    q = _rand(rng, 50, 10.0)  # far outside a one-point grid
    idx, _ = ctx.knn1(_dev(q), _dev(t), 0.0)
    assert np.all(idx.cpu().numpy() == 0)
    idx, _ = ctx.knn1(_dev(q), _dev(t), 0.001)
    ri, _ = O.nn1(q, t, 0.001, "brute")
    assert np.array_equal(idx.cpu().numpy(), ri)
    # empty target: every index is -1
    import torch
    e = torch.zeros((0, 4), dtype=torch.float32, device="cuda")
    idx, _ = ctx.knn1(_dev(q), e, 0.0)
    assert np.all(idx.cpu().numpy() == -1)
    # all points identical (one cell, every distance ties)
    t = np.zeros((3000, 4), np.float32)
    idx, d2 = ctx.knn1(_dev(q[:10]), _dev(t), 0.0)
    assert np.all(idx.cpu().numpy() == 0)


@pytest.mark.parametrize("k", [1, 10, 16, 32])
def test_knn_bit_exact(ctx, k):
    rng = np.random.default_rng(13)
    t = _rand(rng, 6000, 0.5)
    t[100:120] = t[5]
    q = np.concatenate([_rand(rng, 3000, 0.55), t[[5, 110]]])
    idx, d2 = ctx.knn(_dev(q), _dev(t), k)
    ri, rd = O.knn(q, t, k)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)


@pytest.mark.parametrize("box", [False, True])
def test_range_search_equals_oracle(ctx, box):
    """rtr_radius_search / rtr_box_search against the oracle's brute force:
    the same indices in the same (ascending) order and the same counts, with
    cuts at max_per_query, non-finite points and an empty target set."""
    import torch
    rng = np.random.default_rng(5 + box)
    q = rng.uniform(-1, 1, (3000, 4)).astype(np.float32)
    t = rng.uniform(-1, 1, (50000, 4)).astype(np.float32)
    q[[5, 77], 0] = np.nan
    t[[3, 999], 1] = np.inf
    dq, dt = torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda()
    for r, m in ((0.05, 64), (0.12, 16), (0.3, 0), (3.0, 8)):
        idx, cnt = ctx.radius_search(dq, dt, r, m, box=box)
        oidx, ocnt = O.range_search(q, t, r, box, m)
        assert np.array_equal(cnt.cpu().numpy(), ocnt)
        assert np.array_equal(idx.cpu().numpy(), oidx)
    e = torch.zeros((0, 4), dtype=torch.float32, device="cuda")
    idx, cnt = ctx.radius_search(dq, e, 0.1, 4, box=box)
    assert int(cnt.sum()) == 0 and bool((idx == -1).all())


def test_box_search_at_keypoints_of_main_scan(ctx):
    """The reference's use: the +-10 cm box around each keypoint of the scan
    main registers (KeyPoint::getOccupiedGrid, key_point.h:118-140)."""
    import torch
    d = np.load(GOLDEN / "main_clouds.npz")
    scan = np.ascontiguousarray(d["T0_m8111"], np.float32)
    keys = scan[O.uniform_sample(scan, 0.05)]
    idx, cnt = ctx.radius_search(torch.from_numpy(keys).cuda(), torch.from_numpy(scan).cuda(), 0.1, 4096, box=True)
    oidx, ocnt = O.range_search(keys, scan, 0.1, True, 4096)
    assert np.array_equal(cnt.cpu().numpy(), ocnt) and ocnt.max() < 4096
    assert np.array_equal(idx.cpu().numpy(), oidx)
