"""The reference's own descriptor route (getOccupiedGrid, get_TSDF,
get_Distance, the gates of the all-pairs loop, Ransac): the C oracle
(oracle/refmatch.c) against a second, independent numpy restatement of the
same rules on small cases, the gates' written-as-is quirks, and the oracle on
the reference's own clouds (chair1.pcd / T0_m8111.pcd, tests/golden)."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O

F32 = np.float32
EPS = float(np.finfo(np.float32).eps)
GOLDEN = Path(__file__).resolve().parent / "golden"


# ---- numpy restatement of the octree rules ---------------------------------
def np_define(lo, hi, res):
    ext = hi.astype(np.float64) - lo.astype(np.float64)
    mv = max(2, int(np.max(np.ceil((ext - EPS) / res))))
    d = 0
    while (1 << d) < mv:
        d += 1
    over = (float(1 << d) * res - ext) / 2.0
    mn, mx = lo.astype(np.float64), hi.astype(np.float64)
    pad = over > EPS
    mn[pad] -= over[pad]
    mx[pad] += over[pad]
    return {"mn": mn, "mx": mx, "d": d}


def np_outside(b, P):
    P = P.astype(np.float64)
    return np.any(P < b["mn"], axis=1) | np.any(P >= b["mx"], axis=1)


def np_grow(b, p, res):
    while True:
        up = p.astype(np.float64) >= b["mx"]
        if not (np.any(up) or np.any(p.astype(np.float64) < b["mn"])):
            return True
        if b["d"] >= 21:
            return False
        side = float(1 << b["d"]) * res
        b["mn"] = np.where(up, b["mn"], b["mn"] - side)
        b["d"] += 1
        b["mx"] = b["mn"] + (float(1 << b["d"]) * res - EPS)


def np_keys(b, P, res):
    k = np.floor((P.astype(np.float64) - b["mn"]) / res).astype(np.int64)
    return np.minimum(k, (1 << b["d"]) - 1)


def np_morton(K, d):
    m = np.zeros(K.shape[0], np.uint64)
    for lv in range(d - 1, -1, -1):
        bits = ((K[:, 0] >> lv) & 1) * 4 + ((K[:, 1] >> lv) & 1) * 2 + ((K[:, 2] >> lv) & 1)
        m = (m << np.uint64(3)) | bits.astype(np.uint64)
    return m


def np_leaves(b, P, res):
    K = np_keys(b, P, res)
    m = np_morton(K, b["d"])
    _, first = np.unique(m, return_index=True)  # sorted by Morton code
    return K[first]


def np_centre(b, K, res):
    return ((K.astype(np.float64) + 0.5) * res + b["mn"]).astype(F32)


def np_box(key, half):
    k = key[:3].astype(F32)
    return k - F32(half), k + F32(half)


def np_xf(M, P):
    M = M.astype(F32)
    out = np.empty_like(P)
    for a in range(3):
        s = M[a, 0] * P[:, 0]
        s = s + M[a, 1] * P[:, 1]
        s = s + M[a, 2] * P[:, 2]
        out[:, a] = s + M[a, 3]
    return out


def np_mm(A, B):
    C = np.zeros((4, 4), F32)
    for r in range(4):
        for c in range(4):
            s = A[r, 0] * B[0, c]
            s = s + A[r, 1] * B[1, c]
            s = s + A[r, 2] * B[2, c]
            C[r, c] = s + A[r, 3] * B[3, c]
    return C


def np_occupancy(cloud, key, res, half):
    lo, hi = np_box(key, half)
    P = cloud[:, :3]
    inside = np.all(P >= lo, axis=1) & np.all(P <= hi, axis=1)
    idx = np.nonzero(inside)[0]
    b = np_define(lo, hi, float(F32(res)))
    number = np_leaves(b, P[idx], float(F32(res))).shape[0] if idx.size else 0
    return idx, number


def np_tdf_occ(cloud, key, idx, res, half):
    lo, hi = np_box(key, half)
    r = float(F32(res))
    b = np_define(lo, hi, r)
    L = np_leaves(b, cloud[idx, :3], r) if idx.size else np.zeros((0, 3), np.int64)
    L = L[1:]
    ctr = np_centre(b, L, r)
    return ((ctr.astype(np.float64) - lo.astype(np.float64)) / r).astype(np.int32)


def np_distance(cloud, km, idx, grid, ks, res=0.01, half=0.15):
    r32 = F32(res)
    r = float(r32)
    lo, hi = np_box(km, half)
    k3, s3 = km[:3].astype(F32), ks[:3].astype(F32)
    Tm = np.eye(4, dtype=F32)
    Tm[:3, 3] = k3 - s3
    P = np_xf(Tm, cloud[idx, :3].astype(F32))
    theta = F32(np.pi / 18)
    c1, s1 = np.cos(theta, dtype=F32), np.sin(theta, dtype=F32)
    T1, T3, Rs = np.eye(4, dtype=F32), np.eye(4, dtype=F32), np.eye(4, dtype=F32)
    T1[0, 3], T1[1, 3] = -k3[0], -k3[1]
    T3[0, 3], T3[1, 3] = k3[0], k3[1]
    Rs[0, 0], Rs[1, 0], Rs[0, 1], Rs[1, 1] = c1, s1, -s1, c1
    M = np_mm(np_mm(T3, Rs), T1)
    dt, best, best_i = F32(0), F32(1e8), 0
    for i in range(36):
        if i:
            P = np_xf(M, P)
        b = np_define(lo, hi, r)
        while True:
            out = np.nonzero(np_outside(b, P))[0]
            if out.size == 0:
                break
            assert np_grow(b, P[out[0]], r)
        L = np_leaves(b, P, r)
        u = L.shape[0]
        if u > 1:
            ctr = np_centre(b, L[1:], r)
            q = (ctr - lo) / r32
            ix = np.trunc(q).astype(np.int64)
            lin = ix[:, 1] * 30 + ix[:, 2] * 900 + ix[:, 0]
            ok = (lin >= 0) & (lin < 27000)
            v = np.where(ok, grid[np.clip(lin, 0, 26999)], F32(900)).astype(F32)
            # matching.h:179-189: float adds, leaf by leaf in tree order,
            # into the running score that no rotation resets
            for x in v:
                dt = F32(dt + F32(x * x))
        div = F32(18446744073709551615.0) if u == 0 else F32(u - 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            dt = F32(F32(dt) / div)
        if dt < best:
            best, best_i = dt, i
    th = F32(best_i) * theta
    R2 = np.eye(4, dtype=F32)
    c2, s2 = F32(np.cos(np.float64(th))), F32(np.sin(np.float64(th)))
    R2[0, 0], R2[1, 0], R2[0, 1], R2[1, 1] = c2, s2, -s2, c2
    S = np.eye(4, dtype=F32)
    S[0, 0] = S[1, 1] = S[2, 2] = k3[2] / s3[2]
    T = np_mm(np_mm(np_mm(np_mm(S, T3), R2), T1), Tm)
    return F32(best), T


# ---- fixtures ----------------------------------------------------------------
def _chair_case(seed=3, n=3000, nk=12, ns=9, shift=0.0):
    import realtime_robot_gb300 as R
    model = R.synth_shape(R.CHAIR, n, 2024 + seed)
    scan = R.synth_shape(R.CHAIR, n, 7 + seed).copy()
    scan[:, :3] += np.float32(shift)
    rng = np.random.default_rng(seed)
    km = model[rng.choice(n, nk, replace=False)]
    ks = scan[rng.choice(n, ns, replace=False)]
    return model, scan, km, ks


def test_occupancy_and_number_match_numpy():
    model, _, km, _ = _chair_case()
    number, off, idx = O.ref_occupancy(model, km, 0.01, 0.1)
    for k in range(km.shape[0]):
        ref_idx, ref_num = np_occupancy(model, km[k], 0.01, 0.1)
        assert np.array_equal(idx[off[k]:off[k + 1]], ref_idx), k
        assert number[k] == ref_num, k
    # a keypoint far from the cloud: empty box, Number 0
    far = np.array([[50.0, 50.0, 50.0, 0.0]], np.float32)
    n2, o2, _ = O.ref_occupancy(model, far, 0.01, 0.1)
    assert n2[0] == 0 and o2[1] == 0


def test_tdf_drops_the_first_leaf_and_matches_numpy():
    model, _, km, _ = _chair_case()
    _, off, idx = O.ref_occupancy(model, km, 0.01, 0.1)
    tdf = O.ref_tdf(model, km, off, idx, 0.01, 0.15)
    assert tdf.shape == (km.shape[0], 27000)
    for k in range(km.shape[0]):
        occ = np_tdf_occ(model, km[k], idx[off[k]:off[k + 1]], 0.01, 0.15)
        assert np.array_equal(tdf[k], O.tdf(occ, 30)), k
        assert occ.min() >= 0 and occ.max() < 30
    # an empty keypoint: no occupied voxel, the cap everywhere
    far = np.array([[50.0, 50.0, 50.0, 0.0]], np.float32)
    _, o2, i2 = O.ref_occupancy(model, far, 0.01, 0.1)
    assert np.all(O.ref_tdf(model, far, o2, i2) == 900.0)


@pytest.mark.parametrize("shift", [0.0, 0.7, -2.5])
def test_distance_matches_numpy(shift):
    """Scores and transforms bit for bit, including pairs far apart (the
    rotated cloud leaves the field's box: the octree grows)."""
    model, scan, km, ks = _chair_case(nk=4, ns=3, shift=shift)
    _, off, idx = O.ref_occupancy(model, km, 0.01, 0.1)
    tdf = O.ref_tdf(model, km, off, idx, 0.01, 0.15)
    score, T = O.ref_distance(model, km, off, idx, tdf, ks)
    for m in range(km.shape[0]):
        for s in range(ks.shape[0]):
            p = m * ks.shape[0] + s
            sc, Tr = np_distance(model, km[m], idx[off[m]:off[m + 1]], tdf[m], ks[s])
            assert score[p] == sc, (m, s, score[p], sc)
            assert np.array_equal(T[p], Tr), (m, s)


def test_distance_explicit_pairs_equal_all_pairs():
    model, scan, km, ks = _chair_case(nk=5, ns=4)
    _, off, idx = O.ref_occupancy(model, km, 0.01, 0.1)
    tdf = O.ref_tdf(model, km, off, idx)
    s_all, T_all = O.ref_distance(model, km, off, idx, tdf, ks)
    pm = np.array([4, 0, 2, 2], np.int32)
    ps = np.array([3, 1, 0, 0], np.int32)
    s_p, T_p = O.ref_distance(model, km, off, idx, tdf, ks, pm, ps)
    assert np.array_equal(s_p, s_all[pm * 4 + ps]) and np.array_equal(T_p, T_all[pm * 4 + ps])


def test_float_order_agrees_with_exact_sums():
    """The reference adds the squared field values in float, leaf by leaf
    (the route's definition); the variant with exact per-rotation sums and a
    double running score agrees to a few parts in 10^5."""
    model, scan, km, ks = _chair_case(nk=10, ns=10)
    _, off, idx = O.ref_occupancy(model, km, 0.01, 0.1)
    tdf = O.ref_tdf(model, km, off, idx)
    s1, _ = O.ref_distance(model, km, off, idx, tdf, ks, float_order=False)
    s2, _ = O.ref_distance(model, km, off, idx, tdf, ks)
    ok = np.isfinite(s1)
    assert ok.all()
    rel = np.abs(s1.astype(np.float64) - s2) / np.maximum(np.abs(s1.astype(np.float64)), 1e-30)
    assert rel.max() < 1e-4, rel.max()


def test_gates_as_written():
    k = np.array([0.0, 0.0, 1.0, 0.0], np.float32)
    v = np.full(3, 0.16)

    def g(kz, sz, nm=10, ns=10, mv3=v, sv3=v):
        a = np.array([0, 0, kz, 0], np.float32)
        b = np.array([0, 0, sz, 0], np.float32)
        return O.lib().orc_ref_gates(a.ctypes.data, nm, mv3.ctypes.data, b.ctypes.data, ns, sv3.ctypes.data)

    # height: float(2/3) == 0, so any ratio passes but NaN
    assert g(1.0, 1000.0) and g(1000.0, 1.0) and g(-1.0, 1.0) and g(0.0, 0.0) == 0
    # area: above 3 fails, no lower bound (float(1/3) == 0)
    assert g(1, 1, mv3=np.array([0.5, 0.16, 0.16]), sv3=v) == 0
    assert g(1, 1, mv3=np.array([0.001, 0.16, 0.16]), sv3=v) == 1
    # occupancy: integer quotient Number_m / Number_s kept in [1, 2]
    assert g(1, 1, nm=9, ns=10) == 0 and g(1, 1, nm=10, ns=10) and g(1, 1, nm=29, ns=10)
    assert g(1, 1, nm=30, ns=10) == 0 and g(1, 1, nm=5, ns=0) == 0
    del k


def test_ransac_known_answer():
    """Five pairs agree on one transform, two do not: the first of the five
    wins with five inliers."""
    rng = np.random.default_rng(0)
    ks = np.zeros((7, 4), np.float32)
    ks[:, :3] = rng.uniform(-0.3, 0.3, (7, 3))
    Tgood = np.eye(4, dtype=np.float32)
    Tgood[:3, 3] = [0.2, -0.1, 0.05]
    km = ks.copy()
    km[:, :3] = np_xf(Tgood, ks[:, :3])
    km[5, :3] += 1.0
    km[6, :3] -= 1.0
    ns = ks.shape[0]
    pair_idx = np.array([m * ns + m for m in range(7)], np.int32)
    P = 7 * ns
    score = np.zeros(P, np.float32)
    T_all = np.tile(np.eye(4, dtype=np.float32), (P, 1, 1))
    for m in range(7):
        T_all[m * ns + m] = Tgood
    T_all[5 * ns + 5][:3, 3] = [5.0, 5.0, 5.0]
    T_all[6 * ns + 6][:3, 3] = [-5.0, 0.0, 0.0]
    T, inl, best = O.ref_ransac(km, ks, pair_idx, score, T_all)
    assert best == 0 and inl == 5 and np.array_equal(T, Tgood)
    # a pair's score at max_des or above does not count as an inlier
    score[2 * ns + 2] = 100.0
    T, inl, best = O.ref_ransac(km, ks, pair_idx, score, T_all)
    assert inl == 4
    # no inlier anywhere: the identity (the reference's matrix is uninitialised)
    T, inl, best = O.ref_ransac(km, ks, pair_idx, score, np.tile(np.eye(4, dtype=np.float32) * 0, (P, 1, 1)) + 100)
    assert best == -1 and inl == 0 and np.array_equal(T, np.eye(4, dtype=np.float32))


def test_route_on_the_reference_clouds():
    """main's route on its own inputs (chair1.pcd model, T0_m8111.pcd scan),
    keypoints sampled at 5 cm: every stage runs, the scores are finite, and
    the kept pairs are those below 3 that pass the gates."""
    d = np.load(GOLDEN / "main_clouds.npz")
    model, scan = d["chair1"], d["T0_m8111"]
    km = model[O.uniform_sample(model, 0.08)]
    ks = scan[O.uniform_sample(scan, 0.08)]
    mn, mo, mi = O.ref_occupancy(model, km)
    sn, so, si = O.ref_occupancy(scan, ks)
    assert mn.min() > 0 and sn.min() > 0
    tdf = O.ref_tdf(model, km, mo, mi)
    sc, T = O.ref_distance(model, km, mo, mi, tdf, ks)
    assert np.isfinite(sc).all()
    pi = O.ref_correspond(km, mn, ks, sn, sc)
    m, s = pi // ks.shape[0], pi % ks.shape[0]
    assert np.all(sc[pi] < 3)
    q = (mn[m] // sn[s])
    assert np.all((q >= 1) & (q <= 2))
