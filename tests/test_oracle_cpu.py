"""CPU tests: the oracle against the reference's golden fixtures and against
independent numpy restatements.  No GPU needed."""
import numpy as np
import pytest

import oracle as O


def _rand_pts(rng, n, scale=1.0):
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(-scale, scale, (n, 3)).astype(np.float32)
    return p


def _np_d2(q, t):
    # same operation order as the oracle and the GPU: ((dx*dx + dy*dy) + dz*dz) in float32
    d = q[:, None, :3] - t[None, :, :3]
    xx, yy, zz = d[..., 0] * d[..., 0], d[..., 1] * d[..., 1], d[..., 2] * d[..., 2]
    return (xx + yy) + zz


def test_nn1_brute_matches_numpy_with_ties():
    rng = np.random.default_rng(0)
    t = _rand_pts(rng, 300)
    t[150:160] = t[10]  # duplicates: ties must go to the lowest index
    q = np.concatenate([_rand_pts(rng, 200), t[10:11], t[155:156]])
    idx, d2 = O.nn1(q, t, 0.0, "brute")
    D = _np_d2(q, t)
    ref = np.argmin(D, axis=1)  # argmin returns the first (lowest) index on ties
    assert (idx == ref).all()
    assert (d2 == D[np.arange(len(q)), ref]).all()
    assert idx[-1] == 10 and idx[-2] == 10


@pytest.mark.parametrize("max_dist", [0.0, 0.05, 0.2])
def test_nn1_grid_equals_brute(max_dist):
    rng = np.random.default_rng(1)
    t = _rand_pts(rng, 4000, 0.5)
    q = _rand_pts(rng, 3000, 0.7)  # some queries outside the target box
    a, da = O.nn1(q, t, max_dist, "brute")
    b, db = O.nn1(q, t, max_dist, "grid")
    assert (a == b).all() and np.array_equal(da, db)
    if max_dist:
        assert ((a >= 0) == (da <= np.float32(max_dist) * np.float32(max_dist))).all()


def test_knn_brute_matches_numpy():
    rng = np.random.default_rng(2)
    t = _rand_pts(rng, 500)
    q = _rand_pts(rng, 100)
    idx, d2 = O.knn(q, t, 10)
    D = _np_d2(q, t)
    ref = np.argsort(D, axis=1, kind="stable")[:, :10]
    assert (idx == ref).all()


def _umeyama_np(p, q):
    mp, mq = p.mean(0), q.mean(0)
    H = (p - mp).T @ (q - mq)
    U, S, Vt = np.linalg.svd(H)
    d = np.sign(np.linalg.det(Vt.T @ U.T))
    R = Vt.T @ np.diag([1, 1, d]) @ U.T
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = mq - R @ mp
    return T


def test_rigid_fit_matches_numpy_umeyama():
    rng = np.random.default_rng(3)
    import realtime_robot_gb300 as R
    for s in range(5):
        p = _rand_pts(rng, 200)
        T = R.synth_rigid(s, 40.0, 0.5)
        q = R.synth_transform_noise(p, T, 0.01, s)
        Tf, m = O.rigid_fit(p, q)
        Tn = _umeyama_np(p[:, :3].astype(np.float64), q[:, :3].astype(np.float64))
        assert m == 200
        assert np.abs(Tf - Tn).max() < 1e-12


def test_icp_known_answer_translation_pairs(golden):
    """The reference's recorded pairs: 5.pcd -> mcloud.pcd is a translation by
    (+0.8, +0.8, 0); 70761.pcd -> 70761_c.pcd by (+1, +0.5, 0)."""
    E = np.eye(4)
    E[:3, 3] = golden["t5"]
    r = O.icp(golden["p5"], golden["mcloud"], 50, 0.0)
    dt, dr = O.pose_error(r["pose"], E)
    assert dt < 1e-6 and dr < 1e-6
    # 1 m apart: start from the centroid offset (PCL would need a guess too)
    a, b = golden["p70761"], golden["p70761_c"]
    init = np.eye(4)
    init[:3, 3] = b[:, :3].astype(np.float64).mean(0) - a[:, :3].astype(np.float64).mean(0) + 0.01
    E[:3, 3] = golden["t70761"]
    r = O.icp(a, b, 30, 0.0, init=init)
    dt, dr = O.pose_error(r["pose"], E)
    assert dt < 1e-6 and dr < 1e-6


def test_recorded_failure_fixture_is_garbage():
    """transformed_cloud.pcd holds the recorded output of an uninitialised pose
    (function.h:39,108): coordinates around -1e8.  The new code must never emit
    such a pose; this pins what the failure looked like."""
    z = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "pcd_pairs.npz")
    assert np.all(np.abs(z["transformed_cloud_head"][:, :3]) > 1e7)


def test_icp_config0_recovers_pose():
    import realtime_robot_gb300 as R
    src, tgt, T = R.config0_pair(3, 5000)
    r = O.icp(src, tgt, 50, 0.05)
    dt, dr = O.pose_error(r["pose"], T)
    assert r["iterations"] == 50 and dt < 2e-3 and dr < np.deg2rad(0.5)


def test_tdf_oracle_small_cases():
    # single occupied voxel at the origin: value = min(900, x^2+y^2+z^2)
    out = O.tdf(np.array([[0, 0, 0]]), 30)
    z, y, x = np.meshgrid(np.arange(30), np.arange(30), np.arange(30), indexing="ij")
    ref = np.minimum(900, x * x + y * y + z * z).astype(np.float32).reshape(-1)
    assert np.array_equal(out, ref)
    # no occupied voxel: all 900 (kernel.cu:20)
    assert np.all(O.tdf(np.zeros((0, 3), np.int32), 12) == 900)
    # layout: x fastest (kernel.cu:16-18)
    out = O.tdf(np.array([[5, 0, 0]]), 6)
    assert out[5] == 0 and out[6 * 6 * 6 - 1] == (0 + 25 + 25)


def test_mlp_oracle_gradient_finite_differences():
    # pins the oracle's backward pass: central differences of its own loss
    # along the biases (the weight matrices are rounded to BF16 in the
    # forward pass, so their finite differences are steps, not slopes)
    from oracle import mlp as OM
    rng = np.random.default_rng(0)
    theta = OM.init_params(9).astype(np.float64)
    X = np.abs(rng.standard_normal((64, 352))).astype(np.float32)
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    y = (rng.random(64) > 0.5).astype(np.float32)
    _, g = OM.loss_and_grad(theta, X, y)
    p = OM.unpack(np.arange(OM.N_PARAMS))
    for name in ("b1", "b2", "b3"):
        for idx in p[name].ravel()[:8]:
            e = np.zeros(OM.N_PARAMS)
            e[int(idx)] = 1e-5
            lp, _ = OM.loss_and_grad((theta + e).astype(np.float32), X, y)
            lm, _ = OM.loss_and_grad((theta - e).astype(np.float32), X, y)
            fd = (lp - lm) / (2e-5)
            assert abs(fd - g[int(idx)]) < 2e-4 + 1e-2 * abs(fd), (name, int(idx), fd, g[int(idx)])


def test_range_search_oracle_against_numpy():
    """orc_range_search: every target within r (d^2 in float32 as
    ((dx*dx + dy*dy) + dz*dz)) or inside the float32 box [q - r, q + r],
    ascending, the count true and the list cut at max_per_query."""
    rng = np.random.default_rng(11)
    q = rng.uniform(-1, 1, (64, 4)).astype(np.float32)
    t = rng.uniform(-1, 1, (4000, 4)).astype(np.float32)
    q[3, 1] = np.nan
    t[7, 2] = np.inf
    dx = (q[:, None, 0] - t[None, :, 0]).astype(np.float32)
    dy = (q[:, None, 1] - t[None, :, 1]).astype(np.float32)
    dz = (q[:, None, 2] - t[None, :, 2]).astype(np.float32)
    d2 = ((dx * dx + dy * dy).astype(np.float32) + dz * dz).astype(np.float32)
    r = np.float32(0.25)
    lo, hi = (q[:, :3] - r).astype(np.float32), (q[:, :3] + r).astype(np.float32)
    inbox = np.all((t[None, :, :3] >= lo[:, None, :]) & (t[None, :, :3] <= hi[:, None, :]), axis=2)
    for box, want in ((False, d2 <= r * r), (True, inbox)):
        for m in (0, 5, 400):
            idx, cnt = O.range_search(q, t, float(r), box, m)
            assert np.array_equal(cnt, want.sum(1))
            for i in range(len(q)):
                hits = np.nonzero(want[i])[0]
                row = np.full(m, -1, np.int64)
                row[: min(m, len(hits))] = hits[:m]
                assert np.array_equal(idx[i], row)
    assert O.range_search(q, t, 0.25, False, 4)[1][3] == 0


def test_shot_descriptors_do_not_depend_on_point_order():
    """The SHOT restatement sums each keypoint's support in fixed point, so
    the descriptor of a keypoint and its LRF are the same bits whatever the
    order of the cloud (the GPU adds the support in lane and atomic order;
    this property is what lets the two agree bit for bit)."""
    rng = np.random.default_rng(5)
    pts = np.zeros((6000, 4), np.float32)
    # a box corner and a curved patch: support with every LRF case
    pts[:2000, :3] = rng.uniform(0, 0.1, (2000, 3)) * [1, 1, 0]
    pts[2000:4000, :3] = rng.uniform(0, 0.1, (2000, 3)) * [1, 0, 1]
    t = rng.uniform(0, np.pi, 2000)
    z = rng.uniform(0, 0.1, 2000)
    pts[4000:, 0], pts[4000:, 1], pts[4000:, 2] = 0.2 + 0.05 * np.cos(t), 0.05 * np.sin(t), z
    v = O.voxel_downsample(pts, 0.005)
    n = O.normals(v, 10, (0.5, 0.5, 0.5))
    k = O.uniform_sample(v, 0.02)
    d, lrf = O.shot352(v, n, k, 0.04)
    perm = rng.permutation(len(v))
    inv = np.argsort(perm)
    d2, lrf2 = O.shot352(v[perm], n[perm], inv[k].astype(np.int32), 0.04)
    assert np.array_equal(d, d2) and np.array_equal(lrf, lrf2)
    nrm = np.linalg.norm(d, axis=1)
    assert np.all(np.abs(nrm - 1.0) < 1e-5)


def test_shot_atan2_accuracy_and_conventions():
    """SHOT's own atan2 (the GPU kernel runs the same operations): within
    3e-7 rad of the true angle over every octant, 0 at the origin, and -0
    treated as +0."""
    rng = np.random.default_rng(3)
    ys = np.concatenate([rng.uniform(-1, 1, 4000), rng.uniform(-1e-6, 1e-6, 500), [0.0, 1.0, -1.0]])
    xs = np.concatenate([rng.uniform(-1, 1, 4000), rng.uniform(-1, 1, 500), [1.0, 0.0, 0.0]])
    worst = 0.0
    for y, x in zip(ys.astype(np.float32), xs.astype(np.float32)):
        worst = max(worst, abs(O.shot_atan2(float(y), float(x)) - np.arctan2(np.float64(y), np.float64(x))))
    assert worst < 3e-7, worst
    assert O.shot_atan2(0.0, 0.0) == 0.0
    assert O.shot_atan2(-0.0, -1.0) == np.float32(np.pi)
