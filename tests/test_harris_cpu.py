"""The oracle's Harris3D detector (oracle/harris.c), the keypoints of
ModelPoint / ScanPoint::getKeypoint (model_point.h:127-136,
scan_point.h:85-94): corners of box shapes are found and refined onto the
corner; faces and edges give none."""
import numpy as np

import oracle as O
from oracle import synth as S


def _cube(n, e, seed):
    """n points uniform on the surface of an axis-aligned cube of edge e."""
    rng = np.random.default_rng(seed)
    face = rng.integers(0, 6, n)
    uv = rng.uniform(-e / 2, e / 2, (n, 2))
    p = np.zeros((n, 4), np.float32)
    ax = face // 2
    sign = np.where(face % 2 == 0, -1.0, 1.0) * e / 2
    for a in range(3):
        others = [b for b in range(3) if b != a]
        m = ax == a
        p[m, a] = sign[m]
        p[m, others[0]] = uv[m, 0]
        p[m, others[1]] = uv[m, 1]
    return p


def test_cube_corners_found_and_refined():
    e = 0.3
    pts = _cube(30000, e, 1)
    keys, src = O.harris3d(pts)
    raw, _ = O.harris3d(pts, refine=False)
    corners = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]) * e / 2
    d = np.linalg.norm(keys[:, None, :3] - corners[None], axis=2)
    d_raw = np.linalg.norm(raw[:, None, :3] - corners[None], axis=2)
    # one keypoint per corner: 2.5-4 cm in on the faces, refined to about
    # 1 cm (the radius-5 cm normals near the edges are blends of two faces)
    assert len(keys) == len(raw) == 8
    assert np.all(d_raw.min(1) < 0.04) and np.all(d.min(1) < 0.012) and np.all(d.min(1) < d_raw.min(1))
    assert sorted(d.argmin(1).tolist()) == list(range(8))
    assert np.all(keys[:, 3] > 0.01) and np.all(keys[:, 3] <= 1.0 / 27 + 1e-4)


def test_unrefined_keypoints_are_cloud_points_and_local_maxima():
    pts = S.synth_shape(S.CHAIR, 20000, 2024)
    keys, src = O.harris3d(pts, refine=False)
    assert len(keys) > 0 and np.array_equal(keys[:, :3], pts[src, :3])
    all_keys, all_src = O.harris3d(pts, refine=False, non_max=False)
    assert set(src.tolist()) <= set(all_src.tolist()) and len(all_src) > len(src)
    # a plane (faces only) has no keypoint
    rng = np.random.default_rng(3)
    plane = np.zeros((5000, 4), np.float32)
    plane[:, :2] = rng.uniform(-0.5, 0.5, (5000, 2))
    assert len(O.harris3d(plane)[0]) == 0


def test_responses_against_numpy():
    """Every point's Harris response against a float64 numpy restatement of
    the operator: radius neighbours (the point included), normals as the
    smallest covariance eigenvectors, M = mean of n n^T over the neighbours,
    R = det(M) - 0.04 tr(M)^2 + 0.04 (unit normals: R = det(M)).  Points whose
    own or whose neighbours' smallest eigenvalues are not separated (their
    normal is not defined to float precision) are left out."""
    spatial = __import__("pytest").importorskip("scipy.spatial")
    pts = _cube(3000, 0.3, 4)
    keys, src = O.harris3d(pts, 0.05, -1.0, non_max=False, refine=False)
    assert len(src) == len(pts)
    P = pts[:, :3].astype(np.float64)
    nb = spatial.cKDTree(P).query_ball_point(P, 0.05 * (1 + 1e-6))
    nrm = np.zeros((len(P), 3))
    ok = np.zeros(len(P), bool)
    for i, js in enumerate(nb):
        Q = P[js] - P[js].mean(0)
        w, V = np.linalg.eigh(Q.T @ Q / len(js))
        nrm[i] = V[:, 0]
        ok[i] = w[1] - w[0] > 1e-3 * w[2]
    resp = np.full(len(P), np.nan)
    for i, js in enumerate(nb):
        if not ok[js].all():
            continue
        M = nrm[js].T @ nrm[js] / len(js)
        resp[i] = np.linalg.det(M) - 0.04 * np.trace(M) ** 2 + 0.04
    got = np.full(len(P), np.nan)
    got[src] = keys[:, 3]
    sel = ~np.isnan(resp)
    assert sel.mean() > 0.5
    np.testing.assert_allclose(got[sel], resp[sel], atol=2e-5)
