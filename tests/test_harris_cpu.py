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
