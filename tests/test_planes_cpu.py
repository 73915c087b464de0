"""The oracle's plane segmentation and plane-area vector (oracle/planes.c),
restating ModelPoint::getArea / ScanPoint::get_Area (model_point.h:170-245,
scan_point.h:117-188), is_h_plane / is_v_plane (model_point.h:48-79) and
KeyPoint::get_Vector3D (key_point.h:87-111).

The hull measure is pinned against Qhull, the library PCL's ConvexHull
calls (SciPy's bundled copy): for a 2-D hull Qhull reports the enclosed area
as its "volume" and the perimeter as its "area"."""
import numpy as np
import pytest

import oracle as O
from oracle import synth as S


def _rect(n, w, h, seed, z=0.0, noise=0.0, tilt_deg=0.0):
    """n points on a w x h rectangle at height z, tilted about x."""
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 4), np.float32)
    p[:, 0] = rng.uniform(-w / 2, w / 2, n)
    y = rng.uniform(-h / 2, h / 2, n)
    t = np.radians(tilt_deg)
    p[:, 1] = y * np.cos(t)
    p[:, 2] = z + y * np.sin(t) + (rng.normal(0, noise, n) if noise else 0.0)
    return p


def test_hull_area_and_perimeter_match_qhull():
    spatial = pytest.importorskip("scipy.spatial")
    for seed in range(4):
        rng = np.random.default_rng(seed)
        pts = np.zeros((3000, 4), np.float32)
        # a horizontal blob of irregular outline in z = 0
        r = rng.uniform(0, 1, 3000) ** 0.5 * (0.5 + 0.3 * rng.uniform(0, 1))
        a = rng.uniform(0, 2 * np.pi, 3000)
        pts[:, 0] = (r * np.cos(a) * (1 + 0.5 * seed)).astype(np.float32)
        pts[:, 1] = (r * np.sin(a)).astype(np.float32)
        surf, tot = O.plane_segment(pts, remain_frac=0.0)
        assert tot == 1 and surf[0].n_inliers == 3000
        hull = spatial.ConvexHull(pts[:, :2].astype(np.float64))
        assert surf[0].area == pytest.approx(hull.volume, rel=1e-9)
        assert surf[0].perimeter == pytest.approx(hull.area, rel=1e-9)
        assert surf[0].hull_vertices == len(hull.vertices)


def test_planes_of_a_box_scene_known_answers():
    # floor 2 x 1 m, a 1 x 0.6 m wall (vertical), a 45-degree ramp
    floor = _rect(20000, 2.0, 1.0, 1, noise=0.001, tilt_deg=2.0)
    wall = _rect(8000, 1.0, 0.6, 2, noise=0.001)
    wall[:, [1, 2]] = wall[:, [2, 1]]  # into the x-z plane
    wall[:, 1] += 0.8
    wall[:, 2] += 0.4
    ramp = _rect(6000, 0.8, 0.8, 3, noise=0.001)
    c = np.float32(np.sqrt(0.5))
    y, z = ramp[:, 1].copy(), ramp[:, 2].copy()
    ramp[:, 1], ramp[:, 2] = y * c - z * c, y * c + z * c + 1.5
    pts = np.concatenate([floor, wall, ramp])
    surf, tot = O.plane_segment(pts, remain_frac=0.05)
    byn = sorted(surf, key=lambda s: -s.n_inliers)
    f, w, r = byn[:3]
    assert f.n_inliers == 20000 and f.is_vertical == 0 and f.kept and f.area == pytest.approx(2.0, rel=0.01)
    assert abs(f.perimeter - 6.0) < 0.05
    assert w.n_inliers == 8000 and w.is_vertical == 1 and w.kept and w.area == pytest.approx(0.6, rel=0.02)
    assert r.n_inliers == 6000 and r.is_vertical == -1 and not r.kept and r.area == pytest.approx(0.64, rel=0.02)
    for s in byn[:3]:
        assert s.flat == 1


def test_segmentation_stops_at_the_remaining_fraction_and_drops_nonfinite_points():
    pts = np.concatenate([_rect(5000, 1.0, 1.0, 4), _rect(800, 0.5, 0.5, 5, z=0.3)])
    surf, tot = O.plane_segment(pts)  # 800 of 5800 left after the first plane: <= 15 %
    assert tot == 1 and surf[0].n_inliers == 5000
    bad = np.insert(pts, [0, 100, 3000], np.float32([np.nan, 0, 0, 0]), axis=0)
    s2, t2 = O.plane_segment(bad)
    assert t2 == tot and s2[0].n_inliers == surf[0].n_inliers and s2[0].area == surf[0].area


def test_exactly_horizontal_plane_is_neither_as_written():
    """is_h_plane tests 0 < angle < 10 deg and 170 deg < angle < 3.1415926
    on float coefficients: a normal whose float z component is 1 (tilt below
    about 0.02 deg) passes neither, so such a plane is not a surface of the
    reference's list, however large."""
    for noise in (0.0, 0.001):
        surf, _ = O.plane_segment(_rect(4000, 1.0, 1.0, 9, noise=noise))
        assert surf[0].is_vertical == -1 and not surf[0].kept
    surf, _ = O.plane_segment(_rect(4000, 1.0, 1.0, 9, noise=0.001, tilt_deg=2.0))
    assert surf[0].is_vertical == 0 and surf[0].kept


def test_room_planes_and_model_planes():
    scene, _, _ = S.synth_room(1)
    surf, tot = O.plane_segment(scene)
    kept = [s for s in surf if s.kept]
    # floor (horizontal) and the two walls (vertical) of the 5 x 5 x 3 m room
    assert sum(s.is_vertical == 0 and s.area > 10 for s in kept) >= 1
    assert sum(s.is_vertical == 1 and s.area > 3 for s in kept) >= 2
    chair = S.synth_shape(S.CHAIR, 20000, 2024)
    surf, _ = O.plane_segment(chair)
    areas = sorted(round(s.area, 2) for s in surf if s.kept)
    # seat faces 0.45 x 0.45 and the backrest with the back legs below it
    assert areas.count(0.2) == 2 and areas.count(0.42) == 2


def test_vector3d_as_written():
    # get_Vector3D: one horizontal area within 5 cm, two vertical within 2 cm
    # sorted descending, 0.16 elsewhere; only kept surfaces count
    def surf(coeffs, area, vert, kept=1):
        s = O.Surface()
        s.coeffs[:] = coeffs
        s.area, s.is_vertical, s.kept = area, vert, kept
        return s
    ss = [surf([0, 0, 1, 0], 2.0, 0), surf([0, 0, 1, -0.5], 3.0, 0), surf([1, 0, 0, -0.01], 0.3, 1),
          surf([0, 1, 0, 0.0], 0.9, 1), surf([0, 1, 0, -0.015], 5.0, 1, kept=0), surf([1, 0, 0, 0.0], 0.7, 1)]
    keys = np.array([[0, 0, 0.04, 0], [0, 0, 0.06, 0], [0.05, 0.05, 0.49, 0], [5, 5, 5, 0]], np.float32)
    v = O.vector3d(keys, ss)
    np.testing.assert_array_equal(v[0], [2.0, 0.9, 0.3])  # the first two vertical within 2 cm, sorted
    np.testing.assert_array_equal(v[1], [0.16, 0.9, 0.3])
    np.testing.assert_array_equal(v[2], [3.0, 0.16, 0.16])
    np.testing.assert_array_equal(v[3], [0.16, 0.16, 0.16])
