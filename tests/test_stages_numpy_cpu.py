"""The oracle's voxel filter, PCA normals and uniform sampling against
independent numpy restatements of the published methods (the GPU kernels
equal the oracle bit for bit, so these pin the rules both follow):

- voxel grid: one output point per occupied voxel floor(p / leaf), the
  centroid of its points, in ascending linear voxel key (x fastest);
- normals: the k nearest points (the point included, scipy's exact k-d tree
  in float64), normal = the covariance's smallest eigenvector turned towards
  the viewpoint, curvature = l_min / (l0 + l1 + l2);
- uniform sampling: per voxel of edge r the point nearest the voxel centre,
  ties to the lowest index, in ascending voxel key."""
import numpy as np
import pytest

import oracle as O


def _cloud(seed=3, n=20000):
    import realtime_robot_gb300 as R
    return R.synth_shape(R.CHAIR, n, seed)


def _keys(ijk):
    lo = ijk.min(0)
    d = ijk - lo
    ext = d.max(0) + 1
    return (d[:, 2] * ext[1] + d[:, 1]) * ext[0] + d[:, 0]


def test_voxel_grid_against_numpy():
    pts = _cloud()
    leaf = np.float32(0.01)
    got = O.voxel_downsample(pts, float(leaf))
    ijk = np.floor(pts[:, :3] * (np.float32(1.0) / leaf)).astype(np.int64)
    key = _keys(ijk)
    uk, inv = np.unique(key, return_inverse=True)
    cnt = np.bincount(inv)
    cen = np.stack([np.bincount(inv, pts[:, a].astype(np.float64)) / cnt for a in range(3)], 1)
    assert got.shape[0] == uk.shape[0]
    np.testing.assert_allclose(got[:, :3], cen, atol=2e-7)


def test_normals_against_numpy():
    spatial = pytest.importorskip("scipy.spatial")
    pts = O.voxel_downsample(_cloud(), 0.01)
    k, vp = 10, np.array([0.3, -1.0, 0.8])
    got = O.normals(pts, k, tuple(vp))
    P = pts[:, :3].astype(np.float64)
    _, nb = spatial.cKDTree(P).query(P, k)
    ok = 0
    for i in range(P.shape[0]):
        Q = P[nb[i]] - P[nb[i]].mean(0)
        w, V = np.linalg.eigh(Q.T @ Q / k)
        nrm = V[:, 0] * (1.0 if V[:, 0] @ (vp - P[i]) >= 0 else -1.0)
        curv = w[0] / w.sum() if w.sum() > 0 else 0.0
        # a separated smallest eigenvalue fixes the normal; a sign is only
        # undefined when the viewpoint lies in the tangent plane
        if w[1] - w[0] > 1e-3 * w[2] and abs(nrm @ (vp - P[i])) > 1e-3:
            assert nrm @ got[i, :3] > 1 - 1e-4, (i, nrm, got[i])
            assert abs(curv - got[i, 3]) < 1e-4, (i, curv, got[i, 3])
            ok += 1
    assert ok > 0.8 * P.shape[0]


def test_uniform_sampling_against_numpy():
    pts = O.voxel_downsample(_cloud(), 0.01)
    r = np.float32(0.02)
    got = O.uniform_sample(pts, float(r))
    P = pts[:, :3]
    ijk = np.floor(P / r).astype(np.int64)
    key = _keys(ijk)
    cen = (ijk.astype(np.float32) + np.float32(0.5)) * r
    d = ((P - cen) ** 2).sum(1)
    order = np.lexsort((np.arange(len(P)), d, key))  # by key, then distance, then index
    first = np.ones(len(order), bool)
    first[1:] = key[order][1:] != key[order][:-1]
    want = order[first]
    assert np.array_equal(np.sort(got), np.sort(want))
    assert np.all(np.diff(key[got]) > 0)


def test_outward_orientation_against_numpy():
    """Full-model normals turn to the side with fewer cloud points inside a
    cylinder of radius rc along the normal (axial distance in (gap, len]);
    ties keep the sign.  FP32 elementwise in numpy, as the rule states."""
    f32 = np.float32
    pts = O.voxel_downsample(_cloud(5, 8000), 0.01)
    nrm = O.normals(pts, 10, (0.0, 0.0, 0.0))
    got = O.orient_outward(pts, nrm, 0.01, 0.005, 1.0)
    P = pts[:, :3]
    flips = 0
    for i in range(len(P)):
        d = P - P[i]
        n = nrm[i, :3]
        ax = f32(f32(d[:, 0] * n[0] + d[:, 1] * n[1]) + d[:, 2] * n[2])
        aa = np.abs(ax)
        r2 = f32(f32(f32(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) - ax * ax)
        inside = (aa > f32(0.005)) & (aa <= f32(1.0)) & (r2 <= f32(0.01) * f32(0.01))
        cp, cm = int((inside & (ax > 0)).sum()), int((inside & (ax <= 0)).sum())
        want = -nrm[i] if cp > cm else nrm[i]
        want = want.copy()
        want[3] = nrm[i, 3]
        flips += cp > cm
        assert np.array_equal(got[i], want), i
    assert 0 < flips < len(P)
