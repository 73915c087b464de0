"""The oracle's SHOT against a second, independent restatement in float64
numpy written from the descriptor's definition: support within R facing the
keypoint's side; an (R - d)-weighted covariance LRF with x signed by the
majority of offsets and z by the sign of sum w (n . z); 2 radial x 2
elevation x 8 azimuth volumes x 11 cosine bins with quadrilinear
interpolation, clamped at the ends of every axis but the circular azimuth;
the keypoint itself excluded; L2 normalised.  The GPU kernel equals the
oracle bit for bit, so this pins the rules both follow.

The sign rules decide by counts and sums that can sit on a tie.  The voxel
lattice puts many offsets exactly in the plane through the keypoint normal
to an axis, so float32 and float64 may sign an axis differently.  The test
therefore checks the LRF's axes and signs against the rules (up to such
near-zero terms), and the histogram given the oracle's LRF."""
import numpy as np

import oracle as O


def _interp(pos, nb, circular):
    lo = np.floor(pos)
    f = pos - lo
    lo = int(lo)
    if circular:
        b0 = lo % nb
        return [(b0, 1.0 - f), ((b0 + 1) % nb, f)]
    if lo < 0:
        return [(0, 1.0)]
    if lo >= nb - 1:
        return [(nb - 1, 1.0)]
    return [(lo, 1.0 - f), (lo + 1, f)]


def _support(P, N, k, R):
    off = P - P[k]
    d = np.sqrt((off ** 2).sum(1))
    sup = np.nonzero((d <= R) & (N @ N[k] >= -0.2))[0]
    return sup, off[sup], d[sup]


def histogram_numpy(P, N, k, R, x, z):
    sup, o, d = _support(P, N, k, R)
    y = np.cross(z, x)
    H = np.zeros(352)
    for j in range(len(sup)):
        if not d[j] > 0:
            continue
        lx, ly, lz = o[j] @ x, o[j] @ y, o[j] @ z
        cs = min(max(N[sup[j]] @ z, -1.0), 1.0)
        az = np.arctan2(ly, lx)
        el = np.arctan2(lz, np.hypot(lx, ly))
        for rb, rw in _interp(d[j] / R * 2 - 0.5, 2, False):
            for eb, ew in _interp((el + np.pi / 2) * (2 / np.pi) - 0.5, 2, False):
                for ab, aw in _interp((az + np.pi) * (8 / (2 * np.pi)) - 0.5, 8, True):
                    for cb, cw in _interp((cs + 1) * 5.5 - 0.5, 11, False):
                        H[((rb * 2 + eb) * 8 + ab) * 11 + cb] += rw * ew * aw * cw
    s = np.sqrt((H ** 2).sum())
    return H / s if s > 0 else H


def test_oracle_shot_follows_an_independent_float64_restatement():
    rng = np.random.default_rng(11)
    import realtime_robot_gb300 as R
    model = R.synth_shape(R.CHAIR, 8000, 77)
    v = O.voxel_downsample(model, 0.01)
    n = O.orient_outward(v, O.normals(v, 10, (0.0, 0.0, 0.0)))
    keys = O.uniform_sample(v, 0.02)
    keys = np.sort(rng.choice(keys, size=min(300, len(keys)), replace=False)).astype(np.int32)
    Rr = 0.04
    got, lrf = O.shot352(v, n, keys, Rr)
    P, N = v[:, :3].astype(np.float64), n[:, :3].astype(np.float64)
    for r, k in enumerate(keys):
        x, y, z = (lrf[r, 3 * a: 3 * a + 3].astype(np.float64) for a in range(3))
        sup, o, d = _support(P, N, k, Rr)
        w = Rr - d
        ev, V = np.linalg.eigh((o * w[:, None]).T @ o)
        # axes: eigenvectors of the largest (x) and smallest (z) eigenvalue,
        # wherever those are separated from the middle one
        if ev[2] - ev[1] > 1e-3 * ev[2]:
            assert abs(x @ V[:, 2]) > 1 - 1e-4, (r, x @ V[:, 2])
        if ev[1] - ev[0] > 1e-3 * ev[2]:
            assert abs(z @ V[:, 0]) > 1 - 1e-4, (r, z @ V[:, 0])
        assert np.allclose(y, np.cross(z, x), atol=1e-6)
        # signs: the rules hold up to offsets (or terms) within rounding of 0
        px = o @ x
        eps = 1e-6 * Rr
        assert (px > eps).sum() + (np.abs(px) <= eps).sum() >= (px < -eps).sum(), r
        zt = w * (N[sup] @ z)
        assert zt.sum() >= -1e-6 * np.abs(zt).sum(), r
        # the histogram given the oracle's frame: float32 against float64
        ref = histogram_numpy(P, N, k, Rr, x, z)
        assert np.abs(got[r] - ref).max() < 1e-5, (r, np.abs(got[r] - ref).max())
