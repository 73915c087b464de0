"""Repeatability of the SHOT-352 descriptor under the workload's parameters
(1 cm voxels, k=10 normals, 2 cm keypoints, 4 cm support), measured on the
oracle, whose stages the GPU path reproduces bit for bit (SHOT included).
These figures bound what the recognition chain can find on the config-1
room:

- the descriptor is exactly rotation invariant on identical points;
- a second random sample of the same full chair, in the same pose, matches
  its 1-NN model keypoint within 3 cm for only a few percent of keypoints;
  a curved shape does little better at 4 cm and much better at 8 cm, so the
  limit is the support (about 50 voxels for 352 bins), not the box shapes;
- in the room, a chair keypoint's descriptor is farther from the model's
  descriptor at the same position than from its 1-NN model keypoint, and
  the 1-NN matches of chair keypoints are right at chance level."""
import numpy as np
import pytest

import oracle as O
from oracle import pipeline as OP
from oracle import synth as S

CAM = (0.0, -2.5, 1.5)


def _f4(p):
    out = np.zeros((len(p), 4), np.float32)
    out[:, :3] = p
    return out


def _blob(n, seed):
    g = np.random.default_rng(seed)
    u = g.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    th, ph = np.arccos(u[:, 2]), np.arctan2(u[:, 1], u[:, 0])
    r = 0.22 * (1 + 0.25 * np.sin(3 * th) * np.cos(2 * ph) + 0.12 * np.cos(5 * th) + 0.08 * np.sin(4 * ph))
    return _f4(u * r[:, None])


def _features(pts, radius, vp=None):
    v = O.voxel_downsample(pts, 0.01)
    n = O.normals(v, 10, vp or (0.0, 0.0, 0.0))
    if vp is None:
        n = O.orient_outward(v, n)
    k = O.uniform_sample(v, 0.02)
    d, _ = O.shot352(v, n, k, radius)
    return v, n, k, d


def _nn1_within(sd, s_loc, md, m_loc, r=0.03):
    D = (sd * sd).sum(1)[:, None] + (md * md).sum(1)[None, :] - 2 * sd @ md.T
    return float(np.mean(np.linalg.norm(m_loc[D.argmin(1)] - s_loc, axis=1) < r)), D


def test_shot_rotation_invariant_on_identical_points():
    model = S.synth_shape(S.CHAIR, 20000, 2024)
    v, n, k, d0 = _features(model, 0.04)
    T = S.synth_rigid(5, 30.0, 0.3)
    vr = O.transform_f32(T, v)
    nr = n.copy()
    nr[:, :3] = (n[:, :3].astype(np.float64) @ T[:3, :3].T).astype(np.float32)
    d1, _ = O.shot352(vr, nr, k, 0.04)
    same = ((d0 - d1) ** 2).sum(1) < 1e-6
    # the rest are LRF x-axis sign flips on patches symmetric about it
    assert same.mean() >= 0.97, same.mean()


@pytest.mark.parametrize("shape,radius,lo,hi", [("chair", 0.04, 0.0, 0.10), ("blob", 0.04, 0.0, 0.10),
                                                ("blob", 0.08, 0.20, 1.0)])
def test_resampled_shape_repeatability(shape, radius, lo, hi):
    if shape == "chair":
        a, b = S.synth_shape(S.CHAIR, 20000, 2024), S.synth_shape(S.CHAIR, 20000, 77)
    else:
        a, b = _blob(20000, 1), _blob(20000, 2)
    mv, _, mk, md = _features(a, radius)
    sv, _, sk, sd = _features(b, radius)
    frac, _ = _nn1_within(sd, sv[sk][:, :3], md, mv[mk][:, :3])
    assert lo <= frac <= hi, frac


def test_room_chair_descriptors_at_chance():
    scene, shapes, poses = S.synth_room(1)
    chairs = [poses[i] for i in range(len(shapes)) if shapes[i] == 0]
    m = OP.prepare_model(S.synth_shape(S.CHAIR, 20000, 2024), OP.params())
    sv = O.voxel_downsample(scene, 0.01)
    sn = O.normals(sv, 10, CAM)
    keys = O.uniform_sample(sv, 0.02)
    skp = sv[keys][:, :3].astype(np.float64)
    loc = np.full((len(keys), 3), np.nan)
    for P in chairs:
        Pi = np.linalg.inv(P)
        q = skp @ Pi[:3, :3].T + Pi[:3, 3]
        idx, _ = O.nn1(_f4(q), m["vox"], 0.015)
        loc[idx >= 0] = q[idx >= 0]
    on = np.nonzero(~np.isnan(loc[:, 0]))[0]
    assert len(on) > 2000
    sd, _ = O.shot352(sv, sn, keys[on], 0.04)
    mkp = m["kp"][:, :3]
    frac, D = _nn1_within(sd, loc[on], m["desc"], mkp)
    chance = float(np.mean(np.linalg.norm(mkp[None, :, :] - loc[on][:300, None, :], axis=2) < 0.03))
    assert frac <= 2.0 * chance + 0.002, (frac, chance)
    # the model's descriptor at each chair keypoint's true position
    idx, _ = O.nn1(_f4(loc[on]), m["vox"], 0.0)
    ext = np.concatenate([m["vox"], _f4(loc[on])])
    nx = np.concatenate([m["nrm"], m["nrm"][idx]])
    dm, _ = O.shot352(ext, nx, np.arange(len(m["vox"]), len(ext), dtype=np.int32), 0.04)
    same_pos = ((sd - dm) ** 2).sum(1)
    assert np.median(same_pos) > np.median(D.min(1)), (np.median(same_pos), np.median(D.min(1)))
