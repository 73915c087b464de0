"""The oracle's descriptor 1-NN, FP32 rigid transform and hypothesis score
against independent numpy restatements (the GPU kernels equal the oracle bit
for bit, so these pin the rules both follow):

- 1-NN: d^2 = the sequential FP32 sum over the 352 dimensions of
  (q_k - b_k)^2, each operation rounded; the lowest index wins ties;
- transform: each row ((r0 x + r1 y) + r2 z) + t in FP32 from the pose
  rounded to FP32;
- hypothesis score: the fraction of every stride-th model point, moved by the
  pose, with a scene point within r (d^2 <= r^2 in FP32)."""
import numpy as np

import oracle as O

f32 = np.float32


def test_descriptor_match_against_sequential_numpy():
    rng = np.random.default_rng(8)
    db = rng.random((300, 352), dtype=np.float32)
    db /= np.linalg.norm(db, axis=1, keepdims=True)
    db[200] = db[17]  # a duplicated row: ties go to 17
    q = rng.random((60, 352), dtype=np.float32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[3] = db[17]
    q[4] = 0.0
    q[5] = db[250] + f32(1e-7)
    idx, d2 = O.match(q, db)
    diff = q[:, None, :] - db[None, :, :]
    seq = np.cumsum(diff * diff, axis=2, dtype=np.float32)[:, :, -1]  # sequential, in k order
    want = np.argmin(seq, axis=1)  # first (lowest) index on ties
    assert np.array_equal(idx, want)
    assert np.array_equal(d2, seq[np.arange(len(q)), want])
    assert idx[3] == 17 and d2[3] == 0.0 and idx[5] == 250


def _pose(rng):
    import realtime_robot_gb300 as R
    return R.synth_rigid(int(rng.integers(1 << 30)), 40.0, 0.5)


def test_transform_rows_in_order():
    rng = np.random.default_rng(9)
    pts = np.zeros((500, 4), np.float32)
    pts[:, :3] = rng.uniform(-1, 1, (500, 3))
    T = _pose(rng)
    got = O.transform_f32(T, pts)
    Tf = T.astype(np.float32)
    x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
    for a in range(3):
        row = f32(f32(f32(Tf[a, 0] * x + f32(Tf[a, 1] * y)) + f32(Tf[a, 2] * z)) + Tf[a, 3])
        assert np.array_equal(got[:, a], row), a


def test_hypothesis_score_against_brute_force():
    rng = np.random.default_rng(10)
    scene = np.zeros((3000, 4), np.float32)
    scene[:, :3] = rng.uniform(-0.5, 0.5, (3000, 3))
    model = np.zeros((700, 4), np.float32)
    model[:, :3] = rng.uniform(-0.3, 0.3, (700, 3))
    poses = np.stack([_pose(rng) for _ in range(4)] + [np.eye(4)])
    r, stride = 0.02, 4
    g = O.Grid(scene, 0.5 * r)
    got = g.inlier_fraction(model, stride, poses, r)
    g.close()
    sub = model[::stride]
    S = scene[:, :3]
    for h, T in enumerate(poses):
        moved = O.transform_f32(T, sub)[:, :3]
        d = moved[:, None, :] - S[None, :, :]
        d2 = f32(f32(d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
        want = (d2 <= f32(r) * f32(r)).any(axis=1).mean()
        assert got[h] == want, (h, got[h], want)
