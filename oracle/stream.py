"""CPU restatement of the streaming stages (test infrastructure: the checker
of rtr_depth_to_points, rtr_map_* and rtr_synth_depth_frames, never the
product).  No counterpart in the reference: its sensor path (OpenNI) is not
part of the registration chain; the formulas are the pinhole model and a
voxel average."""
from __future__ import annotations

import numpy as np

F32 = np.float32


def backproject(depth: np.ndarray, fx, fy, cx, cy, pose=None, min_z=0.05, max_z=8.0) -> np.ndarray:
    """World points [k, 4] of the pixels with min_z < z < max_z, row by row;
    FP32, each operation rounded in the order the GPU uses."""
    H, W = depth.shape
    z = depth.astype(F32).ravel()
    keep = (z > F32(min_z)) & (z < F32(max_z))
    idx = np.nonzero(keep)[0]
    u = (idx % W).astype(F32)
    v = (idx // W).astype(F32)
    zz = z[idx]
    x = ((u - F32(cx)) * zz) / F32(fx)
    y = ((v - F32(cy)) * zz) / F32(fy)
    T = np.eye(4) if pose is None else np.asarray(pose, np.float64).reshape(4, 4)
    R = T[:3, :3].astype(F32)
    t = T[:3, 3].astype(F32)
    out = np.zeros((len(idx), 4), F32)
    for r in range(3):
        out[:, r] = ((R[r, 0] * x + R[r, 1] * y) + R[r, 2] * zz) + t[r]
    return out


def fuse(points: np.ndarray, voxel: float) -> dict:
    """{voxel key (ix, iy, iz): (mean x, mean y, mean z, count)} with the
    map's fixed-point sums (2^-40 m) of the offsets from the voxel corner."""
    p = np.ascontiguousarray(points[:, :3], F32)
    inv = F32(1.0 / F32(voxel))
    k = np.floor(p * inv).astype(np.int64)
    ok = np.all(np.abs(k) < 1048000, axis=1)
    p, k = p[ok], k[ok]
    off = p.astype(np.float64) - k.astype(np.float64) * float(F32(voxel))
    off = np.clip(off, 0.0, 2.0 * float(F32(voxel)))
    fix = np.rint(off * 1099511627776.0).astype(np.int64)
    keys, inv_idx = np.unique(k, axis=0, return_inverse=True)
    inv_idx = inv_idx.ravel()
    cnt = np.bincount(inv_idx, minlength=len(keys))
    out = {}
    sums = np.zeros((len(keys), 3), np.int64)
    for a in range(3):
        np.add.at(sums[:, a], inv_idx, fix[:, a])
    for j, key in enumerate(map(tuple, keys)):
        c = float(cnt[j])
        mean = [float(F32(key[a] * float(F32(voxel)) + float(sums[j, a]) / 1099511627776.0 / c)) for a in range(3)]
        out[key] = (mean[0], mean[1], mean[2], int(cnt[j]))
    return out


def raycast_depth(boxes12: np.ndarray, pose: np.ndarray, W, H, fx, fy, cx, cy, max_depth=8.0) -> np.ndarray:
    """Noise-free depth of one frame (FP64): floor z = 0, walls x = -2.5 and
    y = 2.5 (room +-2.5 m, 3 m high), boxes in their object frames."""
    T = np.asarray(pose, np.float64).reshape(4, 4)
    u, v = np.meshgrid(np.arange(W, dtype=np.float64), np.arange(H, dtype=np.float64))
    a = (u - cx) / fx
    b = (v - cy) / fy
    d = np.stack([T[k, 0] * a + T[k, 1] * b + T[k, 2] for k in range(3)], -1)
    o = T[:3, 3]
    best = np.full((H, W), np.inf)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = -o[2] / d[..., 2]
        x, y = o[0] + t * d[..., 0], o[1] + t * d[..., 1]
        m = (d[..., 2] < -1e-9) & (np.abs(x) <= 2.5) & (np.abs(y) <= 2.5) & (t > 0)
        best = np.where(m, np.minimum(best, t), best)
        t = (2.5 - o[1]) / d[..., 1]
        x, z = o[0] + t * d[..., 0], o[2] + t * d[..., 2]
        m = (d[..., 1] > 1e-9) & (np.abs(x) <= 2.5) & (z >= 0) & (z <= 3) & (t > 0)
        best = np.where(m, np.minimum(best, t), best)
        t = (-2.5 - o[0]) / d[..., 0]
        y, z = o[1] + t * d[..., 1], o[2] + t * d[..., 2]
        m = (d[..., 0] < -1e-9) & (np.abs(y) <= 2.5) & (z >= 0) & (z <= 3) & (t > 0)
        best = np.where(m, np.minimum(best, t), best)
        for B in np.asarray(boxes12, np.float64).reshape(-1, 12):
            c, s, bx, by = B[:4]
            lo, hi = B[4:7], B[7:10]
            ow = np.array([o[0] - bx, o[1] - by, o[2]])
            oo = np.array([c * ow[0] + s * ow[1], -s * ow[0] + c * ow[1], ow[2]])
            dd = np.stack([c * d[..., 0] + s * d[..., 1], -s * d[..., 0] + c * d[..., 1], d[..., 2]], -1)
            t0 = np.full((H, W), -np.inf)
            t1 = np.full((H, W), np.inf)
            ok = np.ones((H, W), bool)
            for k in range(3):
                small = np.abs(dd[..., k]) < 1e-12
                ok &= ~(small & ((oo[k] < lo[k]) | (oo[k] > hi[k])))
                ta = (lo[k] - oo[k]) / dd[..., k]
                tb = (hi[k] - oo[k]) / dd[..., k]
                t0 = np.where(small, t0, np.maximum(t0, np.minimum(ta, tb)))
                t1 = np.where(small, t1, np.minimum(t1, np.maximum(ta, tb)))
            hit = ok & (t0 <= t1) & (t1 >= 1e-6) & (t0 > 1e-6)
            best = np.where(hit & (t0 < best), t0, best)
    return np.where(best < max_depth, best, 0.0)
