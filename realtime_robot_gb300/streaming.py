"""Streaming multi-object reconstruction over depth frames (the streaming
workload): per frame, back-projection, frame-to-frame ICP odometry, batched
recognition of every model class (optionally with learned pruning) and
fusion of the frame into a voxel-hash map.

Every stage is a librtr.so call; this module sequences them and times each
frame end to end (host clock, the frame's work synchronised).
"""
from __future__ import annotations

import time

import numpy as np

from . import FusionMap, parse_recog_result, recog_default_params, recognize_multi

FX, FY, CX, CY = 525.0, 525.0, 319.5, 239.5


def _angle_deg(R: np.ndarray) -> float:
    c = max(-1.0, min(1.0, (float(np.trace(R)) - 1.0) / 2.0))
    return float(np.degrees(np.arccos(c)))


def trajectory_errors(est, true) -> dict:
    """Accuracy of an estimated camera trajectory against the true one (both
    lists of 4x4 camera-to-world poses, frame 0 shared): the absolute
    trajectory error (RMS of the position errors over every frame), the
    final position and rotation drift, and the relative pose error of each
    frame-to-frame motion (translation in mm, rotation in degrees; median and
    95th percentile)."""
    est = [np.asarray(e, np.float64) for e in est]
    true = [np.asarray(t, np.float64) for t in true]
    if not est:
        return {}
    pos = np.array([np.linalg.norm(e[:3, 3] - t[:3, 3]) for e, t in zip(est, true)])
    out = {"ate_rms_m": float(np.sqrt(np.mean(pos ** 2))),
           "drift_final_m": float(pos[-1]),
           "rot_drift_final_deg": _angle_deg(est[-1][:3, :3].T @ true[-1][:3, :3])}
    if len(est) > 1:
        rt, rr = [], []
        for f in range(1, len(est)):
            re = np.linalg.inv(est[f - 1]) @ est[f]
            rg = np.linalg.inv(true[f - 1]) @ true[f]
            d = np.linalg.inv(rg) @ re
            rt.append(1e3 * float(np.linalg.norm(d[:3, 3])))
            rr.append(_angle_deg(d[:3, :3]))
        out.update({"rpe_trans_mm_median": float(np.median(rt)), "rpe_trans_mm_p95": float(np.percentile(rt, 95)),
                    "rpe_rot_deg_median": float(np.median(rr)), "rpe_rot_deg_p95": float(np.percentile(rr, 95))})
    return out


class StreamPipeline:
    """State of one stream: the models, the previous frame's odometry cloud,
    the current pose estimate and the fusion map."""

    def __init__(self, ctx, models, mlp=None, keep: float = 0.25, map_voxel: float = 0.005,
                 map_capacity: int = 1 << 26, odo_voxel: float = 0.02, odo_iterations: int = 30,
                 odo_max_dist: float = 0.02, params=None):
        self.ctx = ctx
        self.models = list(models)
        self.mlp = mlp
        self.keep = keep
        self.params = params or recog_default_params(viewpoint=(0.0, 0.0, 0.0))
        self.map = FusionMap(ctx, capacity=map_capacity, voxel=map_voxel)
        self.map_capacity = 1 << (int(map_capacity) - 1).bit_length()
        self.odo_voxel = odo_voxel
        self.odo_iterations = odo_iterations
        self.odo_max_dist = odo_max_dist
        self.prev = None
        self.pose = None
        self.vel = np.eye(4)
        self.results = None

    def start(self, pose0: np.ndarray):
        self.pose = np.asarray(pose0, np.float64).reshape(4, 4).copy()
        self.prev = None
        self.vel = np.eye(4)

    def frame(self, depth):
        """Process one depth frame [H, W] (device); returns (pose estimate,
        per-model recognition results)."""
        import torch
        ctx = self.ctx
        pts, cnt = ctx.depth_to_points(depth, FX, FY, CX, CY, pose=None)  # camera frame
        n = int(cnt.item())
        cloud = pts[:n]
        # odometry: this frame at odo_voxel against the previous frame at full
        # resolution (two voxelised clouds pull each other toward their grids,
        # which biases every step toward zero motion), from the last step's
        # motion (constant velocity)
        down = ctx.voxel_downsample(cloud, self.odo_voxel).contiguous()
        if self.prev is not None and down.shape[0] >= 3 and self.prev.shape[0] >= 3:
            res, _, _ = ctx.icp(down, self.prev, self.odo_iterations, self.odo_max_dist, init=self.vel)
            T = ctx.parse_icp_result(res)["pose"]  # current camera -> previous camera
            self.vel = T
            self.pose = self.pose @ T
        self.prev = cloud
        # every model class in this frame: the scene's stages once, the
        # models' stages side by side on worker streams
        out = recognize_multi(ctx, self.models, cloud, self.params, mlp=self.mlp, keep=self.keep if self.mlp else 1.0,
                              results=self.results)
        self.results = out
        wpts, wcnt = ctx.depth_to_points(depth, FX, FY, CX, CY, pose=self.pose)
        self.map.integrate(wpts, wcnt)
        torch.cuda.synchronize()
        return self.pose.copy(), out

    def run(self, frames, pose0, true_poses=None):
        """All frames; returns timing and accuracy figures."""
        self.start(pose0)
        lat, drift, est = [], [], []
        t_all = time.perf_counter()
        for f in range(frames.shape[0]):
            t0 = time.perf_counter()
            pose, _ = self.frame(frames[f])
            lat.append((time.perf_counter() - t0) * 1e3)
            est.append(pose)
            if true_poses is not None:
                drift.append(float(np.linalg.norm(pose[:3, 3] - true_poses[f][:3, 3])))
        total = time.perf_counter() - t_all
        res = [parse_recog_result(bytes(r)) for r in self.results.cpu().numpy()]
        nvox = self.map.count()
        lat = np.asarray(lat)
        return {"frames": int(frames.shape[0]), "fps": frames.shape[0] / total,
                "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
                "odometry_drift_m_final": drift[-1] if drift else None,
                "odometry_drift_m_max": max(drift) if drift else None,
                "map_voxels": nvox, "map_load": nvox / self.map_capacity,
                "last_frame_instances": [len(r["instances"]) for r in res],
                "trajectory": trajectory_errors(est, true_poses[: len(est)]) if true_poses is not None else None}

    def close(self):
        self.map.close()
