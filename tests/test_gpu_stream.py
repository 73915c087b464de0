"""Streaming stages against the CPU restatement (oracle/stream.py):
back-projection bit-exact, fusion-map voxels (count exact, mean bit-exact:
fixed-point sums), ray-cast depth within 1e-4 m of the FP64 ray caster."""
import numpy as np
import pytest

import oracle.stream as OS

pytestmark = pytest.mark.gpu

CAM = dict(fx=525.0, fy=525.0, cx=319.5, cy=239.5)


@pytest.fixture(scope="module")
def room(rtr):
    p = rtr.room_default_params()
    p.n_chairs, p.n_desks, p.n_sofas = 6, 2, 1
    boxes, shapes, poses = rtr.synth_room_boxes(7, p)
    traj = rtr.synth_trajectory(7, 12)
    return boxes, shapes, poses, traj


def test_raycast_matches_fp64(ctx, rtr, room):
    boxes, _, _, traj = room
    d = ctx.synth_depth_frames(boxes, traj[[0, 11]], noise_k=0.0, seed=1).cpu().numpy()
    for k, f in enumerate((0, 11)):
        ref = OS.raycast_depth(boxes, traj[f], 640, 480, **CAM)
        both = (d[k] > 0) & (ref > 0)
        assert both.mean() > 0.9
        # pixels on an edge may hit different faces; the rest agree tightly
        err = np.abs(d[k][both] - ref[both])
        assert np.mean(err < 1e-4) > 0.999, np.percentile(err, [50, 99.9])
        assert np.mean((d[k] > 0) != (ref > 0)) < 1e-3


def test_backprojection_bit_exact(ctx, rtr, room):
    import torch
    boxes, _, _, traj = room
    depth = ctx.synth_depth_frames(boxes, traj[[3]], seed=2)[0]
    pts, cnt = ctx.depth_to_points(depth, pose=traj[3], **CAM)
    n = int(cnt.item())
    ref = OS.backproject(depth.cpu().numpy(), pose=traj[3], **CAM)
    assert n == len(ref)
    assert np.array_equal(pts[:n].cpu().numpy(), ref)
    torch.cuda.synchronize()


def test_fusion_map_matches_oracle(ctx, rtr, room):
    import torch
    boxes, _, _, traj = room
    depth = ctx.synth_depth_frames(boxes, traj[[0, 5, 10]], seed=3)
    fmap = rtr.FusionMap(ctx, capacity=1 << 22, voxel=0.005)
    allp = []
    for f in range(3):
        pts, cnt = ctx.depth_to_points(depth[f], pose=traj[[0, 5, 10][f]], **CAM)
        fmap.integrate(pts, cnt)
        allp.append(pts[: int(cnt.item())].cpu().numpy())
    got = fmap.extract().cpu().numpy()
    ref = OS.fuse(np.concatenate(allp), 0.005)
    assert len(got) == len(ref)
    counts = got[:, 3].view(np.int32)
    assert counts.sum() == sum(v[3] for v in ref.values())
    # the same (mean, count) records, bit for bit
    g = np.column_stack([got[:, :3].astype(np.float64), counts.astype(np.float64)])
    r = np.array([[np.float32(m[0]), np.float32(m[1]), np.float32(m[2]), m[3]] for m in ref.values()], np.float64)
    g = g[np.lexsort(g.T[::-1])]
    r = r[np.lexsort(r.T[::-1])]
    assert np.array_equal(g, r)
    # integrating again doubles every count and keeps every mean
    for f in range(3):
        fmap.integrate(torch.from_numpy(allp[f]).cuda())
    got2 = fmap.extract().cpu().numpy()
    assert len(got2) == len(got)
    assert got2[:, 3].view(np.int32).sum() == 2 * counts.sum()
    fmap.close()


def test_fusion_map_overflow_is_reported(ctx, rtr, room):
    """A table far too small: every insert stops after a bounded probe run,
    the call stays fast and extract reports the overflow."""
    import time
    import torch
    boxes, _, _, traj = room
    depth = ctx.synth_depth_frames(boxes, traj[[0]], seed=4)[0]
    pts, cnt = ctx.depth_to_points(depth, pose=traj[0], **CAM)
    fmap = rtr.FusionMap(ctx, capacity=1 << 12, voxel=0.005)
    t0 = time.perf_counter()
    fmap.integrate(pts, cnt)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(rtr.RtrError) as e:
        fmap.extract()
    assert e.value.status == 6  # RTR_ERR_CAPACITY
    fmap.clear()
    assert fmap.count() == 0
    fmap.close()


def test_stream_pipeline_tracks_the_camera(ctx, rtr, room):
    import torch
    from realtime_robot_gb300 import streaming as S
    boxes, _, _, _ = room
    traj = rtr.synth_trajectory(7, 30)
    frames = ctx.synth_depth_frames(boxes, traj, seed=5)
    prm = rtr.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    models = [rtr.Model(ctx, torch.from_numpy(rtr.synth_shape(sh, 20000, 1000 + sh)).cuda(), prm)
              for sh in (rtr.CHAIR, rtr.DESK)]
    pipe = S.StreamPipeline(ctx, models, mlp=None, params=prm, map_capacity=1 << 24)
    out = pipe.run(frames, traj[0], traj)
    assert out["frames"] == 30 and out["fps"] > 0
    # frame-to-frame ICP over 1 s (0.5 m) of motion with depth noise 1.5 mm * z^2
    assert out["odometry_drift_m_max"] < 0.08, out
    tr = out["trajectory"]
    assert tr["ate_rms_m"] <= out["odometry_drift_m_max"] + 1e-12 and tr["drift_final_m"] == out["odometry_drift_m_final"]
    assert 0.0 <= tr["rpe_trans_mm_median"] <= tr["rpe_trans_mm_p95"] < 20.0 and tr["rpe_rot_deg_p95"] < 2.0, tr
    assert out["map_voxels"] > 100000 and out["map_load"] < 0.5
    pipe.close()
