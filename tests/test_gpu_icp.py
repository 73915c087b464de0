"""GPU parity of the persistent ICP kernel.

Per iteration the FP64 oracle is replayed on the GPU's own pose: the
correspondences must be bit-exact and the oracle's FP64 pose update (on those
same correspondences) must agree with the GPU's to <= 1e-5 m and <= 1e-5 rad."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL_T = 1e-5  # metres
TOL_R = 1e-5  # radians


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _replay_check(ctx, src, tgt, iters, max_dist, init=None):
    res, tp, tc = ctx.icp(_dev(src), _dev(tgt), iters, max_dist, init=init, trace=True)
    r = ctx.parse_icp_result(res)
    assert r["status"] == 0
    n_it = r["iterations"]
    poses = tp.cpu().numpy()[: n_it + 1]
    corr = tc.cpu().numpy()[:n_it]
    ocorr, opose, ncorr = O.icp_replay(src, tgt, max_dist, poses)
    worst_t = worst_r = 0.0
    for k in range(n_it):
        assert np.array_equal(corr[k], ocorr[k]), f"iteration {k}: correspondences differ"
        if ncorr[k] >= 3:
            dt, dr = O.pose_error(poses[k + 1].reshape(4, 4), opose[k + 1])
            worst_t, worst_r = max(worst_t, dt), max(worst_r, dr)
    assert worst_t <= TOL_T and worst_r <= TOL_R, (worst_t, worst_r)
    return r


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_icp_config0_per_iteration_parity(ctx, rtr, seed):
    src, tgt, T = rtr.config0_pair(seed)
    r = _replay_check(ctx, src, tgt, 50, 0.05)
    assert r["iterations"] == 50 and r["converged"] == 1
    dt, dr = O.pose_error(r["pose"], T)
    assert dt < 2e-3 and dr < np.deg2rad(0.5)


def test_icp_matches_full_oracle_run(ctx, rtr):
    src, tgt, _ = rtr.config0_pair(4, 8000)
    res, _, _ = ctx.icp(_dev(src), _dev(tgt), 30, 0.05)
    g = ctx.parse_icp_result(res)
    o = O.icp(src, tgt, 30, 0.05)
    dt, dr = O.pose_error(g["pose"], o["pose"])
    assert dt < 1e-4 and dr < 1e-4
    assert abs(g["n_corr"] - o["n_corr"]) <= 2


def test_icp_known_answer_pairs(ctx, golden):
    E = np.eye(4)
    E[:3, 3] = golden["t5"]
    r = _replay_check(ctx, golden["p5"], golden["mcloud"], 50, 0.0)
    dt, dr = O.pose_error(r["pose"], E)
    assert dt < 1e-5 and dr < 1e-5
    a, b = golden["p70761"], golden["p70761_c"]
    init = np.eye(4)
    init[:3, 3] = b[:, :3].astype(np.float64).mean(0) - a[:, :3].astype(np.float64).mean(0) + 0.01
    E[:3, 3] = golden["t70761"]
    r = _replay_check(ctx, a, b, 30, 0.0, init=init)
    dt, dr = O.pose_error(r["pose"], E)
    assert dt < 1e-5 and dr < 1e-5


def test_icp_host_entry_point(ctx, rtr):
    src, tgt, T = rtr.config0_pair(6, 5000)
    r = ctx.icp_host(src, tgt, 40, 0.05)
    assert r["status"] == 0 and r["iterations"] == 40
    dt, dr = O.pose_error(r["pose"], T)
    assert dt < 3e-3 and dr < np.deg2rad(0.5)


def test_icp_too_few_correspondences_keeps_pose(ctx, rtr):
    src, _, _ = rtr.config0_pair(7, 2000)
    far = src.copy()
    far[:, 0] += 10.0  # 10 m away: nothing within 5 cm
    res, _, _ = ctx.icp(_dev(src), _dev(far), 20, 0.05)
    r = ctx.parse_icp_result(res)
    assert r["converged"] == 0 and r["iterations"] == 1 and r["n_corr"] == 0
    assert np.array_equal(r["pose"], np.eye(4))
    assert np.all(np.isfinite(r["pose"]))


def test_icp_early_stop_criteria(ctx, rtr):
    src, tgt, _ = rtr.config0_pair(8, 5000)
    # stop once an update moves the source by less than 1e-6 m (|dt|^2 < 1e-12)
    res, _, _ = ctx.icp(_dev(src), _dev(tgt), 200, 0.05, transformation_epsilon=1e-12)
    r = ctx.parse_icp_result(res)
    assert 1 <= r["iterations"] < 200
    o = O.icp(src, tgt, 200, 0.05, eps_t=1e-12)
    assert abs(o["iterations"] - r["iterations"]) <= 2
    dt, dr = O.pose_error(r["pose"], o["pose"])
    assert dt < 1e-4 and dr < 1e-4


@pytest.mark.parametrize("seed", [0, 3])
def test_icp_near_cell_search_same_correspondences(ctx, rtr, seed):
    """With a grid cell wider than the correspondence distance, every match
    lies in the 27 cells around a query and the kernel takes the shorter
    search (no rings).  Its correspondences are those of the ring search and
    of the oracle, iteration by iteration."""
    src, tgt, _ = rtr.config0_pair(seed)
    for d in (0.02, 0.05):
        ring, tp_r, tc_r = ctx.icp(_dev(src), _dev(tgt), 20, d, trace=True)
        near, tp_n, tc_n = ctx.icp(_dev(src), _dev(tgt), 20, d, cell_size=1.5 * d, trace=True)
        assert np.array_equal(tc_r.cpu().numpy(), tc_n.cpu().numpy())
        # the source is sorted by target cell, so another cell size changes the
        # order of the compensated sums: poses agree to rounding
        np.testing.assert_allclose(tp_r.cpu().numpy(), tp_n.cpu().numpy(), rtol=0, atol=1e-9)
        r = ctx.parse_icp_result(near)
        poses = tp_n.cpu().numpy()[: r["iterations"] + 1]
        ocorr, _, _ = O.icp_replay(src, tgt, d, poses)
        corr = tc_n.cpu().numpy()[: r["iterations"]]
        for k in range(r["iterations"]):
            assert np.array_equal(corr[k], ocorr[k]), k


def test_icp_multi_equals_oracle_refinement(ctx, rtr):
    """rtr_icp_multi: independent problems from several initial poses over one
    target grid, against the oracle's multi-problem ICP (the recognition's
    refinement) and against one-problem runs of the same kernel."""
    src, tgt, T = rtr.config0_pair(5, 6000)
    inits = []
    for k in range(6):
        E = np.eye(4)
        E[:3, 3] = T[:3, 3] + np.float64(0.01) * np.array([k % 3 - 1, (k // 3) - 0.5, 0.2 * k])
        E[:3, :3] = T[:3, :3]
        inits.append(E)
    inits = np.array(inits)
    got = ctx.icp_multi(_dev(src), _dev(tgt), inits, 30, 0.02, cell_size=0.03)
    g = O.Grid(tgt, 0.03)
    ref = g.icp_multi(src, 30, 0.02, inits)
    g.close()
    for a, b in zip(got, ref):
        assert a["status"] == 0 and a["iterations"] == 30
        dt, dr = O.pose_error(a["pose"], b["pose"])
        assert dt < 1e-5 and dr < 1e-5, (dt, dr)
        assert abs(a["n_corr"] - b["n_corr"]) <= 2


def test_pose_inliers_equals_oracle(ctx, rtr):
    """rtr_pose_inliers: per pose, the model points within r of a scene point,
    as the oracle's grid counts them."""
    src, tgt, T = rtr.config0_pair(6, 5000)
    poses = np.array([T, np.eye(4), T @ np.diag([1.0, 1.0, 1.0, 1.0])])
    poses[2][:3, 3] += 0.015
    import torch
    for r in (0.005, 0.02):
        cnt = ctx.pose_inliers(_dev(src), _dev(tgt), torch.from_numpy(poses), r).cpu().numpy()
        g = O.Grid(tgt, 1.5 * r)
        frac = g.inlier_fraction(src, 1, poses.reshape(-1, 16), r)
        g.close()
        assert np.array_equal(cnt, np.rint(frac * src.shape[0]).astype(np.int32)), (cnt, frac)
