"""Trajectory figures of the streaming workload (host arithmetic only)."""
import numpy as np

from realtime_robot_gb300.streaming import trajectory_errors


def _yaw(deg, t=(0.0, 0.0, 0.0)):
    a = np.radians(deg)
    T = np.eye(4)
    T[:2, :2] = [[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]]
    T[:3, 3] = t
    return T


def test_trajectory_errors_exact_and_known_offsets():
    step = _yaw(1.0, (0.01, 0.0, 0.0))
    true = [np.eye(4)]
    for _ in range(9):
        true.append(true[-1] @ step)
    e = trajectory_errors(true, true)
    assert e["ate_rms_m"] == 0.0 and e["rot_drift_final_deg"] < 1e-6 and e["rpe_trans_mm_p95"] < 1e-9
    # every estimated step 0.1 degree short in yaw: the relative error is
    # 0.1 degree per frame and the rotation drift grows to 0.9 degree
    short = _yaw(0.9, (0.01, 0.0, 0.0))
    est = [np.eye(4)]
    for _ in range(9):
        est.append(est[-1] @ short)
    e = trajectory_errors(est, true)
    assert abs(e["rpe_rot_deg_median"] - 0.1) < 1e-9 and abs(e["rot_drift_final_deg"] - 0.9) < 1e-9
    assert e["rpe_trans_mm_median"] < 1e-9
    # a constant 2 cm position offset after frame 0: RMS over 10 frames
    est = [t.copy() for t in true]
    for t in est[1:]:
        t[2, 3] += 0.02
    e = trajectory_errors(est, true)
    assert abs(e["ate_rms_m"] - 0.02 * np.sqrt(0.9)) < 1e-12 and abs(e["drift_final_m"] - 0.02) < 1e-12
