"""Host logic of the learned form: the row balancing before training, the
pose comparison behind the 1 cm / 1 degree fallback rule, and the pairs'
sizes (no GPU: balancing runs on CPU tensors, the pairs come from the
library's host generators)."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_balance_repeats_positives_to_the_fraction(rtr):
    from realtime_robot_gb300.learned import balance
    g = torch.Generator().manual_seed(0)
    X = torch.rand((2000, 352), generator=g)
    y = torch.zeros(2000)
    pos = torch.tensor([3, 77, 500, 1999])
    y[pos] = 1.0
    Xb, yb = balance(X, y, 0.1, seed=4)
    n_pos = int((yb > 0.5).sum())
    assert Xb.shape[0] == yb.shape[0] > 2000
    assert 0.1 <= n_pos / yb.numel() < 0.1 + 4.0 / yb.numel()
    # every original row is still there, and the added rows are copies of positives
    rows = {tuple(r.tolist()[:4]) for r in Xb}
    assert all(tuple(r.tolist()[:4]) in rows for r in X)
    assert torch.all(yb[(yb > 0.5)] == 1.0)
    pos_rows = {tuple(X[i].tolist()[:4]) for i in pos.tolist()}
    assert {tuple(r.tolist()[:4]) for r in Xb[yb > 0.5]} == pos_rows
    # deterministic for a seed
    Xc, yc = balance(X, y, 0.1, seed=4)
    assert torch.equal(Xb, Xc) and torch.equal(yb, yc)


def test_balance_leaves_balanced_or_empty_labels_alone(rtr):
    from realtime_robot_gb300.learned import balance
    X = torch.rand((100, 352))
    y = torch.zeros(100)
    assert balance(X, y)[0] is X
    y[:20] = 1.0
    Xb, yb = balance(X, y, 0.1)
    assert Xb is X and yb is y


def test_pose_diff_known_motions(rtr):
    from realtime_robot_gb300.learned import pose_diff
    A = np.eye(4)
    B = np.eye(4)
    a = math.radians(30.0)
    B[:2, :2] = [[math.cos(a), -math.sin(a)], [math.sin(a), math.cos(a)]]
    B[:3, 3] = [0.01, 0.0, 0.0]
    dt, dr = pose_diff(A, B)
    assert abs(dt - 0.01) < 1e-12 and abs(dr - 30.0) < 1e-9
    assert pose_diff(B, B) == (0.0, 0.0)


def test_pairs_draw_both_sizes_log_uniform(rtr):
    from realtime_robot_gb300.learned import SHAPES, make_pair
    sizes = []
    for seed in range(3000, 3016):
        shape, model, seg, T = make_pair(seed, n_model=None)
        assert shape == SHAPES[seed % 3]
        assert 2000 <= model.shape[0] <= 60000
        assert 0.6 * 2000 - 1 <= seg.shape[0] <= 60000
        assert np.allclose(T[:3, :3] @ T[:3, :3].T, np.eye(3), atol=1e-9)
        sizes.append(model.shape[0])
    assert len(set(sizes)) == len(sizes)  # drawn, not fixed
