"""rtr_recognize_learned: with every keypoint kept it must reproduce
rtr_recognize exactly; with keep < 1 it keeps ceil(keep * K) keypoints."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair(rtr):
    import torch
    model = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    T = rtr.synth_rigid(5, 30.0, 0.3)
    seg = rtr.synth_transform_noise(rtr.synth_shape(rtr.CHAIR, 20000, 77), T, 0.002, 9)
    return torch.from_numpy(model).cuda(), torch.from_numpy(seg).cuda(), T


def test_learned_keep_all_equals_plain(ctx, rtr, pair):
    model, seg, _ = pair
    prm = rtr.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    m = rtr.Model(ctx, model, prm)
    mlp = rtr.Mlp(ctx, seed=3)
    plain = rtr.recognize(ctx, m, seg, prm).cpu().numpy().tobytes()
    learned = rtr.recognize_learned(ctx, m, mlp, seg, keep=1.0, params=prm).cpu().numpy().tobytes()
    assert plain == learned


@pytest.mark.parametrize("keep", [0.25, 0.5])
def test_learned_keeps_the_requested_fraction(ctx, rtr, pair, keep):
    model, seg, _ = pair
    prm = rtr.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    m = rtr.Model(ctx, model, prm)
    mlp = rtr.Mlp(ctx, seed=4)
    plain = rtr.parse_recog_result(rtr.recognize(ctx, m, seg, prm))
    res = rtr.parse_recog_result(rtr.recognize_learned(ctx, m, mlp, seg, keep=keep, params=prm))
    assert res["n_keypoints"] == math.ceil(keep * plain["n_keypoints"])
    assert res["n_correspondences"] <= plain["n_correspondences"]


def test_learned_rejects_bad_keep(ctx, rtr, pair):
    model, seg, _ = pair
    prm = rtr.recog_default_params()
    m = rtr.Model(ctx, model, prm)
    mlp = rtr.Mlp(ctx, seed=4)
    for bad in (0.0, 1.5):
        with pytest.raises(rtr.RtrError):
            rtr.recognize_learned(ctx, m, mlp, seg, keep=bad, params=prm)


def test_trained_net_beats_a_random_ranking(ctx, rtr):
    """The credibility MLP trained on plain-pose labels (the library's own
    kernels) against an untrained one (an arbitrary ranking) at the same keep
    fraction, on held-out pairs where the plain pipeline finds the object:
    the trained net's pruning reproduces the plain pose (<= 1 cm / 1 deg) on
    more of them.  Keep 0.5: at 0.25 neither reproduces any (the credible
    keypoints are a few in 10^4 of the training rows)."""
    from realtime_robot_gb300 import learned as L
    prm = rtr.recog_default_params(viewpoint=(0.0, 0.0, 0.0))
    X, y = L.build_dataset(ctx, range(4000, 4160), prm, label_pose="plain")
    assert y.sum().item() > 20
    Xb, yb = L.balance(X, y, 0.1)
    assert abs(yb.mean().item() - 0.1) < 0.02
    mlp, losses = L.train(ctx, Xb, yb, epochs=20)
    assert losses[-1] < losses[0]
    rand = rtr.Mlp(ctx, seed=99)

    def found_agree(net):
        rows = L.evaluate(ctx, net, range(6000, 6060), keep=0.5, p=prm, repeats=1)
        return sum(r["agree"] for r in rows if r["plain_found"]), sum(r["plain_found"] for r in rows)

    t, n_found = found_agree(mlp)
    r, _ = found_agree(rand)
    assert n_found >= 20 and t >= 5 and t > r + 2, (t, r, n_found)
