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
