"""rtr_harris3d (the keypoint detector of ModelPoint / ScanPoint::
getKeypoint, model_point.h:127-136, scan_point.h:85-94) against the oracle
(oracle/harris.c), bit for bit: the same keypoints (point indices), refined
positions and responses, with suppression and refinement on and off."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _check(ctx, rtr, pts, **kw):
    k, s = ctx.harris3d(_dev(pts), rtr.harris_default_params(**{a: int(b) for a, b in kw.items()}))
    rk, rs = O.harris3d(pts, **kw)
    assert np.array_equal(s.cpu().numpy(), rs)
    assert np.array_equal(k.cpu().numpy(), rk)
    return len(rs)


@pytest.mark.parametrize("flags", [dict(), dict(refine=False), dict(non_max=False, refine=False)])
def test_harris_on_shapes_and_main_clouds(ctx, rtr, flags):
    d = np.load(GOLDEN / "main_clouds.npz")
    clouds = [rtr.synth_shape(rtr.CHAIR, 20000, 2024), rtr.synth_shape(rtr.DESK, 20000, 3),
              rtr.synth_shape(rtr.SOFA, 30000, 4), d["chair1"], d["T0_m8111"]]
    found = [_check(ctx, rtr, c, **flags) for c in clouds]
    assert all(f > 0 for f in found), found


def test_harris_on_the_room(ctx, rtr):
    scene, _, _ = rtr.synth_room(1)
    assert _check(ctx, rtr, scene) > 0
