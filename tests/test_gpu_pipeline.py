"""End-to-end: rtr_recognize on the GPU vs the oracle pipeline.

Voxel, keypoint and correspondence counts must match exactly (every stage
up to the matcher is bit-exact); the best instance within 1 cm / 1 degree of
the oracle's and of the ground truth."""
import numpy as np
import pytest

import oracle as O
from oracle import pipeline as OP

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _pair(R, seed):
    model = R.synth_shape(R.CHAIR, 20000, 2024)
    T = R.synth_rigid(100 + seed, 30.0, 0.3)
    seg = R.synth_transform_noise(R.synth_crop(R.synth_shape(R.CHAIR, 20000, 500 + seed), 0.4, seed), T,
                                  0.002, 9 + seed)
    return model, seg, T


@pytest.mark.parametrize("seed", [1, 4])
def test_recognize_pair_matches_oracle(ctx, rtr, seed):
    model, seg, T = _pair(rtr, seed)
    prm = rtr.recog_default_params(scene_outward=1)
    m = rtr.Model(ctx, _dev(model), prm)
    om = OP.prepare_model(model, OP.params(scene_outward=1))
    assert m.n_voxels == len(om["vox"]) and m.n_keypoints == len(om["keys"])
    res = rtr.parse_recog_result(rtr.recognize(ctx, m, _dev(seg), prm))
    ref = OP.recognize(om, seg, OP.params(scene_outward=1))
    assert res["n_voxels"] == ref["n_voxels"]
    assert res["n_keypoints"] == ref["n_keypoints"]
    assert res["n_correspondences"] == ref["n_correspondences"]
    assert res["n_clusters"] == ref["n_clusters"]
    assert res["instances"], res
    g = res["instances"][0]["pose"]
    dt, dr = O.pose_error(g, ref["instances"][0]["pose"])
    assert dt < 0.01 and dr < np.radians(1.0), (dt, dr)
    dt, dr = O.pose_error(g, T)
    assert dt < 0.01 and dr < np.radians(1.0), (dt, dr)
    m.close()


def test_recognize_host_entry_and_empty_scene(ctx, rtr):
    import torch
    model, seg, T = _pair(rtr, 1)
    prm = rtr.recog_default_params(scene_outward=1)
    m = rtr.Model(ctx, _dev(model), prm)
    r = rtr.recognize_host(ctx, m, seg, prm)
    assert r["instances"] and O.pose_error(r["instances"][0]["pose"], T)[0] < 0.01
    e = torch.zeros((0, 4), dtype=torch.float32, device="cuda")
    r = rtr.parse_recog_result(rtr.recognize(ctx, m, e, prm))
    assert len(r["instances"]) == 0
    # a scene with nothing like the model: no instance, finite outputs
    far = np.zeros((5000, 4), np.float32)
    far[:, :3] = np.random.default_rng(0).uniform(-1, 1, (5000, 3))
    r = rtr.parse_recog_result(rtr.recognize(ctx, m, _dev(far), prm))
    for inst in r["instances"]:
        assert np.all(np.isfinite(inst["pose"]))
    m.close()


def test_recognize_main_clouds_matches_oracle(ctx, rtr):
    """The recognition chain on main's own inputs (chair1.pcd as the model,
    T0_m8111.pcd as the segment; tests/golden/main_clouds.npz): voxels,
    keypoints and correspondences exact, the same instance as the oracle
    pipeline within 1 cm / 1 degree."""
    from pathlib import Path
    d = np.load(Path(__file__).resolve().parent / "golden" / "main_clouds.npz")
    model, scan = d["chair1"], d["T0_m8111"]
    prm = rtr.recog_default_params(scene_outward=1)
    m = rtr.Model(ctx, _dev(model), prm)
    om = OP.prepare_model(model, OP.params(scene_outward=1))
    assert m.n_voxels == len(om["vox"]) and m.n_keypoints == len(om["keys"])
    res = rtr.parse_recog_result(rtr.recognize(ctx, m, _dev(scan), prm))
    ref = OP.recognize(om, scan, OP.params(scene_outward=1))
    assert res["n_voxels"] == ref["n_voxels"] and res["n_keypoints"] == ref["n_keypoints"]
    assert res["n_correspondences"] == ref["n_correspondences"]
    assert len(res["instances"]) == len(ref["instances"]) == 1, (res["instances"], ref["instances"])
    dt, dr = O.pose_error(res["instances"][0]["pose"], ref["instances"][0]["pose"])
    assert dt < 0.01 and dr < np.radians(1.0), (dt, dr)
    m.close()


@pytest.mark.parametrize("pair", [("p70761", "p70761_c", "t70761"), ("p5", "mcloud", "t5")])
@pytest.mark.parametrize("outward", [0, 1])
def test_recognize_recorded_known_answer_pairs(ctx, rtr, pair, outward):
    """Pinned end to end: the reference's recorded pairs (70761.pcd ->
    70761_c.pcd, a translation by (+1, +0.5, 0); 5.pcd -> mcloud.pcd, by
    (+0.8, +0.8, 0); tests/golden/pcd_pairs.npz) recognised with the first
    cloud as the model and the second as the scene: the best instance is the
    recorded translation within 0.1 mm / 0.01 degree, as the oracle's is."""
    from pathlib import Path
    d = np.load(Path(__file__).resolve().parent / "golden" / "pcd_pairs.npz")
    model, scene = d[pair[0]], d[pair[1]]
    T = np.eye(4)
    T[:3, 3] = d[pair[2]]
    prm = rtr.recog_default_params(scene_outward=outward)
    m = rtr.Model(ctx, _dev(model), prm)
    res = rtr.parse_recog_result(rtr.recognize(ctx, m, _dev(scene), prm))
    m.close()
    assert res["instances"], res
    dt, dr = O.pose_error(res["instances"][0]["pose"], T)
    assert dt < 1e-4 and dr < np.radians(0.01), (dt, dr)
    ref = OP.recognize(OP.prepare_model(model, OP.params(scene_outward=outward)), scene,
                       OP.params(scene_outward=outward))
    dt, dr = O.pose_error(ref["instances"][0]["pose"], T)
    assert dt < 1e-4 and dr < np.radians(0.01), (dt, dr)
