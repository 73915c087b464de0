"""The headline workload at its full size (300,000-point room, 20,000-point
chair model), stage by stage against the oracle where the oracle finishes in
seconds, and through size-independent properties where it does not:

- voxel filter, normals and keypoints: bit-exact over the whole room;
- SHOT: every scene keypoint's descriptor bit-exact;
- matching: all 115k scene descriptors against the 9.2k-row model
  database, indices and distances bit-exact against the oracle;
- grouping: every cluster is pairwise consistent, clusters are disjoint and
  none is below the threshold; and the whole chain against the oracle
  pipeline: the same correspondences, clusters member for member, counts;
- recognition: deterministic (two runs give the same bytes) and the host
  entry point gives what the device one does."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

CAM = (0.0, -2.5, 1.5)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.fixture(scope="module")
def room(rtr):
    p = rtr.room_default_params()
    scene, _, _ = rtr.synth_room(1, p)
    model = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    assert scene.shape[0] == 300000
    return scene, model


@pytest.fixture(scope="module")
def stages(ctx, room):
    import torch
    scene, _ = room
    v = O.voxel_downsample(scene, 0.01)
    n = O.normals(v, 10, CAM)
    keys = O.uniform_sample(v, 0.02)
    gv = ctx.voxel_downsample(_dev(scene), 0.01).contiguous()
    gn = ctx.normals(gv, 10, CAM, 0.02)
    gk = ctx.uniform_sample(gv, 0.02)
    gd = ctx.shot352(gv, gn, gk.contiguous(), 0.04)
    torch.cuda.synchronize()
    return v, n, keys, gv, gn, gk, gd


def test_room_voxels_normals_keypoints_bit_exact(stages):
    v, n, keys, gv, gn, gk, _ = stages
    assert v.shape[0] > 200000
    assert np.array_equal(gv.cpu().numpy()[:, :3], v[:, :3])
    assert np.array_equal(gn.cpu().numpy(), n)
    assert np.array_equal(gk.cpu().numpy(), keys)


def test_room_shot_full_size(stages):
    v, n, keys, _, _, _, gd = stages
    ref, _ = O.shot352(v, n, keys, 0.04)
    assert ref.shape[0] > 100000
    assert np.array_equal(gd.cpu().numpy(), ref), (np.abs(gd.cpu().numpy() - ref).max(axis=1) > 0).sum()


def test_room_match_full_database(ctx, rtr, room, stages):
    scene, model = room
    _, _, _, _, _, _, gd = stages
    mv = O.voxel_downsample(model, 0.01)
    mn = O.orient_outward(mv, O.normals(mv, 10, (0.0, 0.0, 0.0)))
    md, _ = O.shot352(mv, mn, O.uniform_sample(mv, 0.02), 0.04)
    idx, d2 = ctx.match(gd, _dev(md))
    ri, rd = O.match(gd.cpu().numpy(), md)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)


def test_room_grouping_properties(ctx, rtr, room):
    """rtr_gc_group on the room's own correspondences (110k): each cluster
    satisfies the consistency test pairwise, clusters are disjoint and at
    least the threshold in size."""
    import torch
    from realtime_robot_gb300.learned import _model_features, _scene_features
    scene, model = room
    prm = rtr.recog_default_params(viewpoint=CAM)
    mk, mdesc = _model_features(ctx, _dev(model), prm)
    sk, sdesc = _scene_features(ctx, _dev(scene), prm)
    idx, d2 = ctx.match(sdesc, mdesc)
    keep = (idx >= 0) & (d2 <= prm.match_max_d2)
    cs = torch.nonzero(keep).flatten().int()
    cm = idx[keep].int()
    cd = d2[keep].float()
    assert cs.numel() > 50000
    mem, sizes, poses = ctx.gc_group(mk, sk, cm, cs, cd, 0.01, 5, 256, 128)
    mem, sizes = mem.cpu().numpy(), sizes.cpu().numpy()
    ncl = sizes.shape[0]
    assert 0 < ncl <= 256
    mkh, skh = mk.cpu().numpy(), sk.cpu().numpy()
    cmh, csh = cm.cpu().numpy(), cs.cpu().numpy()
    seen = set()
    for c in range(ncl):
        m = mem[c, : sizes[c]]
        assert sizes[c] >= 5 and len(set(m.tolist())) == sizes[c]
        assert not (seen & set(m.tolist()))
        seen |= set(m.tolist())
        pm = mkh[cmh[m], :3].astype(np.float32)
        ps = skh[csh[m], :3].astype(np.float32)
        dm = np.sqrt(((pm[:, None, :] - pm[None, :, :]) ** 2).sum(-1, dtype=np.float32)).astype(np.float32)
        ds = np.sqrt(((ps[:, None, :] - ps[None, :, :]) ** 2).sum(-1, dtype=np.float32)).astype(np.float32)
        # float32 arithmetic in numpy's order: a 1e-5 slack covers the rounding difference
        assert np.all(np.abs(dm - ds) <= 0.01 + 1e-5)


def test_room_chain_matches_oracle_pipeline(ctx, rtr, room):
    """The whole room against the oracle pipeline (every stage bit-exact up
    to the matcher, SHOT included): the same scene keypoints, the same
    correspondences (model and scene index per pair, strict d^2 < 0.25), the
    same clusters member for member with poses within 1e-7 of the oracle's,
    and the same counts out of rtr_recognize."""
    import torch
    from oracle import pipeline as OP
    from realtime_robot_gb300.learned import _model_features, _scene_features
    scene, model = room
    prm = rtr.recog_default_params(viewpoint=CAM)
    p = OP.params(viewpoint=CAM)
    om = OP.prepare_model(model, p)
    st = {}
    ref = OP.recognize(om, scene, p, stages=st)
    mk, mdesc = _model_features(ctx, _dev(model), prm)
    sk, sdesc = _scene_features(ctx, _dev(scene), prm)
    skr = st["sv"][st["keys"]]
    assert np.array_equal(sk.cpu().numpy()[:, :3], skr[:, :3])
    idx, d2 = ctx.match(sdesc, mdesc)
    keep = (idx >= 0) & (d2 < prm.match_max_d2)
    cs = torch.nonzero(keep).flatten().int()
    cm = idx[keep].int()
    cd = d2[keep].float()
    assert np.array_equal(cs.cpu().numpy(), st["corr_s"]) and np.array_equal(cm.cpu().numpy(), st["corr_m"])
    mem, sizes, poses = ctx.gc_group(mk, sk, cm, cs, cd, prm.gc_size, prm.gc_thresh, prm.max_clusters, 512)
    mem, sizes, poses = mem.cpu().numpy(), sizes.cpu().numpy(), poses.cpu().numpy()
    assert np.array_equal(cd.cpu().numpy(), st["d2"][st["corr_s"]])
    _, rposes, rsizes = O.gc_group(om["kp"], skr, st["corr_m"], st["corr_s"], st["d2"][st["corr_s"]], p["gc_size"],
                                   p["gc_thresh"], p["max_clusters"])
    assert np.array_equal(sizes, rsizes) and len(sizes) == ref["n_clusters"]
    for c in range(len(sizes)):
        assert set(mem[c][: sizes[c]].tolist()) == set(np.nonzero(st["cluster_of"] == c)[0].tolist()), c
        dt, dr = O.pose_error(poses[c], rposes[c])
        assert dt < 1e-7 and dr < 1e-7, (c, dt, dr)
    m = rtr.Model(ctx, _dev(model), prm)
    r = rtr.parse_recog_result(rtr.recognize(ctx, m, _dev(scene), prm))
    for k in ("n_voxels", "n_keypoints", "n_correspondences", "n_clusters"):
        assert r[k] == ref[k], (k, r[k], ref[k])
    assert len(r["instances"]) == len(ref["instances"])
    for a, b in zip(r["instances"], ref["instances"]):
        dt, dr = O.pose_error(a["pose"], b["pose"])
        assert dt < 1e-5 and dr < 1e-5, (dt, dr)
    m.close()


def test_room_recognition_deterministic_and_host_entry(ctx, rtr, room):
    scene, model = room
    prm = rtr.recog_default_params(viewpoint=CAM)
    m = rtr.Model(ctx, _dev(model), prm)
    s = _dev(scene)
    a = rtr.recognize(ctx, m, s, prm).cpu().numpy().tobytes()
    b = rtr.recognize(ctx, m, s, prm).cpu().numpy().tobytes()
    assert a == b
    ra, rh = rtr.parse_recog_result(a), rtr.recognize_host(ctx, m, scene, prm)
    for k in ("n_voxels", "n_keypoints", "n_correspondences", "n_clusters", "status"):
        assert ra[k] == rh[k]
    assert ra["n_voxels"] > 200000 and ra["n_keypoints"] > 100000
    assert len(ra["instances"]) == len(rh["instances"])
    for x, y in zip(ra["instances"], rh["instances"]):
        assert np.array_equal(x["pose"], y["pose"])
    m.close()
