"""CPU restatement of rtr_recognize (test infrastructure / CPU baseline).

Same stage order and rules as the GPU pipeline: voxel filter -> normals ->
uniform keypoints (optional curvature gate) -> SHOT-352 -> exact 1-NN
matching -> geometric-consistency grouping -> hypothesis score (fraction of
every hv_subsample-th model voxel with a scene point within hv_inlier_r) ->
ICP refinement of the best refine_top -> final score (all model voxels within
accept_inlier_r) -> non-maximum suppression.  The reference's own consensus
loop this stands for is Ransac (function.h:35-109).
"""
from __future__ import annotations

import numpy as np

from . import (Grid, gc_group, match, normals, orient_outward, shot352, uniform_sample,
               voxel_downsample)

DEFAULTS = dict(voxel_leaf=0.01, normal_k=10, scene_keypoint_r=0.02, model_keypoint_r=0.02,
                descriptor_r=0.04, match_max_d2=0.25, gc_size=0.01, gc_thresh=5, max_clusters=256,
                hv_inlier_r=0.02, hv_subsample=4, refine_top=16, icp_iterations=30,
                icp_max_dist=0.02, accept_inlier_r=0.01, accept_score=0.2, nms_dist=0.1,
                max_instances=8, viewpoint=(0.0, 0.0, 0.0), keypoint_min_curvature=0.0,
                scene_outward=0)


def params(**kw) -> dict:
    p = dict(DEFAULTS)
    p.update(kw)
    return p


def prepare_model(pts, p: dict) -> dict:
    v = voxel_downsample(pts, p["voxel_leaf"])
    n = orient_outward(v, normals(v, p["normal_k"], (0.0, 0.0, 0.0)))
    k = uniform_sample(v, p["model_keypoint_r"])
    d, _ = shot352(v, n, k, p["descriptor_r"])
    return {"vox": v, "nrm": n, "keys": k, "kp": v[k], "desc": d}


def recognize(model: dict, scene, p: dict, stages: dict | None = None, timing: dict | None = None) -> dict:
    """timing (optional): filled with seconds per stage."""
    import time
    clock = [time.perf_counter()]

    def lap(name):
        if timing is not None:
            now = time.perf_counter()
            timing[name] = timing.get(name, 0.0) + now - clock[0]
            clock[0] = now

    sv = voxel_downsample(scene, p["voxel_leaf"])
    lap("voxel")
    sn = normals(sv, p["normal_k"], p["viewpoint"])
    if p["scene_outward"]:
        sn = orient_outward(sv, sn)
    lap("normals")
    keys = uniform_sample(sv, p["scene_keypoint_r"])
    if p["keypoint_min_curvature"] > 0:
        keys = keys[sn[keys, 3] >= np.float32(p["keypoint_min_curvature"])]
    lap("keypoints")
    sd, _ = shot352(sv, sn, keys, p["descriptor_r"])
    lap("shot")
    idx, d2 = match(sd, model["desc"])
    lap("match")
    m = (idx >= 0) & (d2 < np.float32(p["match_max_d2"]))
    cs = np.nonzero(m)[0].astype(np.int32)
    cm = idx[m]
    cd = d2[m]
    out = {"n_voxels": len(sv), "n_keypoints": len(keys), "n_correspondences": int(m.sum()),
           "instances": []}
    if stages is not None:
        stages.update(sv=sv, sn=sn, keys=keys, sd=sd, idx=idx, d2=d2)
    if len(cs) == 0:
        out["n_clusters"] = 0
        return out
    clus, poses, sizes = gc_group(model["kp"], sv[keys], cm, cs, cd, p["gc_size"], p["gc_thresh"],
                                  p["max_clusters"])
    lap("grouping")
    if stages is not None:
        stages.update(corr_s=cs, corr_m=cm, cluster_of=clus)
    out["n_clusters"] = len(sizes)
    if len(sizes) == 0:
        return out
    # one exact search grid over the scene voxels serves the hypothesis
    # scores, the ICP refinements and the final scores
    grid = Grid(sv, 0.5 * p["icp_max_dist"])
    hv = grid.inlier_fraction(model["vox"], p["hv_subsample"], poses, p["hv_inlier_r"])
    order = sorted(range(len(sizes)), key=lambda h: (-hv[h], h))[: p["refine_top"]]
    refined = [r["pose"] for r in grid.icp_multi(model["vox"], p["icp_iterations"], p["icp_max_dist"],
                                                 poses[order])] if order else []
    fscore = list(grid.inlier_fraction(model["vox"], 1, np.array(refined).reshape(-1, 16),
                                       p["accept_inlier_r"])) if refined else []
    grid.close()
    lap("verify_refine")
    picked = []
    for k in sorted(range(len(order)), key=lambda k: (-fscore[k], k)):
        if len(picked) >= p["max_instances"] or fscore[k] < p["accept_score"]:
            break
        if any(np.sum((refined[j][:3, 3] - refined[k][:3, 3]) ** 2) < p["nms_dist"] ** 2 for j in picked):
            continue
        picked.append(k)
        out["instances"].append({"pose": refined[k], "score": fscore[k], "hypothesis": order[k],
                                 "cluster_size": int(sizes[order[k]])})
    return out
