"""The learned form of recognition: training data, training and evaluation of
the keypoint-credibility MLP (rtr_mlp_*, rtr_recognize_learned).

Pairs follow the batched-registration workload: a model shape (box chair,
desk or sofa) and an independently sampled copy of it under a seeded rigid
transform (rotation <= 30 deg, translation +-0.3 m per axis), with
N(0, 2 mm) noise and 0-40 % of it cropped away by a random plane.

Labels: a scene keypoint is credible (label 1) when its descriptor match is
an inlier, within 1 cm, at the plain pipeline's final pose (its first
instance; keypoints of pairs where it finds none are all 0).  This is the
default (label_pose="plain"); label_pose="truth" labels at the generator's
pose instead, a side experiment.  Credible keypoints are a few in 10^4, so
training repeats them (balance) until they make a tenth of the rows.
Training runs on the GPU (rtr_mlp_train: the library's own
forward/backward/Adam kernels).  Evaluation compares the
learned form with the plain one pair by pair; a pair whose learned pose
differs from the plain pose by more than 1 cm or 1 deg counts as a fallback
(the plain result stands).

Every computation goes through librtr.so; this module only orchestrates.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import (CHAIR, DESK, SOFA, Mlp, Model, parse_recog_result, recog_default_params, recognize,
               recognize_learned, synth_crop, synth_rigid, synth_shape, synth_transform_noise)

SHAPES = (CHAIR, DESK, SOFA)


def make_pair(seed: int, shape: int | None = None, n_model: int | None = 20000, n_seg: int | None = None):
    """(shape, model points, segment points, true model->segment pose).
    n_seg / n_model None: drawn log-uniform in [2,000, 60,000] (the batched
    workload draws both the source and the target size)."""
    rng = np.random.default_rng(seed)
    shape = SHAPES[seed % 3] if shape is None else shape
    if n_seg is None:
        n_seg = int(round(math.exp(rng.uniform(math.log(2000), math.log(60000)))))
    if n_model is None:
        n_model = int(round(math.exp(rng.uniform(math.log(2000), math.log(60000)))))
    model = synth_shape(shape, n_model, 1000 + shape)
    T = synth_rigid(seed, 30.0, 0.3)
    seg = synth_transform_noise(synth_shape(shape, n_seg, 7 * seed + 1), T, 0.002, seed + 11)
    seg = synth_crop(seg, 0.4, seed + 13)
    return shape, model, seg, T


def pose_diff(A: np.ndarray, B: np.ndarray):
    """(translation m, rotation deg) between two 4x4 poses."""
    dt = float(np.linalg.norm(A[:3, 3] - B[:3, 3]))
    R = A[:3, :3].T @ B[:3, :3]
    c = max(-1.0, min(1.0, (np.trace(R) - 1.0) / 2.0))
    return dt, math.degrees(math.acos(c))


def _model_features(ctx, model_dev, p):
    """Model keypoints and descriptors, the stages of rtr_model_create."""
    leaf = p.voxel_leaf
    v = ctx.voxel_downsample(model_dev, leaf).contiguous()
    n = ctx.normals(v, p.normal_k, (0.0, 0.0, 0.0), 2.0 * leaf)
    ctx.orient_outward(v, n, 0.01, 0.005, 1.0)
    k = ctx.uniform_sample(v, p.model_keypoint_r).contiguous()
    d = ctx.shot352(v, n, k, p.descriptor_r)
    return v[k.long()].contiguous(), d


def _scene_features(ctx, scene_dev, p):
    """Scene keypoints and descriptors, the stages of rtr_recognize."""
    leaf = p.voxel_leaf
    v = ctx.voxel_downsample(scene_dev, leaf).contiguous()
    n = ctx.normals(v, p.normal_k, tuple(p.viewpoint), 2.0 * leaf)
    if p.scene_outward:
        ctx.orient_outward(v, n, 0.01, 0.005, 1.0)
    k = ctx.uniform_sample(v, p.scene_keypoint_r).contiguous()
    if p.keypoint_min_curvature > 0:
        k = k[n[k.long(), 3] >= p.keypoint_min_curvature].contiguous()
    d = ctx.shot352(v, n, k, p.descriptor_r)
    return v[k.long()].contiguous(), d


def harvest(ctx, model_dev, scene_dev, p=None, model: Model | None = None, truth: np.ndarray | None = None):
    """(descriptors [K,352] device, labels [K] device, plain result dict) for
    one model/scene pair; labels at `truth` when given, else at the plain
    pipeline's first instance."""
    import torch
    p = p or recog_default_params()
    own = model is None
    model = model or Model(ctx, model_dev, p)
    try:
        plain = parse_recog_result(recognize(ctx, model, scene_dev, p))
    finally:
        if own:
            model.close()
    mkp, mdesc = _model_features(ctx, model_dev, p)
    skp, sdesc = _scene_features(ctx, scene_dev, p)
    idx, d2 = ctx.match(sdesc, mdesc)
    y = torch.zeros(skp.shape[0], dtype=torch.float32, device=skp.device)
    ref = truth if truth is not None else (plain["instances"][0]["pose"] if plain["instances"] else None)
    if ref is not None:
        T = torch.as_tensor(np.asarray(ref, np.float64), dtype=torch.float64, device=skp.device)
        ok = (idx >= 0) & (d2 < p.match_max_d2)
        m = mkp[idx.clamp(min=0).long(), :3].double()
        pred = m @ T[:3, :3].T + T[:3, 3]
        err = torch.linalg.norm(pred - skp[:, :3].double(), dim=1)
        y = (ok & (err <= 0.01)).float()
    return sdesc, y, plain


def build_dataset(ctx, seeds, p=None, label_pose: str = "plain"):
    """Descriptors and labels harvested from the pairs of the given seeds."""
    import torch
    xs, ys = [], []
    for s in seeds:
        _, model, seg, T = make_pair(int(s))
        x, y, _ = harvest(ctx, torch.from_numpy(model).cuda(), torch.from_numpy(seg).cuda(), p,
                          truth=T if label_pose == "truth" else None)
        xs.append(x)
        ys.append(y)
    return torch.cat(xs).contiguous(), torch.cat(ys).contiguous()


def balance(X, y, pos_frac: float = 0.1, seed: int = 0):
    """(X, y) with the positive rows repeated until they make about pos_frac
    of the rows (credible keypoints are a few in 10^4; without this the
    network scores every keypoint near 0 and ranks them poorly)."""
    import torch
    pos = torch.nonzero(y > 0.5).flatten()
    n_pos, n = int(pos.numel()), int(y.numel())
    if n_pos == 0 or n_pos >= pos_frac * n:
        return X, y
    reps = int(math.ceil(pos_frac * (n - n_pos) / ((1.0 - pos_frac) * n_pos)))
    extra = pos.repeat(reps - 1)
    g = torch.Generator(device="cpu").manual_seed(seed)
    order = torch.randperm(n + extra.numel(), generator=g).to(y.device)
    Xb = torch.cat([X, X[extra]])[order].contiguous()
    yb = torch.cat([y, y[extra]])[order].contiguous()
    return Xb, yb


def train(ctx, X, y, epochs: int = 20, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
    """A fresh MLP trained on (X, y) with the GPU kernels; returns (mlp, epoch losses)."""
    mlp = Mlp(ctx, seed=seed)
    losses = mlp.train(X, y, batch=batch, epochs=epochs, lr=lr, seed=seed + 1)
    return mlp, losses


def evaluate(ctx, mlp: Mlp, seeds, keep: float = 0.25, p=None, repeats: int = 3):
    """Learned vs plain on the pairs of the given seeds: agreement (<= 1 cm and
    1 deg between the first instances, or neither finds one), fallbacks and
    per-pair times (ms, after warm-up)."""
    import torch
    p = p or recog_default_params()
    rows = []
    for s in seeds:
        _, model, seg, T = make_pair(int(s))
        md = torch.from_numpy(model).cuda()
        sd = torch.from_numpy(seg).cuda()
        mod = Model(ctx, md, p)
        try:
            rp = parse_recog_result(recognize(ctx, mod, sd, p))
            rl = parse_recog_result(recognize_learned(ctx, mod, mlp, sd, keep, p))
            times = {}
            for name, fn in (("plain", lambda: recognize(ctx, mod, sd, p)),
                             ("learned", lambda: recognize_learned(ctx, mod, mlp, sd, keep, p))):
                fn()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(repeats):
                    fn()
                torch.cuda.synchronize()
                times[name] = (time.perf_counter() - t0) / repeats * 1e3
        finally:
            mod.close()
        if rp["instances"] and rl["instances"]:
            dt, dr = pose_diff(rp["instances"][0]["pose"], rl["instances"][0]["pose"])
            agree = dt <= 0.01 and dr <= 1.0
        else:
            dt = dr = float("nan")
            agree = not rp["instances"] and not rl["instances"]
        gt = pose_diff(rp["instances"][0]["pose"], T) if rp["instances"] else (float("nan"), float("nan"))
        lt = pose_diff(rl["instances"][0]["pose"], T) if rl["instances"] else (float("nan"), float("nan"))
        rows.append({"seed": int(s), "agree": bool(agree), "dt": dt, "dr": dr, "plain_found": bool(rp["instances"]),
                     "plain_vs_truth": gt, "learned_vs_truth": lt, "ms_plain": times["plain"], "ms_learned": times["learned"],
                     "kp_plain": rp["n_keypoints"], "kp_learned": rl["n_keypoints"]})
    return rows
