"""rtr_plane_segment and rtr_vector3d (ModelPoint::getArea /
ScanPoint::get_Area, KeyPoint::get_Vector3D) on the GPU against the oracle
(oracle/planes.c), bit for bit: the same planes in the same order, their
float coefficients, inlier counts, hull vertex counts, areas and
perimeters; then the plane-area vectors and the reference's area gate
(match_by_area) that they feed."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _same(gpu, ref):
    assert len(gpu) == len(ref)
    for g, r in zip(gpu, ref):
        assert list(g.coeffs) == list(r.coeffs)
        for f in ("n_inliers", "hull_vertices", "is_vertical", "kept", "flat"):
            assert getattr(g, f) == getattr(r, f), f
        assert g.area == r.area and g.perimeter == r.perimeter


def _clouds(rtr):
    scene, _, _ = rtr.synth_room(1)
    d = np.load(GOLDEN / "main_clouds.npz")
    return {"room": scene, "chair": rtr.synth_shape(rtr.CHAIR, 20000, 2024),
            "sofa": rtr.synth_shape(rtr.SOFA, 30000, 7), "chair1": d["chair1"], "T0_m8111": d["T0_m8111"]}


@pytest.mark.parametrize("name", ["room", "chair", "sofa", "chair1", "T0_m8111"])
def test_plane_segment_equals_oracle(ctx, rtr, name):
    pts = _clouds(rtr)[name]
    for seed in (0, 3):
        got = ctx.plane_segment(_dev(pts), rtr.plane_default_params(seed=seed))
        ref, tot = O.plane_segment(pts, seed=seed)
        assert tot == len(ref)
        _same(got, ref)
    assert any(s.kept for s in got) or name in ("chair1", "T0_m8111")


def test_plane_segment_ignores_nonfinite_points(ctx, rtr):
    pts = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    bad = np.insert(pts, [0, 500, 9000, 20000], np.float32([[np.nan, 0, 0, 0], [np.inf, 1, 1, 0],
                                                            [0, -np.inf, 0, 0], [1, 2, np.nan, 0]]), axis=0)
    _same(ctx.plane_segment(_dev(bad)), ctx.plane_segment(_dev(pts)))
    assert ctx.plane_segment(_dev(np.full((100, 4), np.nan, np.float32))) == []


def test_vector3d_and_area_gate_equal_oracle(ctx, rtr):
    d = np.load(GOLDEN / "main_clouds.npz")
    model, scan = d["chair1"], d["T0_m8111"]
    km = model[O.uniform_sample(model, 0.05)]
    ks = scan[O.uniform_sample(scan, 0.05)]
    room, _, _ = rtr.synth_room(1)
    # surfaces of the room (large floor and walls) and of the chair model
    for cloud, keys in ((room, room[::997].copy()), (rtr.synth_shape(rtr.CHAIR, 20000, 2024), km)):
        surf = ctx.plane_segment(_dev(cloud))
        v = ctx.vector3d(_dev(keys), surf).cpu().numpy()
        assert np.array_equal(v, O.vector3d(keys, surf))
    # main's own clouds: each side's planes and vectors, then the gated
    # all-pairs loop with the area gate live
    ms, ss = ctx.plane_segment(_dev(model)), ctx.plane_segment(_dev(scan))
    mv3 = ctx.vector3d(_dev(km), ms)
    sv3 = ctx.vector3d(_dev(ks), ss)
    dm, ds, dkm, dks = _dev(model), _dev(scan), _dev(km), _dev(ks)
    mn, mo, mi = ctx.ref_occupancy(dm, dkm)
    sn, _, _ = ctx.ref_occupancy(ds, dks)
    tdf = ctx.ref_tdf(dm, dkm, mo, mi)
    sc, _ = ctx.ref_distance(dm, dkm, mo, mi, tdf, dks)
    pi = ctx.ref_correspond(dkm, mn, dks, sn, sc, mv3=mv3, sv3=sv3)
    rpi = O.ref_correspond(km, mn.cpu().numpy(), ks, sn.cpu().numpy(), sc.cpu().numpy(), mv3=mv3.cpu().numpy(),
                           sv3=sv3.cpu().numpy())
    assert np.array_equal(pi.cpu().numpy(), rpi)
