"""GPU parity of the tensor-core descriptor matcher: indices and distances
bit-identical to the exact FP32 oracle, and the BF16(hi+lo) GEMM accurate
enough that almost every query is certified by its top-8 (so the tensor-core
path, not the exact fallback, produces the answer)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.fixture(scope="module")
def descs(rtr):
    model = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    v = O.voxel_downsample(model, 0.01)
    n = O.orient_outward(v, O.normals(v, 10, (0, 0, 0)))
    md, _ = O.shot352(v, n, O.uniform_sample(v, 0.01), 0.04)
    p = rtr.room_default_params()
    p.n_points = 80000
    scene, _, _ = rtr.synth_room(4, p)
    sv = O.voxel_downsample(scene, 0.01)
    sn = O.normals(sv, 10, (0.0, -2.5, 1.5))
    sd, _ = O.shot352(sv, sn, O.uniform_sample(sv, 0.02), 0.04)
    return md, sd


def test_match_tc_bit_exact(ctx, descs):
    md, sd = descs
    idx, d2 = ctx.match(_dev(sd), _dev(md))
    unc = ctx.match_uncertified()
    ri, rd = O.match(sd, md)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)
    # the GEMM, not the fallback, decides: nearly every query certified
    assert unc <= 0.02 * len(sd), (unc, len(sd))


def test_match_tc_ragged_sizes(ctx, descs):
    md, sd = descs
    for nq, ndb in ((1, 1), (5, 3), (129, 257), (300, 1000), (1000, 9)):
        q, db = sd[:nq], md[:ndb]
        idx, d2 = ctx.match(_dev(q), _dev(db))
        ri, rd = O.match(q, db)
        assert np.array_equal(idx.cpu().numpy(), ri), (nq, ndb)
        assert np.array_equal(d2.cpu().numpy(), rd), (nq, ndb)


def test_match_tc_duplicates_tie_to_lowest(ctx, descs):
    md, sd = descs
    db = np.concatenate([md[:50]] * 12)  # every descriptor 12 times
    idx, _ = ctx.match(_dev(md[:50]), _dev(db))
    assert np.array_equal(idx.cpu().numpy(), np.arange(50))


@pytest.mark.parametrize("scale", [1e-3, 37.0, 1e3])
def test_match_tc_scaled_descriptors(ctx, descs, scale):
    # the certification bound scales with the descriptor norms
    md, sd = descs
    q = (sd[:3000] * np.float32(scale)).astype(np.float32)
    db = (md * np.float32(scale)).astype(np.float32)
    idx, d2 = ctx.match(_dev(q), _dev(db))
    ri, rd = O.match(q, db)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)


def test_match_tc_general_vectors(ctx):
    # signed, non-normalised vectors whose distances crowd together: most
    # queries cannot be certified and go through the exact re-scan
    rng = np.random.default_rng(12)
    q = rng.standard_normal((1500, 352)).astype(np.float32)
    db = rng.standard_normal((2500, 352)).astype(np.float32)
    idx, d2 = ctx.match(_dev(q), _dev(db))
    ri, rd = O.match(q, db)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)


def _near_tie_db(md, group, n_groups, seed):
    """n_groups clusters of `group` rows each, equal to a model descriptor up
    to a 1e-6 perturbation: their distances to a query differ far below the
    certification margin, so every query near a cluster is uncertified."""
    rng = np.random.default_rng(seed)
    base = []
    for i in rng.permutation(len(md)):  # well-separated cluster centres (d^2 > 0.05)
        if all(float(((md[i] - b) ** 2).sum()) > 0.05 for b in base):
            base.append(md[i])
        if len(base) == n_groups:
            break
    base = np.asarray(base, np.float32)
    db = np.repeat(base, group, axis=0)
    db = db + np.float32(1e-6) * rng.standard_normal(db.shape).astype(np.float32)
    perm = rng.permutation(len(db))  # cluster members spread over the database
    return base, np.ascontiguousarray(db[perm], np.float32)


@pytest.mark.parametrize("group,expect_full", [(100, False), (400, True)])
def test_match_tc_near_tie_bands(ctx, descs, group, expect_full):
    # clusters up to 256 rows are settled by the band pass; larger ones by
    # the exact scan of the whole database
    md, _ = descs
    base, db = _near_tie_db(md, group, 8, 5 + group)
    rng = np.random.default_rng(group)
    q = np.repeat(base, 40, axis=0) + np.float32(1e-3) * rng.standard_normal((320, 352)).astype(np.float32)
    q = q.astype(np.float32)
    idx, d2 = ctx.match(_dev(q), _dev(db))
    unc, full = ctx.match_uncertified(), ctx.match_full_scans()
    ri, rd = O.match(q, db)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)
    assert unc == len(q)
    assert (full == unc) if expect_full else (full == 0), (unc, full)


def test_match_tc_more_uncertified_than_band_rows(ctx, descs):
    # past 16384 uncertified queries the rest take the full scan
    md, _ = descs
    base, db = _near_tie_db(md, 64, 4, 77)
    rng = np.random.default_rng(3)
    q = (np.repeat(base, 4200, axis=0) + np.float32(1e-3) * rng.standard_normal((16800, 352))).astype(np.float32)
    idx, d2 = ctx.match(_dev(q), _dev(db))
    unc, full = ctx.match_uncertified(), ctx.match_full_scans()
    ri, rd = O.match(q, db)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd)
    assert unc == len(q) and full == len(q) - 16384, (unc, full)


def test_match_tc_zero_and_nonfinite_queries(ctx, descs):
    # a zero query ties with every unit-norm row (band = whole database);
    # Inf or NaN values make the threshold non-finite: both take the full scan
    md, sd = descs
    q = sd[:64].copy()
    q[:8] = 0.0
    q[8, 5] = np.inf
    q[9, 7] = np.nan
    q[10, :] = -np.inf
    idx, d2 = ctx.match(_dev(q), _dev(md))
    ri, rd = O.match(q, md)
    assert np.array_equal(idx.cpu().numpy(), ri)
    assert np.array_equal(d2.cpu().numpy(), rd, equal_nan=True)
    assert ctx.match_full_scans() >= 3
