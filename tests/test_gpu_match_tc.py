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
