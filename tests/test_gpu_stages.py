"""GPU parity of the recognition stages against the CPU oracle.

Voxel filter, uniform sampling, normals and the outward orientation are
integer/rounding-exact restatements: bit-exact.  SHOT sums its support in
64-bit fixed point (order-free) with the same IEEE operations per term as
the oracle: descriptors and LRFs bit-exact.  The descriptor matcher is
bit-exact (sequential FP32 sums, lowest-index ties)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _host(t):
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def clouds(rtr):
    model = rtr.synth_shape(rtr.CHAIR, 20000, 2024)
    p = rtr.room_default_params()
    p.n_points = 60000
    scene, _, _ = rtr.synth_room(3, p)
    return model, scene


@pytest.mark.parametrize("leaf", [0.01, 0.02, 0.0037])
def test_voxel_downsample_bit_exact(ctx, clouds, leaf):
    for pts in clouds:
        got = _host(ctx.voxel_downsample(_dev(pts), leaf))
        ref = O.voxel_downsample(pts, leaf)
        assert got.shape == ref.shape
        assert np.array_equal(got[:, :3], ref[:, :3])


def test_voxel_downsample_edge_cases(ctx, rtr):
    import torch
    one = np.array([[0.5, -0.25, 3.0, 0.0]], np.float32)
    assert np.array_equal(_host(ctx.voxel_downsample(_dev(one), 0.01))[:, :3], one[:, :3])
    dup = np.repeat(one, 100, axis=0)
    got = _host(ctx.voxel_downsample(_dev(dup), 0.01))
    assert got.shape[0] == 1 and np.array_equal(got[:, :3], O.voxel_downsample(dup, 0.01)[:, :3])
    e = torch.zeros((0, 4), dtype=torch.float32, device="cuda")
    assert ctx.voxel_downsample(e, 0.01).shape[0] == 0
    # a key space beyond 2^32 is reported, not wrapped
    far = np.array([[0, 0, 0, 0], [1e6, 1e6, 1e6, 0]], np.float32)
    with pytest.raises(rtr.RtrError):
        ctx.voxel_downsample(_dev(far), 0.001)


@pytest.mark.parametrize("r", [0.02, 0.05])
def test_uniform_sample_exact(ctx, clouds, r):
    for pts in clouds:
        v = O.voxel_downsample(pts, 0.01)
        got = _host(ctx.uniform_sample(_dev(v), r))
        assert np.array_equal(got, O.uniform_sample(v, r))


@pytest.mark.parametrize("k", [10, 16])
def test_normals_bit_exact(ctx, clouds, k):
    vp = (0.0, -2.5, 1.5)
    for pts in clouds:
        v = O.voxel_downsample(pts, 0.01)
        got = _host(ctx.normals(_dev(v), k, vp, 0.02))
        ref = O.normals(v, k, vp)
        assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_orient_outward_exact(ctx, clouds):
    v = O.voxel_downsample(clouds[0], 0.01)
    n = O.normals(v, 10, (0.0, 0.0, 0.0))
    d_n = _dev(n)
    ctx.orient_outward(_dev(v), d_n)
    assert np.array_equal(_host(d_n), O.orient_outward(v, n))


def test_shot352_matches_oracle(ctx, clouds):
    for pts, vp in ((clouds[0], (0, 0, 0)), (clouds[1], (0.0, -2.5, 1.5))):
        v = O.voxel_downsample(pts, 0.01)
        n = O.normals(v, 10, vp)
        keys = O.uniform_sample(v, 0.02)
        import torch
        got, glrf = ctx.shot352(_dev(v), _dev(n), torch.from_numpy(keys).cuda(), 0.04, lrf=True)
        got = _host(got)
        ref, rlrf = O.shot352(v, n, keys, 0.04)
        assert np.array_equal(got, ref), (np.abs(got - ref).max(axis=1) > 0).sum()
        assert np.array_equal(_host(glrf), rlrf)
        # unit-norm histograms, or all-zero for a keypoint with an empty support
        nrm = np.linalg.norm(got, axis=1)
        assert np.all((np.abs(nrm - 1.0) < 1e-5) | (nrm == 0.0))


def test_shot352_independent_of_point_order(ctx, clouds):
    """The same voxels in a shuffled order (so the grid cells hold them in
    another order and the lanes meet them in another order) give the same
    descriptor and LRF bits per keypoint."""
    import torch
    v = O.voxel_downsample(clouds[1], 0.01)
    n = O.normals(v, 10, (0.0, -2.5, 1.5))
    keys = O.uniform_sample(v, 0.02)
    perm = np.random.default_rng(9).permutation(len(v))
    inv = np.argsort(perm).astype(np.int32)
    a, la = ctx.shot352(_dev(v), _dev(n), torch.from_numpy(keys).cuda(), 0.04, lrf=True)
    b, lb = ctx.shot352(_dev(v[perm]), _dev(n[perm]), torch.from_numpy(inv[keys]).cuda(), 0.04, lrf=True)
    assert torch.equal(a, b) and torch.equal(la, lb)


def test_match_exact_bit_exact(ctx, clouds):
    v = O.voxel_downsample(clouds[0], 0.01)
    n = O.normals(v, 10, (0, 0, 0))
    km = O.uniform_sample(v, 0.01)
    ks = O.uniform_sample(v, 0.02)
    md, _ = O.shot352(v, n, km, 0.04)
    sd, _ = O.shot352(v, n, ks, 0.04)
    sd = sd[:3000]
    idx, d2 = ctx.match_exact(_dev(sd), _dev(md))
    ri, rd = O.match(sd, md)
    assert np.array_equal(_host(idx), ri)
    assert np.array_equal(_host(d2), rd)
    # duplicates in the database: ties go to the lowest index
    md2 = np.concatenate([md[:100], md[:100]])
    idx, _ = ctx.match_exact(_dev(md[:100]), _dev(md2))
    assert np.array_equal(_host(idx), np.arange(100))
