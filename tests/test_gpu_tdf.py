"""GPU parity of the TDF (kernel.cu's ComputeTDF / ComputeTDFWithCuda) against
the oracle's restatement of kernel.cu:8-31.  Integer-exact."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _occ(rng, n, dim):
    return rng.integers(0, dim, size=(n, 3)).astype(np.int32)


@pytest.mark.parametrize("n_occ", [0, 1, 37, 900, 5000])
def test_compute_tdf_with_cuda_dim30(rtr, n_occ):
    rng = np.random.default_rng(n_occ)
    occ = _occ(rng, n_occ, 30)
    g = np.full(27000, -7.0, np.float32)
    assert rtr.compute_tdf_with_cuda(occ, g, 30) == 0
    assert np.array_equal(g, O.tdf(occ, 30))


@pytest.mark.parametrize("dim", [1, 5, 12, 29])
def test_compute_tdf_small_dims_reproduce_the_extra_write(rtr, dim):
    """For dim < 30 the reference's guard (kernel.cu:13) also writes voxel
    index dim^3, i.e. the voxel (0, 0, dim), inside the 27,000-float buffer;
    everything after it keeps the caller's contents."""
    rng = np.random.default_rng(dim)
    occ = _occ(rng, 40, dim)
    g = np.full(27000, -7.0, np.float32)
    assert rtr.compute_tdf_with_cuda(occ, g, dim) == 0
    v = dim ** 3
    assert np.array_equal(g[:v], O.tdf(occ, dim))
    d = (0 - occ[:, 0]) ** 2 + (0 - occ[:, 1]) ** 2 + (dim - occ[:, 2]) ** 2
    assert g[v] == np.float32(min(900, d.min()))
    assert np.all(g[v + 1:] == -7.0)


def test_tdf_batch_many_keypoints(ctx):
    import torch
    rng = np.random.default_rng(3)
    counts = rng.integers(0, 3000, size=64)
    counts[5] = 0
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    occ = _occ(rng, int(offs[-1]), 30)
    out = ctx.tdf_batch(torch.from_numpy(occ).cuda(), torch.from_numpy(offs).cuda(), 30)
    out = out.cpu().numpy()
    for k in range(64):
        assert np.array_equal(out[k], O.tdf(occ[offs[k]:offs[k + 1]], 30)), k
