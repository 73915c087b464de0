"""rtr_knn1_static (the allocation-free 1-NN whose grid sits in a fixed
device array of the library) against rtr_knn1 on the same inputs.  Both run
the same search kernel, so the tolerance is zero: indices and squared
distances must be identical.  Two different calls in a row check that the
second call does not see the first one's grid.  This file is collected last
so that the check also holds after every other test has used the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _rand(rng, n, scale):
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(-scale, scale, (n, 3))
    return p


def test_knn1_static_matches_knn1_twice(ctx, rtr):
    import torch
    rng = np.random.default_rng(77)
    cases = [
        (_rand(rng, 30000, 0.5), _rand(rng, 20000, 0.6), 0.05),          # bounded
        (_rand(rng, rtr.KNN1_STATIC_MAX_TARGET, 2.0), _rand(rng, 9000, 2.5), 0.0),  # at the maximum
    ]
    outs = []
    for t, q, r in cases:  # two calls in a row on one stream, no sync between
        dq, dt = _dev(q), _dev(t)
        outs.append((dq, dt, r, ctx.knn1_static(dq, dt, r)))
    torch.cuda.synchronize()
    for dq, dt, r, (si, sd) in outs:
        ki, kd = ctx.knn1(dq, dt, r)
        si, sd, ki, kd = (x.cpu().numpy() for x in (si, sd, ki, kd))
        assert np.array_equal(si, ki)
        ok = ki >= 0
        np.testing.assert_array_equal(sd[ok], kd[ok])  # tolerance 0
        assert np.all(np.isinf(sd[~ok]))


def test_knn1_static_flat_and_duplicate_targets(ctx, rtr):
    """Where the cell table's size limit binds (a flat target, unbounded
    search) and where targets repeat (ties go to the lowest index), the
    static call still equals rtr_knn1, on two calls in a row."""
    import torch
    rng = np.random.default_rng(79)
    flat = _rand(rng, 6000, 1.0)
    flat[:, 2] = 0.0
    dup = _rand(rng, 3000, 0.2)
    dup = np.concatenate([dup, dup[::-1], dup[:500]])  # every point at least twice
    q1, q2 = _rand(rng, 4000, 1.2), dup[:, :].copy()
    q2[:, :3] += rng.normal(0, 1e-3, (q2.shape[0], 3)).astype(np.float32)
    outs = []
    for t, q in ((flat, q1), (dup, q2)):
        dq, dt = _dev(q), _dev(t)
        outs.append((dq, dt, ctx.knn1_static(dq, dt, 0.0)))
    torch.cuda.synchronize()
    for dq, dt, (si, sd) in outs:
        ki, kd = ctx.knn1(dq, dt, 0.0)
        assert torch.equal(si, ki) and torch.equal(sd, kd)


def test_knn1_static_preallocated_outputs_and_limit(ctx, rtr):
    import torch
    rng = np.random.default_rng(78)
    t, q = _rand(rng, 5000, 0.3), _rand(rng, 3000, 0.3)
    dq, dt = _dev(q), _dev(t)
    out = (torch.full((3000,), -7, dtype=torch.int32, device="cuda"),
           torch.zeros(3000, dtype=torch.float32, device="cuda"))
    ctx.knn1_static(dq, dt, 0.0, out=out)
    ki, kd = ctx.knn1(dq, dt, 0.0)
    assert torch.equal(out[0], ki) and torch.equal(out[1], kd)
    # beyond the fixed maximum: refused on the host before any launch
    big = torch.zeros((rtr.KNN1_STATIC_MAX_TARGET + 1, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(rtr.RtrError, match="exceeds the fixed maximum"):
        ctx.knn1_static(dq, big, 0.0, out=out)
    assert torch.equal(out[0], ki)  # outputs untouched by the refused call
    # a host buffer is refused on the host, before any launch
    host_q = np.ascontiguousarray(q)
    st = rtr.lib().rtr_knn1_static(host_q.ctypes.data, 3000, dt.data_ptr(), 5000, 0.0, out[0].data_ptr(),
                                   out[1].data_ptr(), 0)
    assert st == 1 and "not device memory" in rtr.lib().rtr_last_error().decode()
    assert torch.equal(out[0], ki)
