"""A recognition replayed from the context's own CUDA graph ("auto_graph").

The second identical rtr_recognize captures its launches and later ones
replay them.  Every replay must give the bytes of a direct call: with new
scene contents in the same buffer, after a parameter change, after the
scratch arena grew, with a new model, in the learned form and through the
host entry point; and it launches the same number of kernels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _segment(R, seed, n=None):
    T = R.synth_rigid(100 + seed, 30.0, 0.3)
    seg = R.synth_transform_noise(R.synth_crop(R.synth_shape(R.CHAIR, 20000, 500 + seed), 0.4, seed), T,
                                  0.002, 9 + seed)
    return seg if n is None else seg[:n]


def _result(R):
    import torch
    return torch.zeros(R.C.sizeof(R.RecogResult), dtype=torch.uint8, device="cuda")


def _direct(ctx, R, fn):
    """fn() run with the graph replay off; the context's setting restored."""
    ctx.set_tuning("auto_graph", 0)
    try:
        return fn()
    finally:
        ctx.set_tuning("auto_graph", 1)


def _run(R, ctx, m, scene, prm, res):
    import torch
    res.zero_()
    R.recognize(ctx, m, scene, prm, result=res)
    torch.cuda.synchronize()
    return bytes(res.cpu().numpy())


def test_replay_equals_direct_call(ctx, rtr):
    R = rtr
    model = R.synth_shape(R.CHAIR, 20000, 2024)
    prm = R.recog_default_params(scene_outward=1)
    m = R.Model(ctx, _dev(model), prm)
    s1, s2 = _segment(R, 1), _segment(R, 4)
    n = min(len(s1), len(s2))
    s1, s2 = s1[:n], s2[:n]
    scene = _dev(s1)
    res = _result(R)
    ref1 = _direct(ctx, R, lambda: _run(R, ctx, m, scene, prm, res))
    scene.copy_(_dev(s2))
    ref2 = _direct(ctx, R, lambda: _run(R, ctx, m, scene, prm, res))
    assert ref1 != ref2
    scene.copy_(_dev(s1))
    counts = []
    for _ in range(4):  # direct, capture + launch, replay, replay
        c0 = R.launch_count()
        assert _run(R, ctx, m, scene, prm, res) == ref1
        counts.append(R.launch_count() - c0)
    assert len(set(counts)) == 1 and counts[0] > 100, counts
    # new contents in the same buffer: the replay reads them
    scene.copy_(_dev(s2))
    assert _run(R, ctx, m, scene, prm, res) == ref2
    # another parameter set: a direct call, then its own graph
    prm2 = R.recog_default_params(scene_outward=1)
    prm2.max_instances = 1
    ref3 = _direct(ctx, R, lambda: _run(R, ctx, m, scene, prm2, res))
    for _ in range(3):
        assert _run(R, ctx, m, scene, prm2, res) == ref3
    m.close()


def test_replay_after_arena_growth_and_new_model(ctx, rtr):
    R = rtr
    prm = R.recog_default_params(scene_outward=1)
    m = R.Model(ctx, _dev(R.synth_shape(R.CHAIR, 20000, 2024)), prm)
    seg = _segment(R, 1)
    scene = _dev(seg)
    res = _result(R)
    ref = _direct(ctx, R, lambda: _run(R, ctx, m, scene, prm, res))
    for _ in range(3):
        assert _run(R, ctx, m, scene, prm, res) == ref
    # a much larger scene grows the arena: the graph's buffers moved
    big = np.concatenate([seg + np.float32([3.0 * k, 0, 0, 0]) for k in range(12)])
    big[:, 3] = 0
    R.recognize(ctx, m, _dev(big), prm)
    for _ in range(3):
        assert _run(R, ctx, m, scene, prm, res) == ref
    # a new model (possibly at the old one's address) is a new key
    m.close()
    m2 = R.Model(ctx, _dev(R.synth_shape(R.CHAIR, 20000, 77)), prm)
    ref2 = _direct(ctx, R, lambda: _run(R, ctx, m2, scene, prm, res))
    for _ in range(3):
        assert _run(R, ctx, m2, scene, prm, res) == ref2
    m2.close()


def test_replay_host_entry_and_learned(ctx, rtr):
    import torch
    R = rtr
    prm = R.recog_default_params(scene_outward=1)
    m = R.Model(ctx, _dev(R.synth_shape(R.CHAIR, 20000, 2024)), prm)
    seg = _segment(R, 4)
    ref = _direct(ctx, R, lambda: R.recognize_host(ctx, m, seg, prm))
    for _ in range(3):
        r = R.recognize_host(ctx, m, seg, prm)
        assert r["n_keypoints"] == ref["n_keypoints"] and len(r["instances"]) == len(ref["instances"])
        for a, b in zip(r["instances"], ref["instances"]):
            assert np.array_equal(a["pose"], b["pose"]) and a["score"] == b["score"]
    mlp = R.Mlp(ctx, seed=3)
    scene = _dev(seg)
    res = _result(R)

    def learned():
        res.zero_()
        R.recognize_learned(ctx, m, mlp, scene, keep=0.5, params=prm, result=res)
        torch.cuda.synchronize()
        return bytes(res.cpu().numpy())

    ref_l = _direct(ctx, R, learned)
    for _ in range(3):
        assert learned() == ref_l
    mlp.close()
    m.close()
