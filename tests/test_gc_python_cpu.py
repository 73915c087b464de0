"""The oracle's geometric-consistency grouping against a pure-Python
restatement of the sequential definition (PCL's GeometricConsistencyGrouping
rule, Chen & Bhanu 2007): correspondences in ascending descriptor distance
(ties: input order); each one not yet taken seeds a set that admits, in that
order, every other correspondence not yet taken whose model-side and
scene-side distances to every member differ by at most gc_size (FP32
distances); a set of at least gc_thresh members becomes a cluster and takes
its members; at most max_clusters clusters.  The GPU grouping equals the
oracle member for member, so this pins the rule both follow."""
import numpy as np

import oracle as O

f32 = np.float32


def _dist(a, b):
    dx, dy, dz = f32(a[0] - b[0]), f32(a[1] - b[1]), f32(a[2] - b[2])
    return np.sqrt(f32(f32(dx * dx + dy * dy) + dz * dz))


def gc_python(mk, sk, cm, cs, cd, gc, thresh, max_clusters):
    order = sorted(range(len(cd)), key=lambda i: (cd[i], i))
    taken = [False] * len(cd)
    cluster_of = [-1] * len(cd)
    sizes = []
    for i in order:
        if len(sizes) >= max_clusters:
            break
        if taken[i]:
            continue
        members = [i]
        for j in order:
            if j == i or taken[j]:
                continue
            if all(not abs(f32(_dist(mk[cm[m]], mk[cm[j]]) - _dist(sk[cs[m]], sk[cs[j]]))) > f32(gc)
                   for m in members):
                members.append(j)
        if len(members) >= thresh:
            for m in members:
                taken[m] = True
                cluster_of[m] = len(sizes)
            sizes.append(len(members))
    return np.array(cluster_of), np.array(sizes)


def test_oracle_grouping_equals_the_sequential_definition():
    import realtime_robot_gb300 as R
    rng = np.random.default_rng(2)
    nm, ns = 120, 600
    mk = np.zeros((nm, 4), np.float32)
    mk[:, :3] = rng.uniform(-0.3, 0.3, (nm, 3))
    sk = np.zeros((ns, 4), np.float32)
    sk[:, :3] = rng.uniform(-1.5, 1.5, (ns, 3))
    cm, cs = [], []
    for t in range(3):  # three planted rigid copies of model subsets, 2 mm noise
        T = R.synth_rigid(40 + t, 90.0, 1.0)
        pick = rng.choice(nm, 12, replace=False)
        idx = rng.choice(ns, 12, replace=False)
        sk[idx] = O.transform_f32(T, mk[pick]) + np.float32(0.002) * rng.standard_normal((12, 4)).astype(
            np.float32) * [1, 1, 1, 0]
        cm += list(pick)
        cs += list(idx)
    cm += list(rng.integers(0, nm, 250))
    cs += list(rng.integers(0, ns, 250))
    cm, cs = np.array(cm, np.int32), np.array(cs, np.int32)
    cd = rng.uniform(0, 0.3, len(cm)).astype(np.float32)
    cd[5] = cd[6]  # a distance tie: input order decides
    for gc, thresh, maxc in ((0.01, 5, 64), (0.03, 3, 64), (0.03, 3, 2)):
        clus, _, sizes = O.gc_group(mk, sk, cm, cs, cd, gc, thresh, maxc)
        ref_clus, ref_sizes = gc_python(mk, sk, cm, cs, cd, gc, thresh, maxc)
        assert np.array_equal(sizes, ref_sizes), (gc, thresh, sizes, ref_sizes)
        assert np.array_equal(clus, ref_clus), (gc, thresh)
    assert len(ref_sizes) == 2 and len(O.gc_group(mk, sk, cm, cs, cd, 0.01, 5, 64)[2]) >= 3
