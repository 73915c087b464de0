"""The reference's C++ entry points (ModelPoint / ScanPoint::getKeypoint, the
correspondence loop, Ransac, keyPointICP) as kept by
realtime_robot_gb300/cpp/realtime_robot.hpp over the C ABI, driven as main
drives them (realtime_robot_demo) on a cropped, moved chair.

The demo exits 0 when its refined pose is within 1 cm / 1 degree of the
generator's.  With the workload's 2 cm model keypoints the oracle pipeline
itself registers only some crops within 1 cm / 1 degree (others keep a
slide along the chair or settle on the chair turned by 180 degrees).  So
wherever the oracle pipeline registers the chair the demo must register it
too, and it must register at least as many seeds as the oracle does."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEMO = Path(__file__).resolve().parents[1] / "realtime_robot_gb300" / "realtime_robot_demo"
SEEDS = range(8)


def _oracle_found(R, O, OP, om, seed):
    """The oracle pipeline on the demo's clouds (same generator calls):
    whether its best instance is within 1 cm / 1 degree of the truth."""
    Tm = R.synth_rigid(100 + seed, 30.0, 0.3)
    seg = R.synth_transform_noise(R.synth_crop(R.synth_shape(R.CHAIR, 20000, 500 + seed), 0.4, seed), Tm, 0.002,
                                  9 + seed)
    ref = OP.recognize(om, seg, OP.params(scene_outward=1))
    if not ref["instances"]:
        return False
    e = O.pose_error(ref["instances"][0]["pose"], Tm)
    return e[0] < 0.01 and e[1] < np.radians(1.0)


def test_cpp_entry_points_register_a_chair(rtr):
    import oracle as O
    from oracle import pipeline as OP
    assert DEMO.exists(), "build() makes the demo next to librtr.so"
    om = OP.prepare_model(rtr.synth_shape(rtr.CHAIR, 20000, 2024), OP.params(scene_outward=1))
    ok = found = 0
    for seed in SEEDS:
        r = subprocess.run([str(DEMO), str(seed)], capture_output=True, text=True, timeout=120)
        assert r.returncode in (0, 1), (seed, r.returncode, r.stdout, r.stderr)
        m = re.search(r"pairs (\d+)", r.stdout)
        assert m and int(m.group(1)) > 50, (seed, r.stdout)
        m = re.search(r"refined ([0-9.]+) m ([0-9.]+) deg", r.stdout)
        assert m, (seed, r.stdout)
        within = float(m.group(1)) < 0.01 and float(m.group(2)) < 1.0
        assert within == (r.returncode == 0), (seed, r.stdout)
        if _oracle_found(rtr, O, OP, om, seed):
            found += 1
            assert within, (seed, r.stdout)
        ok += within
    assert found >= 2 and ok >= found, (ok, found)


@pytest.mark.parametrize("seed", [1, 3])
def test_cpp_reference_route_members(rtr, seed):
    """main's own route on the kept KeyPoint members (getArea / get_Area,
    getOccupiedGrid, get_TSDF, get_Vector3D, get_Distance, match_by_*; one
    keypoint / pair per call): every pair's score bit for bit and every keep
    decision (the area gate live on the clouds' plane areas) equal to the
    oracle's batched route on the same clouds."""
    from oracle import plane_segment, ref_correspond, ref_distance, ref_occupancy, ref_tdf, vector3d
    r = subprocess.run([str(DEMO), "ref", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr)
    got = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("pair ")]
    model = rtr.synth_shape(rtr.CHAIR, 3000, 40 + seed)
    scan = rtr.synth_shape(rtr.CHAIR, 3000, 41 + seed).copy()
    scan[:, 0] += np.float32(0.01) * np.float32(seed % 5)
    km, ks = model[::150].copy(), scan[::200].copy()
    mn, mo, mi = ref_occupancy(model, km)
    sn, _, _ = ref_occupancy(scan, ks)
    sc, _ = ref_distance(model, km, mo, mi, ref_tdf(model, km, mo, mi), ks)
    ms, ss = plane_segment(model)[0], plane_segment(scan)[0]
    m_surf = re.search(r"surfaces (\d+) (\d+)", r.stdout)
    assert m_surf and (int(m_surf.group(1)), int(m_surf.group(2))) == (sum(x.kept for x in ms), sum(x.kept for x in ss))
    from oracle import harris3d
    m_h = re.search(r"harris (\d+) (\d+)", r.stdout)
    assert m_h and (int(m_h.group(1)), int(m_h.group(2))) == (len(harris3d(model)[0]), len(harris3d(scan)[0]))
    kept = set(ref_correspond(km, mn, ks, sn, sc, mv3=vector3d(km, ms), sv3=vector3d(ks, ss)).tolist())
    assert len(got) == km.shape[0] * ks.shape[0]
    for g in got:
        m, s = int(g[1]), int(g[2])
        p = m * ks.shape[0] + s
        assert int(g[3], 16) == int(sc[p:p + 1].view(np.uint32)[0]), (m, s, g, sc[p])
        assert (g[4] == "1") == (p in kept), (m, s)
