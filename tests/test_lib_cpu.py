"""CPU tests of the C-ABI library: it loads without a GPU, exports every entry
point the headers declare, and its host-only parts (synthetic inputs, argument
checks) behave."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        for m in re.finditer(r"\b([A-Za-z_]\w*)\s*\(([^;{}]*)\)\s*;", txt):
            name = m.group(1)
            pre = txt[max(0, m.start() - 200):m.start()]
            stmt = pre[pre.rfind(";") + 1:] if ";" in pre else pre
            stmt = stmt[stmt.rfind("}") + 1:] if "}" in stmt else stmt
            if "typedef" in stmt or name in ("sizeof", "defined"):
                continue
            names.add(name)
    return sorted(names)


def test_headers_declare_entry_points():
    names = _declared_functions()
    assert "ComputeTDFWithCuda" in names and "rtr_icp" in names and "rtr_knn1" in names


def test_library_exports_every_declared_symbol(rtr):
    L = C.CDLL(str(rtr.LIB_PATH))
    missing = [n for n in _declared_functions() if not hasattr(L, n)]
    assert not missing, f"librtr.so lacks {missing}"
    # the Python mirror binds each of them with a signature
    unbound = [n for n in _declared_functions() if n not in rtr.declared_symbols()]
    assert not unbound, f"realtime_robot_gb300 has no binding for {unbound}"


def test_status_strings(rtr):
    L = rtr.lib()
    assert L.rtr_status_string(0) == b"RTR_OK"
    assert L.rtr_status_string(3) == b"RTR_ERR_TIMEOUT"
    assert L.rtr_version().decode().count(".") == 2


def test_synth_is_deterministic_and_on_the_chair(rtr):
    a = rtr.synth_shape(rtr.CHAIR, 5000, 7)
    b = rtr.synth_shape(rtr.CHAIR, 5000, 7)
    c = rtr.synth_shape(rtr.CHAIR, 5000, 8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    lo, hi = a[:, :3].min(0), a[:, :3].max(0)
    assert np.allclose(lo, [-0.225, -0.225, 0.0], atol=1e-6)
    assert np.allclose(hi, [0.225, 0.225, 0.93], atol=1e-6)
    assert np.all(a[:, 3] == 0)


def test_synth_rigid_is_a_rotation(rtr):
    for s in range(20):
        T = rtr.synth_rigid(s, 15.0, 0.1)
        R = T[:3, :3]
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12)
        assert abs(np.linalg.det(R) - 1) < 1e-12
        ang = np.arccos(np.clip((np.trace(R) - 1) / 2, -1, 1))
        assert ang <= np.deg2rad(15.0) + 1e-12
        assert np.all(np.abs(T[:3, 3]) <= 0.1)


def test_synth_room_shape_and_instances(rtr):
    p = rtr.room_default_params()
    p.n_points = 20000
    pts, shapes, poses = rtr.synth_room(11, p)
    assert pts.shape == (20000, 4)
    assert list(shapes).count(0) == 3 and list(shapes).count(1) == 1
    assert pts[:, 2].min() > -0.05 and pts[:, 1].max() < 2.55
    # camera at y = -2.5 sees everything in front of it
    assert pts[:, 1].min() > -2.55


def test_synth_crop_keeps_order(rtr):
    a = rtr.synth_shape(rtr.SOFA, 3000, 1)
    b = rtr.synth_crop(a, 0.4, 5)
    assert 0.6 * 3000 <= len(b) <= 3000
    # kept points appear in their original order
    pos = {tuple(r): i for i, r in enumerate(a)}
    order = [pos[tuple(r)] for r in b]
    assert order == sorted(order)


def test_context_without_gpu_fails_cleanly(rtr):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = rtr.lib().rtr_context_create(0, C.byref(h))
    assert st == 7  # RTR_ERR_NO_DEVICE
    assert b"device" in rtr.lib().rtr_last_error()


def test_compute_tdf_rejects_bad_sizes_without_touching_the_gpu(rtr):
    g = np.zeros(27000, np.float32)
    assert rtr.compute_tdf_with_cuda(np.zeros((1, 3), np.int32), g, 31) == 1  # cudaErrorInvalidValue
    assert rtr.lib().ComputeTDFWithCuda(None, g.ctypes.data, 30, -1) == 1


def test_cpp_mirror_fails_cleanly_without_a_gpu(rtr):
    """The C++ driver of the reference's entry points reports the missing
    device through rtr_status (exit 2), not a crash."""
    import subprocess
    from pathlib import Path
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    demo = Path(__file__).resolve().parents[1] / "realtime_robot_gb300" / "realtime_robot_demo"
    if not demo.exists():
        pytest.skip("demo not built")
    r = subprocess.run([str(demo)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "RTR_ERR_NO_DEVICE" in r.stderr, (r.returncode, r.stderr)


def _write_pcd(path, pts, binary, extra_rgb=False):
    """A PCD v0.7 file laid out like the reference's (chair1.pcd: binary
    x y z rgb; T0_m8111.pcd: ascii x y z)."""
    n = pts.shape[0]
    fields = "x y z rgb" if extra_rgb else "x y z"
    k = 4 if extra_rgb else 3
    hdr = (f"# .PCD v0.7 - Point Cloud Data file format\nVERSION 0.7\nFIELDS {fields}\nSIZE {' '.join(['4'] * k)}\n"
           f"TYPE {' '.join(['F'] * k)}\nCOUNT {' '.join(['1'] * k)}\nWIDTH {n}\nHEIGHT 1\n"
           f"VIEWPOINT 0 0 0 1 0 0 0\nPOINTS {n}\nDATA {'binary' if binary else 'ascii'}\n")
    rec = np.zeros((n, k), np.float32)
    rec[:, :3] = pts[:, :3]
    if extra_rgb:
        rec[:, 3] = np.arange(n, dtype=np.float32)
    with open(path, "wb") as f:
        f.write(hdr.encode())
        if binary:
            f.write(rec.tobytes())
        else:
            f.write("".join(" ".join(f"{v:.9g}" for v in r) + "\n" for r in rec).encode())


def test_pcd_io_round_trips_main_clouds(tmp_path):
    """pcl::io::loadPCDFile / savePCDFileASCII / savePCDFileBinary of the C++
    header (RealTimeRobot.cpp:34-35, 108-109) on main's two clouds, in both
    layouts the reference's files use: every coordinate read back exactly."""
    import sys
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import read_pcd
    demo = Path(__file__).resolve().parents[1] / "realtime_robot_gb300" / "realtime_robot_demo"
    if not demo.exists():
        pytest.skip("demo not built")
    d = np.load(Path(__file__).resolve().parent / "golden" / "main_clouds.npz")
    for name, binary, rgb in (("chair1", True, True), ("T0_m8111", False, False)):
        src = tmp_path / f"{name}.pcd"
        _write_pcd(src, d[name], binary, rgb)
        oa, ob = tmp_path / f"{name}_a.pcd", tmp_path / f"{name}_b.pcd"
        r = subprocess.run([str(demo), "pcd", str(src), str(oa), str(ob)], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        assert f"points {d[name].shape[0]}" in r.stdout
        for out in (oa, ob):
            back = read_pcd(out)
            assert np.array_equal(back[:, :3], d[name][:, :3]), (name, out)
    bad = tmp_path / "bad.pcd"
    bad.write_text("VERSION 0.7\nFIELDS a b\nSIZE 4 4\nTYPE F F\nCOUNT 1 1\nPOINTS 1\nDATA ascii\n1 2\n")
    r = subprocess.run([str(demo), "pcd", str(bad), str(tmp_path / "x.pcd"), str(tmp_path / "y.pcd")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 2


def test_corrupt_pcd_files_are_refused(tmp_path):
    """Corrupt PCD files make loadPCDFile return -1 (the demo exits 2 with a
    message), never crash or allocate from a corrupt header: truncated
    binary data, a POINTS count far beyond the file, truncated ascii rows,
    binary_compressed data, a missing DATA line, an empty file."""
    demo = Path(__file__).resolve().parents[1] / "realtime_robot_gb300" / "realtime_robot_demo"
    if not demo.exists():
        pytest.skip("demo not built")
    pts = np.arange(30, dtype=np.float32).reshape(10, 3)
    hdr = ("VERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\nCOUNT 1 1 1\nWIDTH {n}\nHEIGHT 1\n"
           "POINTS {n}\nDATA {d}\n")
    cases = {
        "truncated_binary": hdr.format(n=10, d="binary").encode() + pts.tobytes()[:100],
        "huge_points_binary": hdr.format(n=1 << 40, d="binary").encode() + pts.tobytes(),
        "huge_points_ascii": hdr.format(n=1 << 40, d="ascii").encode() + b"1 2 3\n",
        "truncated_ascii": hdr.format(n=10, d="ascii").encode() + b"1 2 3\n4 5\n",
        "compressed": hdr.format(n=10, d="binary_compressed").encode() + b"\x00" * 64,
        "no_data_line": b"VERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\nCOUNT 1 1 1\nPOINTS 1\n",
        "empty": b"",
    }
    for name, blob in cases.items():
        f = tmp_path / f"{name}.pcd"
        f.write_bytes(blob)
        r = subprocess.run([str(demo), "pcd", str(f), str(tmp_path / "a.pcd"), str(tmp_path / "b.pcd")],
                           capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and "cannot read" in r.stderr, (name, r.returncode, r.stderr)
    # the same header with its data intact reads
    ok = tmp_path / "ok.pcd"
    ok.write_bytes(hdr.format(n=10, d="binary").encode() + pts.tobytes())
    r = subprocess.run([str(demo), "pcd", str(ok), str(tmp_path / "a.pcd"), str(tmp_path / "b.pcd")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "points 10" in r.stdout


def test_host_only_generator_matches_the_library(rtr):
    """oracle/libsynth.so (the CPU baseline's input generator, built without
    CUDA from the same synth.cpp) gives the same clouds as librtr.so."""
    from oracle import synth as S
    a, sa, pa = rtr.synth_room(1)
    b, sb, pb = S.synth_room(1)
    assert np.array_equal(a, b) and np.array_equal(sa, sb) and np.array_equal(pa, pb)
    assert np.array_equal(rtr.synth_shape(rtr.CHAIR, 20000, 2024), S.synth_shape(S.CHAIR, 20000, 2024))
    for x, y in zip(rtr.config0_pair(2024, 5000), S.config0_pair(2024, 5000)):
        assert np.array_equal(x, y)
    crop = rtr.synth_crop(rtr.synth_shape(rtr.SOFA, 3000, 4), 0.4, 4)
    assert np.array_equal(crop, S.synth_crop(S.synth_shape(S.SOFA, 3000, 4), 0.4, 4))


def test_oracle_pipeline_defaults_equal_the_library_defaults(rtr):
    """The oracle pipeline and rtr_recog_default_params describe the same
    recognition (the GPU-vs-oracle pipeline tests rest on it)."""
    from oracle import pipeline as OP
    p = rtr.recog_default_params()
    for k, v in OP.DEFAULTS.items():
        got = getattr(p, k)
        if k == "viewpoint":
            assert list(got) == [float(np.float32(x)) for x in v], k
        elif isinstance(v, float):
            assert got == float(np.float32(v)), (k, got, v)
        else:
            assert got == v, (k, got, v)
    assert p.model_keypoint_r == np.float32(0.02) and p.scene_keypoint_r == np.float32(0.02)
