"""Generate the golden fixtures under tests/golden from the reference's own data.

Run in a checkout that has the reference mounted (it is read here only; the
fixtures it writes are committed and are all the tests need):

    python tests/golden/make_golden.py /path/to/RealTime_Robot

Fixtures:
  pcd_pairs.npz — the reference's recorded ICP known-answer pairs
    (RealTimeRobot/70761.pcd -> 70761_c.pcd, a translation by (+1, +0.5, 0)
    written by the synthetic-pair generator commented at function.h:131-143;
    RealTimeRobot/5.pcd -> mcloud.pcd, a translation by (+0.8, +0.8, 0), the
    keyPointICP input pair, function.h:111-127) and the recorded failure
    transformed_cloud.pcd (an uninitialised pose applied, function.h:39,108).
  main_clouds.npz — the two clouds main registers (RealTimeRobot.cpp:34-35):
    chair1.pcd, the model (1,818 points), and T0_m8111.pcd, the scan
    (3,218 points); the inputs of the reference's own descriptor route
    (occupancy grids, TDF, get_Distance, Ransac).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def read_pcd(path: Path) -> np.ndarray:
    """Minimal PCD v0.7 reader (ascii / binary, float fields) -> [n,4] float32 xyz0."""
    raw = path.read_bytes()
    hdr = {}
    pos = 0
    while True:
        end = raw.index(b"\n", pos)
        line = raw[pos:end].decode("ascii", "replace").strip()
        pos = end + 1
        if not line or line.startswith("#"):
            continue
        key, *vals = line.split()
        hdr[key.upper()] = vals
        if key.upper() == "DATA":
            break
    fields = hdr["FIELDS"]
    sizes = [int(s) for s in hdr["SIZE"]]
    types = hdr["TYPE"]
    counts = [int(c) for c in hdr.get("COUNT", ["1"] * len(fields))]
    n = int(hdr["POINTS"][0])
    mode = hdr["DATA"][0].lower()
    ix = [fields.index(a) for a in ("x", "y", "z")]
    out = np.zeros((n, 4), np.float32)
    if mode == "ascii":
        rows = raw[pos:].decode("ascii").split("\n")
        rows = [r for r in rows if r.strip()][:n]
        arr = np.array([[float(v) for v in r.split()] for r in rows], dtype=np.float64)
        col = np.cumsum([0] + counts)[:-1]
        for a, f in enumerate(ix):
            out[:, a] = arr[:, col[f]].astype(np.float32)
    elif mode == "binary":
        dt = []
        for f, s, t, c in zip(fields, sizes, types, counts):
            code = {"F": "f", "I": "i", "U": "u"}[t] + str(s)
            dt.append((f if f != "_" else f"pad{len(dt)}", "<" + code, (c,) if c > 1 else ()))
        rec = np.frombuffer(raw[pos:pos + n * sum(s * c for s, c in zip(sizes, counts))],
                            dtype=np.dtype(dt), count=n)
        for a, f in enumerate(("x", "y", "z")):
            out[:, a] = rec[f].astype(np.float32)
    else:
        raise ValueError(f"unsupported DATA {mode}")
    return out


def main(ref_root: str) -> None:
    d = Path(ref_root) / "RealTimeRobot"
    a, ac = read_pcd(d / "70761.pcd"), read_pcd(d / "70761_c.pcd")
    b, bm = read_pcd(d / "5.pcd"), read_pcd(d / "mcloud.pcd")
    bad = read_pcd(d / "transformed_cloud.pcd")
    t1 = (ac[:, :3].astype(np.float64) - a[:, :3]).mean(0)
    t2 = (bm[:, :3].astype(np.float64) - b[:, :3]).mean(0)
    r1 = np.abs(ac[:, :3] - a[:, :3] - t1).max()
    r2 = np.abs(bm[:, :3] - b[:, :3] - t2).max()
    print(f"70761 -> 70761_c: t = {t1}, max residual {r1:.2e}")
    print(f"5 -> mcloud: t = {t2}, max residual {r2:.2e}")
    np.savez_compressed(HERE / "pcd_pairs.npz", p70761=a, p70761_c=ac, p5=b, mcloud=bm,
                        t70761=np.array([1.0, 0.5, 0.0]), t5=np.array([0.8, 0.8, 0.0]),
                        transformed_cloud_head=bad[:16])
    chair, scan = read_pcd(d / "chair1.pcd"), read_pcd(d / "T0_m8111.pcd")
    print(f"chair1 {chair.shape[0]} points, T0_m8111 {scan.shape[0]} points")
    np.savez_compressed(HERE / "main_clouds.npz", chair1=chair, T0_m8111=scan)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the RealTime_Robot checkout>")
    main(sys.argv[1])
