"""CPU oracle (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package; the product (``realtime_robot_gb300``) never does.
It wraps ``liboracle.so`` (oracle.c, a plain-C restatement of the hot path)
and holds numpy restatements for the later stages.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
_lib = None

_P, _I, _F, _D = C.c_void_p, C.c_int, C.c_float, C.c_double


class IcpOut(C.Structure):
    _fields_ = [("pose", C.c_double * 16), ("fitness", C.c_double), ("iterations", C.c_int),
                ("converged", C.c_int), ("n_corr", C.c_int)]


_SIG = {
    "orc_num_threads": (_I, []),
    "orc_set_threads": (None, [_I]),
    "orc_nn1_brute": (None, [_P, _I, _P, _I, _F, _P, _P]),
    "orc_nn1_grid": (None, [_P, _I, _P, _I, _F, _F, _P, _P]),
    "orc_knn_brute": (None, [_P, _I, _P, _I, _I, _P, _P]),
    "orc_range_search": (None, [_P, _I, _P, _I, C.c_float, _I, _I, _P, _P]),
    "orc_transform_f32": (None, [_P, _P, _I, _P]),
    "orc_rigid_fit": (_I, [_P, _P, _P, _I, _P]),
    "orc_icp": (None, [_P, _I, _P, _I, _I, _F, _D, _D, _P, C.POINTER(IcpOut), _P, _P]),
    "orc_grid_create": (_P, [_P, _I, _F]),
    "orc_grid_destroy": (None, [_P]),
    "orc_grid_nn1": (None, [_P, _P, _I, _F, _P, _P]),
    "orc_grid_inlier_fraction": (None, [_P, _P, _I, _I, _P, _I, _F, _P]),
    "orc_grid_icp": (None, [_P, _P, _I, _I, _F, _D, _D, _P, C.POINTER(IcpOut)]),
    "orc_grid_icp_multi": (None, [_P, _P, _I, _I, _F, _P, _I, _P]),
    "orc_icp_replay": (None, [_P, _I, _P, _I, _F, _P, _I, _P, _P, _P]),
    "orc_tdf": (None, [_P, _I, _I, _P]),
    "orc_voxel_downsample": (_I, [_P, _I, _F, _P]),
    "orc_normals": (None, [_P, _I, _I, _P, _P]),
    "orc_eig3": (None, [_P, _P, _P]),
    "orc_uniform_sample": (_I, [_P, _I, _F, _P]),
    "orc_set_shot_flags": (None, [_I]),
    "orc_shot_atan2": (_F, [_F, _F]),
    "orc_shot352": (None, [_P, _P, _I, _P, _I, _F, _P, _P]),
    "orc_match": (None, [_P, _I, _P, _I, _I, _P, _P]),
    "orc_gc_group": (_I, [_P, _P, _P, _P, _P, _I, _F, _I, _I, _P, _P, _P]),
    "orc_orient_outward": (None, [_P, _P, _I, _F, _F, _F]),
    "orc_plane_segment": (_I, [_P, _I, _I, _F, _D, _D, C.c_uint64, _I, _P, _P]),
    "orc_vector3d": (None, [_P, _I, _P, _I, _P]),
    "orc_harris3d": (_I, [_P, _I, _F, _F, _I, _I, _P, _P]),
    "orc_ref_occupancy": (C.c_longlong, [_P, _I, _P, _I, _F, _F, _P, _P, _P, C.c_longlong]),
    "orc_ref_tdf": (_I, [_P, _P, _I, _P, _P, _F, _F, _P]),
    "orc_ref_distance": (None, [_P, _P, _P, _P, _P, _I, _P, _I, _P, _P, C.c_longlong, _F, _F, _I, _P, _P]),
    "orc_ref_gates": (_I, [_P, _I, _P, _P, _I, _P]),
    "orc_ref_correspond": (C.c_longlong, [_P, _P, _P, _I, _P, _P, _P, _I, _P, _F, _P, C.c_longlong]),
    "orc_ref_ransac": (_I, [_P, _P, _I, _P, _I, _P, _P, _F, _F, _P, _P]),
}


def orient_outward(pts, nrm, rc=0.01, gap=0.005, length=1.0) -> np.ndarray:
    pts = _f4(pts)
    out = np.array(nrm, dtype=np.float32, copy=True, order="C")
    lib().orc_orient_outward(pts.ctypes.data, out.ctypes.data, pts.shape[0], float(rc), float(gap),
                             float(length))
    return out


def build() -> Path:
    """Compile liboracle.so with the recipe in oracle/Makefile."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIG.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _f4(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != 4:
        raise ValueError("expected [n,4] float32 points")
    return a


def _r2(max_dist: float) -> float:
    return max_dist * max_dist if (max_dist and 0 < max_dist < 1e18) else float("inf")


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return lib().orc_num_threads()


def nn1(q, t, max_dist: float = 0.0, method: str = "grid", cell: float = 0.0):
    q, t = _f4(q), _f4(t)
    idx = np.empty(q.shape[0], np.int32)
    d2 = np.empty(q.shape[0], np.float32)
    if method == "brute":
        lib().orc_nn1_brute(q.ctypes.data, q.shape[0], t.ctypes.data, t.shape[0], _r2(max_dist),
                            idx.ctypes.data, d2.ctypes.data)
    else:
        lib().orc_nn1_grid(q.ctypes.data, q.shape[0], t.ctypes.data, t.shape[0], _r2(max_dist),
                           float(cell), idx.ctypes.data, d2.ctypes.data)
    return idx, d2


def knn(q, t, k: int):
    q, t = _f4(q), _f4(t)
    idx = np.empty((q.shape[0], k), np.int32)
    d2 = np.empty((q.shape[0], k), np.float32)
    lib().orc_knn_brute(q.ctypes.data, q.shape[0], t.ctypes.data, t.shape[0], int(k),
                        idx.ctypes.data, d2.ctypes.data)
    return idx, d2


def range_search(q, t, r: float, box: bool = False, max_per_query: int = 64):
    """Every target within r of each query (box: inside [q - r, q + r]), in
    ascending index: (idx [nq, max_per_query] with -1 past the count,
    count [nq]).  orc_range_search."""
    q, t = _f4(q), _f4(t)
    m = max(int(max_per_query), 0)
    idx = np.empty((q.shape[0], max(m, 1)), np.int32)
    cnt = np.empty(q.shape[0], np.int32)
    lib().orc_range_search(q.ctypes.data, q.shape[0], t.ctypes.data, t.shape[0], float(r), 1 if box else 0, m,
                           idx.ctypes.data, cnt.ctypes.data)
    return idx[:, :m], cnt


def transform_f32(T, pts) -> np.ndarray:
    pts = _f4(pts)
    Tc = np.ascontiguousarray(T, np.float64).reshape(16)
    out = np.empty_like(pts)
    lib().orc_transform_f32(Tc.ctypes.data, pts.ctypes.data, pts.shape[0], out.ctypes.data)
    return out


def rigid_fit(p, q, corr=None) -> tuple[np.ndarray, int]:
    p, q = _f4(p), _f4(q)
    T = np.empty(16, np.float64)
    c = None if corr is None else np.ascontiguousarray(corr, np.int32)
    m = lib().orc_rigid_fit(p.ctypes.data, q.ctypes.data, None if c is None else c.ctypes.data,
                            p.shape[0], T.ctypes.data)
    return T.reshape(4, 4), m


def icp(src, tgt, max_iterations=10, max_corr_dist=0.0, init=None, eps_t=0.0, eps_r=0.0,
        trace=False):
    src, tgt = _f4(src), _f4(tgt)
    out = IcpOut()
    ini = None if init is None else np.ascontiguousarray(init, np.float64).reshape(16)
    tp = np.zeros((max_iterations + 1, 16), np.float64) if trace else None
    tc = np.full((max_iterations, src.shape[0]), -2, np.int32) if trace else None
    lib().orc_icp(src.ctypes.data, src.shape[0], tgt.ctypes.data, tgt.shape[0], max_iterations,
                  float(max_corr_dist), eps_t, eps_r, None if ini is None else ini.ctypes.data,
                  C.byref(out), None if tp is None else tp.ctypes.data,
                  None if tc is None else tc.ctypes.data)
    res = {"pose": np.array(out.pose[:]).reshape(4, 4), "fitness": out.fitness,
           "iterations": out.iterations, "converged": out.converged, "n_corr": out.n_corr}
    if trace:
        res["trace_pose"] = tp
        res["trace_corr"] = tc
    return res


class Grid:
    """A target cloud's search grid kept across calls (exact searches: the
    results equal the one-shot nn1 / icp calls')."""

    def __init__(self, pts, cell: float = 0.0):
        self.pts = _f4(pts)
        self.h = lib().orc_grid_create(self.pts.ctypes.data, self.pts.shape[0], float(cell))

    def close(self):
        if self.h:
            lib().orc_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def nn1(self, q, max_dist: float = 0.0):
        q = _f4(q)
        idx = np.empty(q.shape[0], np.int32)
        d2 = np.empty(q.shape[0], np.float32)
        lib().orc_grid_nn1(self.h, q.ctypes.data, q.shape[0], _r2(max_dist), idx.ctypes.data, d2.ctypes.data)
        return idx, d2

    def inlier_fraction(self, src, stride: int, poses, r: float) -> np.ndarray:
        src = _f4(src)
        P = np.ascontiguousarray(poses, np.float64).reshape(-1, 16)
        out = np.zeros(P.shape[0], np.float64)
        lib().orc_grid_inlier_fraction(self.h, src.ctypes.data, src.shape[0], int(stride), P.ctypes.data,
                                       P.shape[0], float(r), out.ctypes.data)
        return out

    def icp(self, src, max_iterations=10, max_corr_dist=0.0, init=None) -> dict:
        src = _f4(src)
        out = IcpOut()
        ini = None if init is None else np.ascontiguousarray(init, np.float64).reshape(16)
        lib().orc_grid_icp(self.h, src.ctypes.data, src.shape[0], max_iterations, float(max_corr_dist), 0.0, 0.0,
                           None if ini is None else ini.ctypes.data, C.byref(out))
        return {"pose": np.array(out.pose[:]).reshape(4, 4), "fitness": out.fitness,
                "iterations": out.iterations, "converged": out.converged, "n_corr": out.n_corr}

    def icp_multi(self, src, max_iterations, max_corr_dist, inits) -> list[dict]:
        """Independent ICP problems from several initial poses, one per thread."""
        src = _f4(src)
        P = np.ascontiguousarray(inits, np.float64).reshape(-1, 16)
        outs = (IcpOut * max(1, P.shape[0]))()
        lib().orc_grid_icp_multi(self.h, src.ctypes.data, src.shape[0], int(max_iterations), float(max_corr_dist),
                                 P.ctypes.data, P.shape[0], outs)
        return [{"pose": np.array(o.pose[:]).reshape(4, 4), "fitness": o.fitness, "iterations": o.iterations,
                 "converged": o.converged, "n_corr": o.n_corr} for o in outs[: P.shape[0]]]


def icp_replay(src, tgt, max_corr_dist, poses_in):
    """Replay GPU iterations: poses_in[k] -> (corr[k], poses_out[k+1])."""
    src, tgt = _f4(src), _f4(tgt)
    poses_in = np.ascontiguousarray(poses_in, np.float64).reshape(-1, 16)
    iters = poses_in.shape[0] - 1
    corr = np.empty((iters, src.shape[0]), np.int32)
    pout = np.zeros((iters + 1, 16), np.float64)
    ncorr = np.zeros(iters, np.int32)
    lib().orc_icp_replay(src.ctypes.data, src.shape[0], tgt.ctypes.data, tgt.shape[0],
                         float(max_corr_dist), poses_in.ctypes.data, iters, corr.ctypes.data,
                         pout.ctypes.data, ncorr.ctypes.data)
    return corr, pout.reshape(-1, 4, 4), ncorr


def tdf(occ, dim: int) -> np.ndarray:
    occ = np.ascontiguousarray(occ, np.int32).reshape(-1, 3)
    out = np.empty(dim ** 3, np.float32)
    lib().orc_tdf(occ.ctypes.data if occ.size else None, occ.shape[0], int(dim), out.ctypes.data)
    return out


def voxel_downsample(pts, leaf: float) -> np.ndarray:
    pts = _f4(pts)
    out = np.empty_like(pts)
    v = lib().orc_voxel_downsample(pts.ctypes.data, pts.shape[0], float(leaf), out.ctypes.data)
    if v < 0:
        raise ValueError("voxel key space exceeds 32 bits")
    return out[:v].copy()


def normals(pts, k: int = 10, vp=(0.0, 0.0, 0.0)) -> np.ndarray:
    pts = _f4(pts)
    out = np.empty_like(pts)
    v = np.ascontiguousarray(vp, np.float32)
    lib().orc_normals(pts.ctypes.data, pts.shape[0], int(k), v.ctypes.data, out.ctypes.data)
    return out


def eig3(A) -> tuple[np.ndarray, np.ndarray]:
    A = np.ascontiguousarray(A, np.float32).reshape(9)
    w = np.empty(3, np.float32)
    V = np.empty(9, np.float32)
    lib().orc_eig3(A.ctypes.data, w.ctypes.data, V.ctypes.data)
    return w, V.reshape(3, 3)


def uniform_sample(pts, r: float) -> np.ndarray:
    pts = _f4(pts)
    out = np.empty(pts.shape[0], np.int32)
    k = lib().orc_uniform_sample(pts.ctypes.data, pts.shape[0], float(r), out.ctypes.data)
    if k < 0:
        raise ValueError("voxel key space exceeds 32 bits")
    return out[:k].copy()


def set_shot_flags(flags: int) -> None:
    """Probe switches of the SHOT conventions (0 = the GPU path's): bit 0
    keeps support points whose normals face away, bit 1 signs the LRF z axis
    by the majority rule over the support's offsets."""
    lib().orc_set_shot_flags(int(flags))


def shot_atan2(y: float, x: float) -> float:
    """The atan2 that SHOT's angle bins use (own restatement, see oracle.c)."""
    return float(lib().orc_shot_atan2(float(y), float(x)))


def shot352(pts, nrm, keys, radius: float):
    pts, nrm = _f4(pts), _f4(nrm)
    keys = np.ascontiguousarray(keys, np.int32)
    desc = np.zeros((keys.shape[0], 352), np.float32)
    lrf = np.zeros((keys.shape[0], 9), np.float32)
    lib().orc_shot352(pts.ctypes.data, nrm.ctypes.data, pts.shape[0], keys.ctypes.data,
                      keys.shape[0], float(radius), desc.ctypes.data, lrf.ctypes.data)
    return desc, lrf


def match(q, db):
    q = np.ascontiguousarray(q, np.float32)
    db = np.ascontiguousarray(db, np.float32)
    idx = np.empty(q.shape[0], np.int32)
    d2 = np.empty(q.shape[0], np.float32)
    lib().orc_match(q.ctypes.data, q.shape[0], db.ctypes.data, db.shape[0], q.shape[1],
                    idx.ctypes.data, d2.ctypes.data)
    return idx, d2


def gc_group(model_kp, scene_kp, corr_m, corr_s, corr_d, gc_size=0.01, gc_thresh=5,
             max_clusters=64):
    mk, sk = _f4(model_kp), _f4(scene_kp)
    cm = np.ascontiguousarray(corr_m, np.int32)
    cs = np.ascontiguousarray(corr_s, np.int32)
    cd = np.ascontiguousarray(corr_d, np.float32)
    nc = cm.shape[0]
    clus = np.empty(nc, np.int32)
    poses = np.zeros((max_clusters, 16), np.float64)
    sizes = np.zeros(max_clusters, np.int32)
    n = lib().orc_gc_group(mk.ctypes.data, sk.ctypes.data, cm.ctypes.data, cs.ctypes.data,
                           cd.ctypes.data, nc, float(gc_size), int(gc_thresh), max_clusters,
                           clus.ctypes.data, poses.ctypes.data, sizes.ctypes.data)
    return clus, poses[:n].reshape(n, 4, 4), sizes[:n]


def harris3d(pts, radius: float = 0.05, threshold: float = 0.01, non_max: bool = True, refine: bool = True):
    """Harris3D keypoints restated (harris.c): (keys [K, 4] = x, y, z,
    response; point index [K])."""
    pts = _f4(pts)
    n = pts.shape[0]
    keys = np.zeros((max(n, 1), 4), np.float32)
    src = np.zeros(max(n, 1), np.int32)
    k = lib().orc_harris3d(pts.ctypes.data, n, float(radius), float(threshold), int(bool(non_max)),
                           int(bool(refine)), keys.ctypes.data, src.ctypes.data)
    return keys[:k].copy(), src[:k].copy()


class Surface(C.Structure):
    _fields_ = [("area", C.c_double), ("perimeter", C.c_double), ("coeffs", C.c_float * 4),
                ("is_vertical", C.c_int), ("kept", C.c_int), ("n_inliers", C.c_int), ("hull_vertices", C.c_int),
                ("flat", C.c_int), ("pad", C.c_int)]


def plane_segment(pts, max_iterations: int = 150, distance: float = 0.005, remain_frac: float = 0.15,
                  min_area: float = 0.16, seed: int = 0, max_planes: int = 64):
    """ModelPoint::getArea / ScanPoint::get_Area restated (planes.c): the
    extracted planes in order (kept or not) as Surface records, and the
    number extracted (more than max_planes means some were not stored)."""
    pts = _f4(pts)
    out = (Surface * max_planes)()
    tot = C.c_int(0)
    n = lib().orc_plane_segment(pts.ctypes.data, pts.shape[0], int(max_iterations), float(distance),
                                float(remain_frac), float(min_area), int(seed), int(max_planes), out,
                                C.byref(tot))
    return list(out[:n]), tot.value


def vector3d(keys, surfaces) -> np.ndarray:
    """KeyPoint::get_Vector3D for every keypoint over the surfaces' kept
    ones: [nk, 3] float64."""
    keys = _f4(keys)
    arr = (Surface * max(1, len(surfaces)))()
    for i, x in enumerate(surfaces):  # any record with this layout (the GPU path's too)
        C.memmove(C.byref(arr[i]), C.byref(x), C.sizeof(Surface))
    v = np.zeros((keys.shape[0], 3), np.float64)
    lib().orc_vector3d(keys.ctypes.data, keys.shape[0], arr, len(surfaces), v.ctypes.data)
    return v


def pose_error(Ta, Tb) -> tuple[float, float]:
    """(translation error m, rotation error rad) between two 4x4 poses."""
    Ta, Tb = np.asarray(Ta, np.float64), np.asarray(Tb, np.float64)
    dt = float(np.linalg.norm(Ta[:3, 3] - Tb[:3, 3]))
    Rd = Ta[:3, :3] @ Tb[:3, :3].T
    c = np.clip((np.trace(Rd) - 1.0) / 2.0, -1.0, 1.0)
    # accurate for small angles: use the skew part
    s = 0.5 * np.linalg.norm([Rd[2, 1] - Rd[1, 2], Rd[0, 2] - Rd[2, 0], Rd[1, 0] - Rd[0, 1]])
    return dt, float(np.arctan2(s, c))


# ---- the reference's own descriptor route (refmatch.c) ---------------------
def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def ref_occupancy(cloud, keys, res: float = 0.01, half: float = 0.1):
    """KeyPoint::getOccupiedGrid for every keypoint: (number, offsets,
    indices), the box's points in ascending index order."""
    cloud, keys = _f4(cloud), _f4(keys)
    nk = keys.shape[0]
    number = np.zeros(nk, np.int32)
    offsets = np.zeros(nk + 1, np.int32)
    total = lib().orc_ref_occupancy(_ptr(cloud), cloud.shape[0], _ptr(keys), nk, float(res), float(half),
                                    _ptr(number), offsets.ctypes.data, None, 0)
    indices = np.zeros(max(total, 1), np.int32)
    lib().orc_ref_occupancy(_ptr(cloud), cloud.shape[0], _ptr(keys), nk, float(res), float(half), _ptr(number),
                            offsets.ctypes.data, indices.ctypes.data, total)
    return number, offsets, indices[:total]


def ref_tdf(cloud, keys, offsets, indices, res: float = 0.01, half: float = 0.15) -> np.ndarray:
    """KeyPoint::get_TSDF for every keypoint: [nk, dim^3] float32."""
    cloud, keys, offsets, indices = _f4(cloud), _f4(keys), _i32(offsets), _i32(indices)
    dim = int(np.float32(np.float32(half) / np.float32(res)) * np.float32(2))
    out = np.zeros((keys.shape[0], dim ** 3), np.float32)
    got = lib().orc_ref_tdf(_ptr(cloud), _ptr(keys), keys.shape[0], offsets.ctypes.data, _ptr(indices), float(res),
                            float(half), _ptr(out))
    if got != dim:
        raise ValueError(f"dim {got} (expected {dim})")
    return out


def ref_distance(mcloud, mkeys, moff, midx, mtdf, skeys, pair_m=None, pair_s=None, res: float = 0.01,
                 half: float = 0.15, float_order: bool = True):
    """get_Distance for pairs (all model x scan pairs, model-major, when
    pair_m is None): (score [P] float32, T [P, 4, 4] float32).  float_order
    (default): the reference's float running sum, leaf by leaf in tree order;
    False: exact integer sums per rotation with a double running score (a
    variant kept to measure the difference)."""
    mcloud, mkeys, skeys = _f4(mcloud), _f4(mkeys), _f4(skeys)
    moff, midx = _i32(moff), _i32(midx)
    mtdf = np.ascontiguousarray(mtdf, np.float32)
    nm, ns = mkeys.shape[0], skeys.shape[0]
    if pair_m is None:
        pm = ps = None
        P = nm * ns
    else:
        pm, ps = _i32(pair_m), _i32(pair_s)
        P = pm.shape[0]
    score = np.zeros(P, np.float32)
    T = np.zeros((P, 4, 4), np.float32)
    lib().orc_ref_distance(_ptr(mcloud), _ptr(mkeys), moff.ctypes.data, _ptr(midx), _ptr(mtdf), nm, _ptr(skeys), ns,
                           _ptr(pm), _ptr(ps), P, float(res), float(half), int(bool(float_order)), _ptr(score),
                           _ptr(T))
    return score, T


def ref_correspond(mkeys, mnum, skeys, snum, score_all, max_score: float = 3.0, mv3=None, sv3=None) -> np.ndarray:
    """The all-pairs loop with its gates: indices p = m * ns + s of the kept
    pairs, ascending."""
    mkeys, skeys = _f4(mkeys), _f4(skeys)
    mnum, snum = _i32(mnum), _i32(snum)
    score_all = np.ascontiguousarray(score_all, np.float32)
    mv3 = None if mv3 is None else np.ascontiguousarray(mv3, np.float64)
    sv3 = None if sv3 is None else np.ascontiguousarray(sv3, np.float64)
    nm, ns = mkeys.shape[0], skeys.shape[0]
    args = (_ptr(mkeys), _ptr(mnum), _ptr(mv3), nm, _ptr(skeys), _ptr(snum), _ptr(sv3), ns, _ptr(score_all),
            float(max_score))
    c = lib().orc_ref_correspond(*args, None, 0)
    out = np.zeros(max(c, 1), np.int32)
    lib().orc_ref_correspond(*args, out.ctypes.data, c)
    return out[:c]


def ref_ransac(mkeys, skeys, pair_idx, score_all, T_all, inlier: float = 0.15, max_des: float = 100.0):
    """Ransac over the kept pairs: (T [4, 4] float32, inliers, position of
    the winner in pair_idx or -1)."""
    mkeys, skeys, pair_idx = _f4(mkeys), _f4(skeys), _i32(pair_idx)
    score_all = np.ascontiguousarray(score_all, np.float32)
    T_all = np.ascontiguousarray(T_all, np.float32)
    T = np.zeros((4, 4), np.float32)
    inl = np.zeros(1, np.int32)
    best = lib().orc_ref_ransac(_ptr(mkeys), _ptr(skeys), skeys.shape[0], _ptr(pair_idx), pair_idx.shape[0],
                                _ptr(score_all), _ptr(T_all), float(inlier), float(max_des), T.ctypes.data,
                                inl.ctypes.data)
    return T, int(inl[0]), int(best)
