"""realtime_robot_gb300 — Python host mirror of the rtr C ABI (include/rtr.h).

The compute path is ``librtr.so`` (hand-written sm_103a CUDA kernels).  This
module only loads it with ctypes, passes device pointers of torch tensors and
turns status codes into exceptions.  There is no CPU fallback: every call that
computes raises ``RtrError`` when the library or the GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import weakref

import numpy as np

__all__ = ["lib", "RtrError", "Context", "IcpParams", "IcpResult", "RoomParams", "LIB_PATH"]

LIB_PATH = Path(__file__).resolve().parent / "librtr.so"
_lib = None


class RtrError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{_status_name(status)}: {msg}")
        self.status = status


_STATUS = {0: "RTR_OK", 1: "RTR_ERR_INVALID_ARG", 2: "RTR_ERR_OOM", 3: "RTR_ERR_TIMEOUT",
           4: "RTR_ERR_NOT_FOUND", 5: "RTR_ERR_CUDA", 6: "RTR_ERR_CAPACITY", 7: "RTR_ERR_NO_DEVICE"}


def _status_name(s: int) -> str:
    return _STATUS.get(s, f"status {s}")


class IcpParams(C.Structure):
    _fields_ = [("max_iterations", C.c_int), ("max_corr_dist", C.c_float),
                ("transformation_epsilon", C.c_double), ("rotation_epsilon", C.c_double),
                ("cell_size", C.c_float), ("record_trace", C.c_int)]


class IcpResult(C.Structure):
    _fields_ = [("pose", C.c_double * 16), ("fitness", C.c_double), ("iterations", C.c_int),
                ("converged", C.c_int), ("n_corr", C.c_int), ("status", C.c_int)]


class RoomParams(C.Structure):
    _fields_ = [("n_points", C.c_int), ("n_chairs", C.c_int), ("n_desks", C.c_int),
                ("n_sofas", C.c_int), ("sigma", C.c_double), ("cam", C.c_double * 3),
                ("look_at", C.c_double * 3), ("width", C.c_int), ("height", C.c_int),
                ("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double), ("cy", C.c_double)]


MAX_INSTANCES = 16
KNN1_STATIC_MAX_TARGET = 65536  # RTR_KNN1_STATIC_MAX_TARGET


class HarrisParams(C.Structure):
    _fields_ = [("radius", C.c_float), ("threshold", C.c_float), ("non_max", C.c_int), ("refine", C.c_int)]


def harris_default_params(**kw) -> HarrisParams:
    p = HarrisParams()
    lib().rtr_harris_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class PlaneParams(C.Structure):
    _fields_ = [("max_iterations", C.c_int), ("distance", C.c_float), ("remain_frac", C.c_double),
                ("min_area", C.c_double), ("seed", C.c_uint64)]


class Surface(C.Structure):
    """rtr_surface: one extracted plane (area and perimeter of its hull in
    the plane, unit-normal coefficients, class, kept flag)."""
    _fields_ = [("area", C.c_double), ("perimeter", C.c_double), ("coeffs", C.c_float * 4),
                ("is_vertical", C.c_int), ("kept", C.c_int), ("n_inliers", C.c_int), ("hull_vertices", C.c_int),
                ("flat", C.c_int), ("pad", C.c_int)]


def plane_default_params(**kw) -> PlaneParams:
    p = PlaneParams()
    lib().rtr_plane_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class RecogParams(C.Structure):
    _fields_ = [("voxel_leaf", C.c_float), ("normal_k", C.c_int), ("scene_keypoint_r", C.c_float),
                ("model_keypoint_r", C.c_float), ("descriptor_r", C.c_float),
                ("match_max_d2", C.c_float), ("gc_size", C.c_float), ("gc_thresh", C.c_int),
                ("max_clusters", C.c_int), ("hv_inlier_r", C.c_float), ("hv_subsample", C.c_int),
                ("refine_top", C.c_int), ("icp_iterations", C.c_int), ("icp_max_dist", C.c_float),
                ("accept_inlier_r", C.c_float), ("accept_score", C.c_float), ("nms_dist", C.c_float),
                ("max_instances", C.c_int), ("viewpoint", C.c_float * 3),
                ("keypoint_min_curvature", C.c_float), ("scene_outward", C.c_int)]


class Instance(C.Structure):
    _fields_ = [("pose", C.c_double * 16), ("score", C.c_float), ("hypothesis", C.c_int),
                ("cluster_size", C.c_int), ("pad", C.c_int)]


class RecogResult(C.Structure):
    _fields_ = [("n_instances", C.c_int), ("n_voxels", C.c_int), ("n_keypoints", C.c_int),
                ("n_correspondences", C.c_int), ("n_clusters", C.c_int), ("status", C.c_int),
                ("pad", C.c_int * 2), ("inst", Instance * MAX_INSTANCES)]


def recog_default_params(**kw) -> RecogParams:
    p = RecogParams()
    lib().rtr_recog_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "viewpoint":
            p.viewpoint[:] = list(v)
        else:
            setattr(p, k, v)
    return p


def parse_recog_result(raw) -> dict:
    if not isinstance(raw, (bytes, bytearray)):
        raw = bytes(raw.cpu().numpy().tobytes())
    r = RecogResult.from_buffer_copy(raw[: C.sizeof(RecogResult)])
    inst = []
    for i in range(r.n_instances):
        I = r.inst[i]
        inst.append({"pose": np.array(I.pose[:]).reshape(4, 4), "score": I.score,
                     "hypothesis": I.hypothesis, "cluster_size": I.cluster_size})
    return {"instances": inst, "n_voxels": r.n_voxels, "n_keypoints": r.n_keypoints,
            "n_correspondences": r.n_correspondences, "n_clusters": r.n_clusters,
            "status": r.status}


_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_D = C.c_double
_U64 = C.c_uint64
_SIG = {
    "rtr_status_string": (C.c_char_p, [_I]),
    "rtr_last_error": (C.c_char_p, []),
    "rtr_version": (C.c_char_p, []),
    "rtr_context_create": (_I, [_I, C.POINTER(_P)]),
    "rtr_context_destroy": (_I, [_P]),
    "rtr_context_reserve": (_I, [_P, C.c_size_t]),
    "rtr_context_scratch_bytes": (C.c_size_t, [_P]),
    "rtr_context_set_wait_budget_ms": (_I, [_P, _D]),
    "rtr_context_check": (_I, [_P, _P]),
    "rtr_context_set_tuning": (_I, [_P, C.c_char_p, _I]),
    "rtr_context_get_tuning": (_I, [_P, C.c_char_p, C.POINTER(C.c_int)]),
    "rtr_context_set_profiling": (_I, [_P, _I]),
    "rtr_context_profile_count": (_I, [_P]),
    "rtr_context_profile_get": (_I, [_P, _I, C.POINTER(C.c_char_p), C.POINTER(C.c_float)]),
    "rtr_context_profile_clear": (None, [_P]),
    "rtr_launch_count": (C.c_uint64, []),
    "ComputeTDFWithCuda": (_I, [_P, _P, _I, _I]),
    "rtr_tdf_batch": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "rtr_ref_occupancy": (_I, [_P, _P, _I, _P, _I, _F, _F, _P, _P, _P, C.c_longlong, C.POINTER(C.c_longlong), _P]),
    "rtr_ref_tdf": (_I, [_P, _P, _P, _I, _P, _P, _F, _F, _P, C.POINTER(C.c_int), _P]),
    "rtr_ref_distance": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _I, _P, _P, C.c_longlong, _F, _F, _P, _P, _P]),
    "rtr_ref_correspond": (_I, [_P, _P, _P, _P, _I, _P, _P, _P, _I, _P, _F, _P, _I, C.POINTER(C.c_int), _P]),
    "rtr_ref_ransac": (_I, [_P, _P, _I, _P, _I, _P, _I, _P, _P, _F, _F, _P, C.POINTER(C.c_int),
                            C.POINTER(C.c_int), _P]),
    "rtr_knn1": (_I, [_P, _P, _I, _P, _I, _F, _P, _P, _P]),
    "rtr_knn1_static": (_I, [_P, _I, _P, _I, _F, _P, _P, _P]),
    "rtr_harris_default_params": (None, [C.c_void_p]),
    "rtr_harris3d": (_I, [_P, _P, _I, C.c_void_p, _P, _P, _P, _P]),
    "rtr_plane_default_params": (None, [C.c_void_p]),
    "rtr_plane_segment": (_I, [_P, _P, _I, C.c_void_p, C.c_void_p, _I, C.POINTER(C.c_int), _P]),
    "rtr_vector3d": (_I, [_P, _P, _I, C.c_void_p, _I, _P, _P]),
    "rtr_knn": (_I, [_P, _P, _I, _P, _I, _I, _P, _P, _P]),
    "rtr_radius_search": (_I, [_P, _P, _I, _P, _I, C.c_float, _I, _P, _P, _P]),
    "rtr_box_search": (_I, [_P, _P, _I, _P, _I, C.c_float, _I, _P, _P, _P]),
    "rtr_icp_default_params": (None, [C.POINTER(IcpParams)]),
    "rtr_icp": (_I, [_P, _P, _I, _P, _I, C.POINTER(IcpParams), _P, _P, _P, _P, _P]),
    "rtr_icp_host": (_I, [_P, _P, _I, _P, _I, C.POINTER(IcpParams), _P, C.POINTER(IcpResult)]),
    "rtr_icp_multi": (_I, [_P, _P, _I, _P, _I, C.POINTER(IcpParams), _P, _I, _P, _P]),
    "rtr_pose_inliers": (_I, [_P, _P, _I, _P, _I, _P, _I, C.c_float, _P, _P]),
    "rtr_voxel_downsample": (_I, [_P, _P, _I, _F, _P, _P, _P]),
    "rtr_uniform_sample": (_I, [_P, _P, _I, _F, _P, _P, _P]),
    "rtr_normals": (_I, [_P, _P, _I, _I, _P, _F, _P, _P]),
    "rtr_orient_normals_outward": (_I, [_P, _P, _P, _I, _F, _F, _F, _P]),
    "rtr_shot352": (_I, [_P, _P, _P, _I, _P, _I, _F, _P, _P, _P]),
    "rtr_match_exact": (_I, [_P, _P, _I, _P, _I, _P, _P, _P]),
    "rtr_match": (_I, [_P, _P, _I, _P, _I, _P, _P, _P]),
    "rtr_match_stats": (_I, [_P, C.POINTER(C.c_int)]),
    "rtr_icp_stats": (_I, [_P, _P]),
    "rtr_match_stats_ex": (_I, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "rtr_gc_group": (_I, [_P, _P, _P, _P, _P, _P, _I, _F, _I, _I, _I, _P, _P, _P,
                          C.POINTER(C.c_int), _P]),
    "rtr_gc_stats": (_I, [_P, C.POINTER(C.c_int * 8)]),
    "rtr_mlp_create": (_I, [_P, _P, _U64, C.POINTER(_P)]),
    "rtr_mlp_destroy": (_I, [_P]),
    "rtr_mlp_get_params": (_I, [_P, _P]),
    "rtr_mlp_set_params": (_I, [_P, _P]),
    "rtr_mlp_score": (_I, [_P, _P, _P, _I, _P, _P]),
    "rtr_mlp_loss_grad": (_I, [_P, _P, _P, _P, _I, _P, _P, _P]),
    "rtr_mlp_train_step": (_I, [_P, _P, _P, _P, _I, _F, _P, _P]),
    "rtr_mlp_train": (_I, [_P, _P, _P, _P, _I, _I, _I, _F, _U64, _P]),
    "rtr_recog_default_params": (None, [C.POINTER(RecogParams)]),
    "rtr_model_create": (_I, [_P, _P, _I, C.POINTER(RecogParams), C.POINTER(_P)]),
    "rtr_model_destroy": (_I, [_P]),
    "rtr_model_info": (_I, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "rtr_model_buffers": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
                               C.POINTER(_P)]),
    "rtr_recognize": (_I, [_P, _P, _P, _I, C.POINTER(RecogParams), _P, _P]),
    "rtr_recognize_learned": (_I, [_P, _P, _P, _F, _P, _I, C.POINTER(RecogParams), _P, _P]),
    "rtr_recognize_multi": (_I, [_P, _P, _I, _P, _F, _P, _I, C.POINTER(RecogParams), _P, _P]),
    "rtr_recognize_batch": (_I, [_P, _P, _I, C.POINTER(RecogParams), _P, _F, _P]),
    "rtr_batch_graph_create": (_I, [_P, _P, _I, C.POINTER(RecogParams), _P, _F, _P, C.POINTER(_P)]),
    "rtr_batch_graph_launch": (_I, [_P, _P]),
    "rtr_batch_graph_destroy": (_I, [_P]),
    "rtr_batch_autotune": (_I, [_P, _P, _I, C.POINTER(RecogParams), _P, _F, _P, C.POINTER(C.c_int),
                                C.POINTER(C.c_int)]),
    "rtr_recognize_host": (_I, [_P, _P, _P, _I, C.POINTER(RecogParams), C.POINTER(RecogResult)]),
    "rtr_synth_shape": (_I, [_I, _U64, _I, _P]),
    "rtr_synth_rigid": (None, [_U64, _D, _D, _P]),
    "rtr_synth_transform_noise": (None, [_P, _I, _P, _D, _U64, _P]),
    "rtr_synth_crop": (_I, [_P, _I, _D, _U64, _P]),
    "rtr_room_default_params": (None, [C.POINTER(RoomParams)]),
    "rtr_synth_room_boxes": (_I, [C.POINTER(RoomParams), _U64, _P, _I, C.POINTER(C.c_int), _P, _P, _I,
                                  C.POINTER(C.c_int)]),
    "rtr_synth_trajectory": (None, [_U64, _I, _D, _P]),
    "rtr_synth_depth_frames": (_I, [_P, _P, _I, _P, _I, _I, _I, _F, _F, _F, _F, _F, _U64, _P, _P]),
    "rtr_depth_to_points": (_I, [_P, _P, _I, _I, _F, _F, _F, _F, _P, _F, _F, _P, _P, _P]),
    "rtr_map_create": (_I, [_P, _I, _F, C.POINTER(_P)]),
    "rtr_map_destroy": (_I, [_P]),
    "rtr_map_clear": (_I, [_P, _P]),
    "rtr_map_integrate": (_I, [_P, _P, _I, _P, _P]),
    "rtr_map_extract": (_I, [_P, _P, _P, _I, C.POINTER(C.c_int)]),
    "rtr_synth_room": (_I, [C.POINTER(RoomParams), _U64, _P, _I, _P, _P, _P]),
}


def lib():
    """Load librtr.so (built by ``__graft_entry__.build()``); raises if absent."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RtrError(5, f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIG.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def declared_symbols() -> list[str]:
    return list(_SIG)


def launch_count() -> int:
    """Kernels launched by librtr.so in this process so far."""
    return int(lib().rtr_launch_count())


def check(st: int) -> None:
    if st != 0:
        raise RtrError(st, lib().rtr_last_error().decode(errors="replace"))


def _ptr(t) -> int:
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(stream)


class Context:
    """Owns an rtr_context (scratch arena + status words) on one device."""

    def __init__(self, device: int = 0):
        h = _P()
        check(lib().rtr_context_create(device, C.byref(h)))
        self.h = h
        self.device = device
        self._graphs = weakref.WeakSet()  # batch graphs, destroyed before the context

    def close(self):
        if self.h:
            for g in list(self._graphs):
                g.close()
            lib().rtr_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, nbytes: int):
        check(lib().rtr_context_reserve(self.h, nbytes))

    def scratch_bytes(self) -> int:
        return lib().rtr_context_scratch_bytes(self.h)

    def set_wait_budget_ms(self, ms: float):
        check(lib().rtr_context_set_wait_budget_ms(self.h, ms))

    def get_tuning(self, key: str) -> int:
        v = C.c_int(0)
        check(lib().rtr_context_get_tuning(self.h, key.encode(), C.byref(v)))
        return v.value

    def set_tuning(self, key: str, value: int):
        check(lib().rtr_context_set_tuning(self.h, key.encode(), int(value)))

    def check(self, stream=None):
        check(lib().rtr_context_check(self.h, _stream(stream)))

    def set_profiling(self, on: bool):
        check(lib().rtr_context_set_profiling(self.h, 1 if on else 0))

    def profile(self, clear: bool = True) -> list[tuple[str, float]]:
        """Recorded stages [(name, ms)] since the last clear (synchronises)."""
        out = []
        for i in range(lib().rtr_context_profile_count(self.h)):
            nm, ms = C.c_char_p(), C.c_float()
            check(lib().rtr_context_profile_get(self.h, i, C.byref(nm), C.byref(ms)))
            out.append((nm.value.decode(), ms.value))
        if clear:
            lib().rtr_context_profile_clear(self.h)
        return out

    # -- searches -----------------------------------------------------------
    def knn1(self, query, target, max_dist: float = 0.0, stream=None):
        import torch
        nq, nt = query.shape[0], target.shape[0]
        idx = torch.empty(nq, dtype=torch.int32, device=query.device)
        d2 = torch.empty(nq, dtype=torch.float32, device=query.device)
        check(lib().rtr_knn1(self.h, _ptr(query), nq, _ptr(target), nt, float(max_dist),
                             _ptr(idx), _ptr(d2), _stream(stream)))
        return idx, d2

    def radius_search(self, query, target, radius: float, max_per_query: int = 64, box: bool = False,
                      stream=None):
        """rtr_radius_search (box=True: rtr_box_search with half extent
        `radius`): (idx int32 [nq, max_per_query], ascending, -1 past the
        count; count int32 [nq], the true count)."""
        import torch
        nq, nt = query.shape[0], target.shape[0]
        m = int(max_per_query)
        idx = torch.empty((nq, max(m, 1)), dtype=torch.int32, device=query.device)
        cnt = torch.empty(nq, dtype=torch.int32, device=query.device)
        fn = lib().rtr_box_search if box else lib().rtr_radius_search
        check(fn(self.h, _ptr(query), nq, _ptr(target), nt, float(radius), m, _ptr(idx) if m > 0 else None,
                 _ptr(cnt), _stream(stream)))
        return idx[:, :m], cnt

    def knn1_static(self, query, target, max_dist: float = 0.0, out=None, stream=None):
        """rtr_knn1_static: rtr_knn1 with its grid in the library's fixed
        device array (no allocation inside the call; n_target at most
        KNN1_STATIC_MAX_TARGET).  `out` = (idx int32 [nq], d2 float32 [nq])
        preallocated by the caller; allocated here when omitted."""
        import torch
        nq, nt = query.shape[0], target.shape[0]
        for t in (target,) + (tuple(out) if out is not None else ()):
            if t.device != query.device:
                raise ValueError("knn1_static: query, target and outputs must be on one device")
        if out is None:
            out = (torch.empty(nq, dtype=torch.int32, device=query.device),
                   torch.empty(nq, dtype=torch.float32, device=query.device))
        idx, d2 = out
        # the entry point runs on the calling thread's current device
        with torch.cuda.device(query.device):
            check(lib().rtr_knn1_static(_ptr(query), nq, _ptr(target), nt, float(max_dist),
                                        _ptr(idx), _ptr(d2), _stream(stream)))
        return idx, d2

    def synth_depth_frames(self, boxes: np.ndarray, poses: np.ndarray, width=640, height=480, fx=525.0, fy=525.0,
                           cx=319.5, cy=239.5, noise_k=0.0015, seed=0, stream=None):
        """Ray-cast depth frames [n_frames, height, width] (device) of the room
        boxes from camera->world poses [n_frames, 4, 4]."""
        import torch
        boxes = np.ascontiguousarray(boxes, np.float32).reshape(-1, 12)
        poses = np.ascontiguousarray(poses, np.float64).reshape(-1, 16)
        out = torch.empty((poses.shape[0], height, width), dtype=torch.float32, device="cuda")
        check(lib().rtr_synth_depth_frames(self.h, boxes.ctypes.data, boxes.shape[0], poses.ctypes.data,
                                           poses.shape[0], width, height, fx, fy, cx, cy, noise_k, seed,
                                           _ptr(out), _stream(stream)))
        return out

    def depth_to_points(self, depth, fx=525.0, fy=525.0, cx=319.5, cy=239.5, pose=None, min_z=0.05, max_z=8.0,
                        out=None, count=None, stream=None):
        """World points [k, 4] of one depth frame [height, width] (device)."""
        import torch
        h, w = depth.shape
        if out is None:
            out = torch.empty((h * w, 4), dtype=torch.float32, device=depth.device)
        if count is None:
            count = torch.zeros(1, dtype=torch.int32, device=depth.device)
        P = None if pose is None else np.ascontiguousarray(pose, np.float64).reshape(16)
        check(lib().rtr_depth_to_points(self.h, _ptr(depth), w, h, fx, fy, cx, cy,
                                        None if P is None else P.ctypes.data, min_z, max_z, _ptr(out),
                                        _ptr(count), _stream(stream)))
        return out, count

    def harris3d(self, pts, params: HarrisParams | None = None, stream=None):
        """rtr_harris3d (the detector of ModelPoint / ScanPoint::getKeypoint):
        (keys [K, 4] = x, y, z, response; point indices [K]) on the device."""
        import torch
        p = params or harris_default_params()
        n = pts.shape[0]
        keys = torch.empty((max(n, 1), 4), dtype=torch.float32, device=pts.device)
        src = torch.empty(max(n, 1), dtype=torch.int32, device=pts.device)
        cnt = torch.zeros(1, dtype=torch.int32, device=pts.device)
        check(lib().rtr_harris3d(self.h, _ptr(pts), n, C.byref(p), _ptr(keys), _ptr(src), _ptr(cnt), _stream(stream)))
        k = int(cnt.item())
        return keys[:k], src[:k]

    def plane_segment(self, pts, params: PlaneParams | None = None, max_surfaces: int = 64, stream=None):
        """rtr_plane_segment (ModelPoint::getArea / ScanPoint::get_Area):
        the extracted planes, kept or not, as a list of Surface records."""
        p = params or plane_default_params()
        out = (Surface * max_surfaces)()
        n = C.c_int(0)
        check(lib().rtr_plane_segment(self.h, _ptr(pts), pts.shape[0], C.byref(p), out, max_surfaces, C.byref(n),
                                      _stream(stream)))
        return list(out[: n.value])

    def vector3d(self, keys, surfaces, stream=None):
        """rtr_vector3d (KeyPoint::get_Vector3D) for device keypoints [k, 4]:
        the plane-area vectors [k, 3] float64 on the device."""
        import torch
        nk = keys.shape[0]
        out = torch.empty((max(nk, 1), 3), dtype=torch.float64, device=keys.device)
        arr = (Surface * max(1, len(surfaces)))()
        for i, x in enumerate(surfaces):  # any record with the rtr_surface layout
            C.memmove(C.byref(arr[i]), C.byref(x), C.sizeof(Surface))
        check(lib().rtr_vector3d(self.h, _ptr(keys), nk, arr, len(surfaces), _ptr(out), _stream(stream)))
        return out[:nk]

    def knn(self, query, target, k: int, stream=None):
        import torch
        nq, nt = query.shape[0], target.shape[0]
        idx = torch.empty((nq, k), dtype=torch.int32, device=query.device)
        d2 = torch.empty((nq, k), dtype=torch.float32, device=query.device)
        check(lib().rtr_knn(self.h, _ptr(query), nq, _ptr(target), nt, int(k), _ptr(idx),
                            _ptr(d2), _stream(stream)))
        return idx, d2

    # -- ICP ------------------------------------------------------------------
    def icp(self, src, tgt, max_iterations=10, max_corr_dist=0.0, init=None,
            transformation_epsilon=0.0, rotation_epsilon=0.0, cell_size=0.0,
            trace=False, result=None, stream=None):
        """Run ICP on device tensors [n,4] float32.  Returns a device result
        buffer (bytes of rtr_icp_result) and, with trace=True, the per-iteration
        poses [(it+1),16] and correspondences [it, n_src]."""
        import torch
        p = IcpParams(max_iterations, max_corr_dist, transformation_epsilon, rotation_epsilon,
                      cell_size, 1 if trace else 0)
        dev = src.device
        if result is None:
            result = torch.zeros(C.sizeof(IcpResult), dtype=torch.uint8, device=dev)
        tp = tc = None
        if trace:
            tp = torch.zeros((max_iterations + 1, 16), dtype=torch.float64, device=dev)
            tc = torch.full((max_iterations, src.shape[0]), -2, dtype=torch.int32, device=dev)
        ini = None
        if init is not None:
            ini = np.ascontiguousarray(np.asarray(init, dtype=np.float64).reshape(16))
        check(lib().rtr_icp(self.h, _ptr(src), src.shape[0], _ptr(tgt), tgt.shape[0], C.byref(p),
                            None if ini is None else ini.ctypes.data, _ptr(result), _ptr(tp),
                            _ptr(tc), _stream(stream)))
        return result, tp, tc

    def icp_multi(self, src, tgt, inits, max_iterations=10, max_corr_dist=0.0, cell_size=0.0,
                  transformation_epsilon=0.0, rotation_epsilon=0.0, stream=None) -> list:
        """rtr_icp_multi: one ICP per initial pose (inits: [n, 16] or [n, 4, 4]
        float64, host or device) of src onto tgt; the parsed results."""
        import torch
        ini = torch.as_tensor(inits, dtype=torch.float64).reshape(-1, 16).contiguous().to(src.device)
        n = ini.shape[0]
        p = IcpParams(max_iterations, max_corr_dist, transformation_epsilon, rotation_epsilon, cell_size, 0)
        res = torch.zeros(n * C.sizeof(IcpResult), dtype=torch.uint8, device=src.device)
        check(lib().rtr_icp_multi(self.h, _ptr(src), src.shape[0], _ptr(tgt), tgt.shape[0], C.byref(p), _ptr(ini), n,
                                  _ptr(res), _stream(stream)))
        raw = bytes(res.cpu().numpy().tobytes())
        k = C.sizeof(IcpResult)
        return [self.parse_icp_result(raw[i * k:(i + 1) * k]) for i in range(n)]

    def pose_inliers(self, model, scene, poses, radius: float, stream=None):
        """rtr_pose_inliers: per model -> scene pose ([n, 16] or [n, 4, 4]
        float64), the model points with a scene point within radius."""
        import torch
        P = torch.as_tensor(poses, dtype=torch.float64).reshape(-1, 16).contiguous().to(model.device)
        cnt = torch.zeros(P.shape[0], dtype=torch.int32, device=model.device)
        check(lib().rtr_pose_inliers(self.h, _ptr(model), model.shape[0], _ptr(scene), scene.shape[0], _ptr(P),
                                     P.shape[0], float(radius), _ptr(cnt), _stream(stream)))
        return cnt

    @staticmethod
    def parse_icp_result(buf) -> dict:
        raw = bytes(buf.cpu().numpy().tobytes()) if not isinstance(buf, (bytes, bytearray)) else buf
        r = IcpResult.from_buffer_copy(raw)
        return {"pose": np.array(r.pose[:], dtype=np.float64).reshape(4, 4), "fitness": r.fitness,
                "iterations": r.iterations, "converged": r.converged, "n_corr": r.n_corr,
                "status": r.status}

    def icp_host(self, src: np.ndarray, tgt: np.ndarray, max_iterations=10, max_corr_dist=0.0,
                 init=None, transformation_epsilon=0.0, rotation_epsilon=0.0, cell_size=0.0):
        src = np.ascontiguousarray(src, dtype=np.float32)
        tgt = np.ascontiguousarray(tgt, dtype=np.float32)
        p = IcpParams(max_iterations, max_corr_dist, transformation_epsilon, rotation_epsilon,
                      cell_size, 0)
        r = IcpResult()
        ini = None if init is None else np.ascontiguousarray(np.asarray(init, np.float64).reshape(16))
        check(lib().rtr_icp_host(self.h, src.ctypes.data, src.shape[0], tgt.ctypes.data,
                                 tgt.shape[0], C.byref(p),
                                 None if ini is None else ini.ctypes.data, C.byref(r)))
        return {"pose": np.array(r.pose[:]).reshape(4, 4), "fitness": r.fitness,
                "iterations": r.iterations, "converged": r.converged, "n_corr": r.n_corr,
                "status": r.status}

    # -- recognition stages ---------------------------------------------------
    def voxel_downsample(self, pts, leaf: float, stream=None):
        import torch
        n = pts.shape[0]
        out = torch.empty((max(n, 1), 4), dtype=torch.float32, device=pts.device)
        cnt = torch.zeros(1, dtype=torch.int32, device=pts.device)
        check(lib().rtr_voxel_downsample(self.h, _ptr(pts), n, float(leaf), _ptr(out), _ptr(cnt),
                                         _stream(stream)))
        v = int(cnt.item())
        if v < 0:
            raise RtrError(1, "voxel key space exceeds 32 bits")
        return out[:v]

    def uniform_sample(self, pts, radius: float, stream=None):
        import torch
        n = pts.shape[0]
        out = torch.empty(max(n, 1), dtype=torch.int32, device=pts.device)
        cnt = torch.zeros(1, dtype=torch.int32, device=pts.device)
        check(lib().rtr_uniform_sample(self.h, _ptr(pts), n, float(radius), _ptr(out), _ptr(cnt),
                                       _stream(stream)))
        k = int(cnt.item())
        if k < 0:
            raise RtrError(1, "voxel key space exceeds 32 bits")
        return out[:k]

    def normals(self, pts, k: int = 10, vp=(0.0, 0.0, 0.0), search_cell: float = 0.0, stream=None):
        import torch
        n = pts.shape[0]
        out = torch.empty((n, 4), dtype=torch.float32, device=pts.device)
        v = np.ascontiguousarray(vp, np.float32)
        check(lib().rtr_normals(self.h, _ptr(pts), n, int(k), v.ctypes.data, float(search_cell),
                                _ptr(out), _stream(stream)))
        return out

    def orient_outward(self, pts, nrm, rc=0.01, gap=0.005, length=1.0, stream=None):
        check(lib().rtr_orient_normals_outward(self.h, _ptr(pts), _ptr(nrm), pts.shape[0], float(rc),
                                               float(gap), float(length), _stream(stream)))
        return nrm

    def shot352(self, pts, nrm, keys, radius: float, lrf: bool = False, stream=None):
        import torch
        nk = keys.shape[0]
        desc = torch.empty((nk, 352), dtype=torch.float32, device=pts.device)
        L = torch.empty((nk, 9), dtype=torch.float32, device=pts.device) if lrf else None
        check(lib().rtr_shot352(self.h, _ptr(pts), _ptr(nrm), pts.shape[0], _ptr(keys), nk,
                                float(radius), _ptr(desc), _ptr(L), _stream(stream)))
        return (desc, L) if lrf else desc

    def match(self, q, db, stream=None):
        import torch
        idx = torch.empty(q.shape[0], dtype=torch.int32, device=q.device)
        d2 = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
        check(lib().rtr_match(self.h, _ptr(q), q.shape[0], _ptr(db), db.shape[0], _ptr(idx), _ptr(d2),
                              _stream(stream)))
        return idx, d2

    def match_uncertified(self) -> int:
        n = C.c_int(0)
        check(lib().rtr_match_stats(self.h, C.byref(n)))
        return n.value

    def match_full_scans(self) -> int:
        """Uncertified queries of the last match that needed the exact scan
        of the whole database (band over 256 rows or non-finite values)."""
        n, f = C.c_int(0), C.c_int(0)
        check(lib().rtr_match_stats_ex(self.h, C.byref(n), C.byref(f)))
        return f.value

    def match_exact(self, q, db, stream=None):
        import torch
        idx = torch.empty(q.shape[0], dtype=torch.int32, device=q.device)
        d2 = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
        check(lib().rtr_match_exact(self.h, _ptr(q), q.shape[0], _ptr(db), db.shape[0], _ptr(idx),
                                    _ptr(d2), _stream(stream)))
        return idx, d2

    def icp_stats(self) -> dict:
        """Time of the last ICP launch (first problem), summed over iterations."""
        v = (C.c_longlong * 6)()
        check(lib().rtr_icp_stats(self.h, v))
        return {"search_ns": v[0], "serial_ns": v[1], "wait_ns": v[2], "iterations": v[3],
                "serial_reduce_ns": v[4], "serial_solve_ns": v[5]}

    def gc_stats(self) -> dict:
        """Work of the last grouping: rounds, walk end position, sets computed,
        microseconds per round phase."""
        v = (C.c_int * 8)()
        check(lib().rtr_gc_stats(self.h, C.byref(v)))
        return {"rounds": v[0], "walk_end": v[1], "sets": v[2], "candidates": v[7],
                "us": {"select": v[3], "seed_tests": v[4], "admission": v[5], "walk": v[6]}}

    def gc_group(self, model_kp, scene_kp, corr_m, corr_s, corr_d, gc_size=0.01, gc_thresh=5,
                 max_clusters=64, max_members=128, stream=None):
        import torch
        dev = model_kp.device
        mem = torch.full((max_clusters, max_members), -1, dtype=torch.int32, device=dev)
        sizes = torch.zeros(max_clusters, dtype=torch.int32, device=dev)
        poses = torch.zeros((max_clusters, 16), dtype=torch.float64, device=dev)
        n = C.c_int(0)
        check(lib().rtr_gc_group(self.h, _ptr(model_kp), _ptr(scene_kp), _ptr(corr_m), _ptr(corr_s),
                                 _ptr(corr_d), corr_m.shape[0], float(gc_size), int(gc_thresh),
                                 int(max_clusters), int(max_members), _ptr(mem), _ptr(sizes),
                                 _ptr(poses), C.byref(n), _stream(stream)))
        k = n.value
        return mem[:k], sizes[:k], poses[:k].reshape(k, 4, 4)

    # -- TDF ------------------------------------------------------------------
    # ---- the reference's own descriptor route (rtr_ref_*) -----------------
    def ref_occupancy(self, cloud, keys, resolution: float = 0.01, half_box: float = 0.1, stream=None):
        """KeyPoint::getOccupiedGrid for every keypoint: (number [nk] int32,
        offsets [nk+1] int32, indices [total] int32), device tensors."""
        import torch
        nk = keys.shape[0]
        dev = keys.device
        number = torch.empty(nk, dtype=torch.int32, device=dev)
        offsets = torch.empty(nk + 1, dtype=torch.int32, device=dev)
        total = C.c_longlong(0)
        cap = 1 << 16
        for _ in range(2):
            indices = torch.empty(max(cap, 1), dtype=torch.int32, device=dev)
            st = lib().rtr_ref_occupancy(self.h, _ptr(cloud), cloud.shape[0], _ptr(keys), nk, float(resolution),
                                         float(half_box), _ptr(number), _ptr(offsets), _ptr(indices), cap,
                                         C.byref(total), _stream(stream))
            if st == 6 and total.value > cap:  # RTR_ERR_CAPACITY: allocate and call again
                cap = total.value
                continue
            check(st)
            return number, offsets, indices[:total.value]
        raise RtrError(6, "rtr_ref_occupancy: capacity")

    def ref_tdf(self, cloud, keys, offsets, indices, resolution: float = 0.01, half_tdf: float = 0.15,
                stream=None):
        """KeyPoint::get_TSDF for every keypoint: [nk, dim^3] float32."""
        import torch
        nk = keys.shape[0]
        dim = int(np.float32(np.float32(half_tdf) / np.float32(resolution)) * np.float32(2))
        out = torch.empty((nk, max(dim, 1) ** 3), dtype=torch.float32, device=keys.device)
        got = C.c_int(0)
        check(lib().rtr_ref_tdf(self.h, _ptr(cloud), _ptr(keys), nk, _ptr(offsets), _ptr(indices),
                                float(resolution), float(half_tdf), _ptr(out), C.byref(got), _stream(stream)))
        return out

    def ref_distance(self, mcloud, mkeys, moffsets, mindices, mtdf, skeys, pair_m=None, pair_s=None,
                     resolution: float = 0.01, half_tdf: float = 0.15, stream=None):
        """get_Distance for explicit pairs, or all model x scan pairs
        (model-major) when pair_m is None: (score [P], T [P, 4, 4])."""
        import torch
        nm, ns = mkeys.shape[0], skeys.shape[0]
        P = nm * ns if pair_m is None else pair_m.shape[0]
        score = torch.empty(P, dtype=torch.float32, device=mkeys.device)
        T = torch.empty((P, 4, 4), dtype=torch.float32, device=mkeys.device)
        check(lib().rtr_ref_distance(self.h, _ptr(mcloud), _ptr(mkeys), nm, _ptr(moffsets), _ptr(mindices),
                                     _ptr(mtdf), _ptr(skeys), ns, _ptr(pair_m), _ptr(pair_s), P,
                                     float(resolution), float(half_tdf), _ptr(score), _ptr(T), _stream(stream)))
        return score, T

    def ref_correspond(self, mkeys, mnumber, skeys, snumber, score_all, max_score: float = 3.0, mv3=None,
                       sv3=None, stream=None):
        """The all-pairs loop with its gates: kept pair indices
        p = m * n_scan + s, ascending (device int32)."""
        import torch
        nm, ns = mkeys.shape[0], skeys.shape[0]
        cap = max(nm * ns, 1)
        out = torch.empty(cap, dtype=torch.int32, device=mkeys.device)
        n = C.c_int(0)
        check(lib().rtr_ref_correspond(self.h, _ptr(mkeys), _ptr(mnumber), _ptr(mv3), nm, _ptr(skeys),
                                       _ptr(snumber), _ptr(sv3), ns, _ptr(score_all), float(max_score), _ptr(out),
                                       cap, C.byref(n), _stream(stream)))
        return out[:n.value]

    def ref_ransac(self, mkeys, skeys, pair_idx, score_all, T_all, inlier: float = 0.15, max_des: float = 100.0,
                   stream=None):
        """Ransac over the kept pairs: (T [4, 4] numpy float32, inliers,
        position of the winner in pair_idx or -1)."""
        T = np.zeros(16, np.float32)
        inl, best = C.c_int(0), C.c_int(-1)
        check(lib().rtr_ref_ransac(self.h, _ptr(mkeys), mkeys.shape[0], _ptr(skeys), skeys.shape[0],
                                   _ptr(pair_idx), pair_idx.shape[0], _ptr(score_all), _ptr(T_all), float(inlier),
                                   float(max_des), T.ctypes.data, C.byref(inl), C.byref(best), _stream(stream)))
        return T.reshape(4, 4), inl.value, best.value

    def tdf_batch(self, occ, offsets, dim: int, stream=None):
        import torch
        n = offsets.shape[0] - 1
        out = torch.empty((n, dim * dim * dim), dtype=torch.float32, device=offsets.device)
        check(lib().rtr_tdf_batch(self.h, _ptr(occ), _ptr(offsets), n, dim, _ptr(out),
                                  _stream(stream)))
        return out


MLP_PARAMS = 53505  # RTR_MLP_PARAMS


class Mlp:
    """The keypoint-credibility MLP on the device (rtr_mlp_*)."""

    def __init__(self, ctx: "Context", params: np.ndarray | None = None, seed: int = 0):
        self.ctx = ctx
        h = _P()
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        check(lib().rtr_mlp_create(ctx.h, None if p is None else p.ctypes.data, seed, C.byref(h)))
        self.h = h

    def params(self) -> np.ndarray:
        out = np.empty(MLP_PARAMS, np.float32)
        check(lib().rtr_mlp_get_params(self.h, out.ctypes.data))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().rtr_mlp_set_params(self.h, p.ctypes.data))

    def score(self, x, stream=None):
        import torch
        s = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        check(lib().rtr_mlp_score(self.ctx.h, self.h, _ptr(x), x.shape[0], _ptr(s), _stream(stream)))
        return s

    def loss_grad(self, x, y, stream=None):
        import torch
        g = torch.empty(MLP_PARAMS, dtype=torch.float32, device=x.device)
        loss = torch.empty(1, dtype=torch.float32, device=x.device)
        check(lib().rtr_mlp_loss_grad(self.ctx.h, self.h, _ptr(x), _ptr(y), x.shape[0], _ptr(g), _ptr(loss),
                                      _stream(stream)))
        return loss, g

    def train_step(self, x, y, lr=1e-3, stream=None):
        import torch
        loss = torch.empty(1, dtype=torch.float32, device=x.device)
        check(lib().rtr_mlp_train_step(self.ctx.h, self.h, _ptr(x), _ptr(y), x.shape[0], float(lr), _ptr(loss),
                                       _stream(stream)))
        return loss

    def train(self, x, y, batch=4096, epochs=20, lr=1e-3, seed=0) -> np.ndarray:
        out = np.zeros(epochs, np.float32)
        check(lib().rtr_mlp_train(self.ctx.h, self.h, _ptr(x), _ptr(y), x.shape[0], int(batch), int(epochs),
                                  float(lr), int(seed), out.ctypes.data))
        return out

    def close(self):
        if self.h:
            lib().rtr_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Model:
    """A prepared object model (voxel cloud, outward normals, keypoints, SHOT)."""

    def __init__(self, ctx: "Context", pts, params: RecogParams | None = None):
        self.params = params or recog_default_params()
        h = _P()
        check(lib().rtr_model_create(ctx.h, _ptr(pts), pts.shape[0], C.byref(self.params),
                                     C.byref(h)))
        self.h = h
        nv, nk = C.c_int(), C.c_int()
        check(lib().rtr_model_info(self.h, C.byref(nv), C.byref(nk)))
        self.n_voxels, self.n_keypoints = nv.value, nk.value

    def buffers(self):
        ptrs = [_P() for _ in range(5)]
        check(lib().rtr_model_buffers(self.h, *[C.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]

    def close(self):
        if self.h:
            lib().rtr_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def recognize(ctx: "Context", model: Model, scene, params: RecogParams | None = None, result=None,
              stream=None):
    """Run rtr_recognize on a device scene [n,4]; returns the device result
    buffer (parse with parse_recog_result)."""
    import torch
    p = params or model.params
    if result is None:
        result = torch.zeros(C.sizeof(RecogResult), dtype=torch.uint8, device=scene.device)
    check(lib().rtr_recognize(ctx.h, model.h, _ptr(scene), scene.shape[0], C.byref(p),
                              _ptr(result), _stream(stream)))
    return result


def recognize_learned(ctx: "Context", model: Model, mlp: "Mlp", scene, keep: float = 0.25,
                      params: RecogParams | None = None, result=None, stream=None):
    """rtr_recognize_learned: recognition with the MLP keeping the `keep`
    fraction of most credible scene keypoints before matching."""
    import torch
    p = params or model.params
    if result is None:
        result = torch.zeros(C.sizeof(RecogResult), dtype=torch.uint8, device=scene.device)
    check(lib().rtr_recognize_learned(ctx.h, model.h, mlp.h, float(keep), _ptr(scene), scene.shape[0], C.byref(p),
                                      _ptr(result), _stream(stream)))
    return result


class BatchPair(C.Structure):
    _fields_ = [("model", _P), ("d_scene", _P), ("n", C.c_int)]


def _batch_args(models, scenes):
    arr = (BatchPair * len(scenes))()
    for i, (m, s) in enumerate(zip(models, scenes)):
        arr[i].model = m.h.value if isinstance(m.h, C.c_void_p) else m.h
        arr[i].d_scene = _ptr(s)
        arr[i].n = s.shape[0]
    return arr


def recognize_batch(ctx: "Context", models, scenes, params: RecogParams, mlp: "Mlp | None" = None,
                    keep: float = 1.0, results=None):
    """rtr_recognize_batch over pairs (models[i], scenes[i]); returns the device
    result buffer [n_pairs, sizeof(rtr_recog_result)]."""
    import torch
    n = len(scenes)
    if results is None:
        results = torch.zeros((max(n, 1), C.sizeof(RecogResult)), dtype=torch.uint8, device="cuda")
    arr = _batch_args(models, scenes)
    check(lib().rtr_recognize_batch(ctx.h, arr, n, C.byref(params), mlp.h if mlp else None, float(keep),
                                    _ptr(results)))
    return results


def recognize_multi(ctx: "Context", models, scene, params: RecogParams, mlp: "Mlp | None" = None,
                    keep: float = 1.0, results=None, stream=None):
    """rtr_recognize_multi: every model in one device scene [n, 4], the
    scene's stages once; returns the device result buffer [n_models,
    sizeof(rtr_recog_result)]."""
    import torch
    n = len(models)
    if results is None:
        results = torch.zeros((max(n, 1), C.sizeof(RecogResult)), dtype=torch.uint8, device="cuda")
    arr = (_P * max(n, 1))()
    for i, m in enumerate(models):
        arr[i] = m.h.value if isinstance(m.h, C.c_void_p) else m.h
    check(lib().rtr_recognize_multi(ctx.h, arr, n, mlp.h if mlp else None, float(keep), _ptr(scene), scene.shape[0],
                                    C.byref(params), _ptr(results), _stream(stream)))
    return results


class BatchGraph:
    """rtr_batch_graph_*: the batch captured once, replayed by launch()."""

    def __init__(self, ctx: "Context", models, scenes, params: RecogParams, mlp: "Mlp | None" = None,
                 keep: float = 1.0, results=None):
        import torch
        n = len(scenes)
        self.results = results if results is not None else torch.zeros(
            (n, C.sizeof(RecogResult)), dtype=torch.uint8, device="cuda")
        self._keep = (models, scenes, params, mlp)  # inputs must outlive the graph
        h = _P()
        check(lib().rtr_batch_graph_create(ctx.h, _batch_args(models, scenes), n, C.byref(params),
                                           mlp.h if mlp else None, float(keep), _ptr(self.results), C.byref(h)))
        self.h = h
        self._ctx = ctx  # the context outlives the graph
        ctx._graphs.add(self)

    def launch(self, stream=None):
        check(lib().rtr_batch_graph_launch(self.h, _stream(stream)))
        return self.results

    def close(self):
        if self.h:
            lib().rtr_batch_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_autotune(ctx: "Context", models, scenes, params: RecogParams, mlp: "Mlp | None" = None,
                   keep: float = 1.0):
    import torch
    n = len(scenes)
    results = torch.zeros((max(n, 1), C.sizeof(RecogResult)), dtype=torch.uint8, device="cuda")
    w, g = C.c_int(), C.c_int()
    check(lib().rtr_batch_autotune(ctx.h, _batch_args(models, scenes), n, C.byref(params),
                                   mlp.h if mlp else None, float(keep), _ptr(results), C.byref(w), C.byref(g)))
    return w.value, g.value


def batch_tuning(ctx: "Context") -> dict:
    """The tuple the autotuner settled on (0 = the automatic choice)."""
    return {k: ctx.get_tuning(k) for k in ("batch_workers", "icp_group", "scene_grid_mm", "normals_grid_mm")}


def recognize_host(ctx: "Context", model: Model, scene: np.ndarray, params: RecogParams | None = None):
    p = params or model.params
    s = np.ascontiguousarray(scene, np.float32)
    r = RecogResult()
    check(lib().rtr_recognize_host(ctx.h, model.h, s.ctypes.data, s.shape[0], C.byref(p), C.byref(r)))
    return parse_recog_result(bytes(r))


def compute_tdf_with_cuda(occ: np.ndarray, grid_value: np.ndarray, dim: int) -> int:
    """The reference's ComputeTDFWithCuda (kernel.cu:34): host arrays in/out."""
    occ = np.ascontiguousarray(occ, dtype=np.int32).reshape(-1)
    assert grid_value.dtype == np.float32 and grid_value.flags.c_contiguous
    return lib().ComputeTDFWithCuda(occ.ctypes.data if occ.size else None, grid_value.ctypes.data,
                                    int(dim), occ.size // 3)


# -- synthetic inputs (host) -------------------------------------------------
CHAIR, DESK, SOFA = 0, 1, 2


def synth_shape(shape: int, n: int, seed: int) -> np.ndarray:
    out = np.empty((n, 4), dtype=np.float32)
    check(lib().rtr_synth_shape(shape, seed, n, out.ctypes.data))
    return out


def synth_rigid(seed: int, max_angle_deg: float, max_t: float) -> np.ndarray:
    T = np.empty(16, dtype=np.float64)
    lib().rtr_synth_rigid(seed, max_angle_deg, max_t, T.ctypes.data)
    return T.reshape(4, 4)


def synth_transform_noise(pts: np.ndarray, T: np.ndarray, sigma: float, seed: int) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    out = np.empty_like(pts)
    Tc = np.ascontiguousarray(T, dtype=np.float64).reshape(16)
    lib().rtr_synth_transform_noise(pts.ctypes.data, pts.shape[0], Tc.ctypes.data, sigma, seed,
                                    out.ctypes.data)
    return out


def synth_crop(pts: np.ndarray, max_frac: float, seed: int) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    out = np.empty_like(pts)
    m = lib().rtr_synth_crop(pts.ctypes.data, pts.shape[0], max_frac, seed, out.ctypes.data)
    return out[:m].copy()


class FusionMap:
    """rtr_map_*: GPU voxel-hash map of point means and counts."""

    def __init__(self, ctx: "Context", capacity: int = 1 << 23, voxel: float = 0.005):
        self.ctx = ctx
        h = _P()
        check(lib().rtr_map_create(ctx.h, int(capacity), float(voxel), C.byref(h)))
        self.h = h

    def clear(self, stream=None):
        check(lib().rtr_map_clear(self.h, _stream(stream)))

    def integrate(self, pts, count=None, stream=None):
        check(lib().rtr_map_integrate(self.h, _ptr(pts), pts.shape[0], _ptr(count), _stream(stream)))

    def extract(self, max_out: int = 1 << 23):
        """[k, 4] device tensor {mean x, y, z, count as int bits} of the occupied voxels."""
        import torch
        out = torch.empty((max_out, 4), dtype=torch.float32, device="cuda")
        n = C.c_int(0)
        check(lib().rtr_map_extract(self.ctx.h, self.h, _ptr(out), int(max_out), C.byref(n)))
        if n.value > max_out:  # only counted: extract again into a buffer that holds them
            out = torch.empty((n.value, 4), dtype=torch.float32, device="cuda")
            check(lib().rtr_map_extract(self.ctx.h, self.h, _ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def count(self) -> int:
        """Occupied voxels (synchronises)."""
        n = C.c_int(0)
        check(lib().rtr_map_extract(self.ctx.h, self.h, None, 0, C.byref(n)))
        return n.value

    def close(self):
        if self.h:
            lib().rtr_map_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def synth_room_boxes(seed: int, params: RoomParams | None = None, max_boxes: int = 256, max_instances: int = 32):
    """(boxes [k, 12], shapes, poses [n, 4, 4]) of the room's furniture."""
    p = params or room_default_params()
    boxes = np.zeros((max_boxes, 12), np.float32)
    nb, ni = C.c_int(0), C.c_int(0)
    shapes = np.zeros(max_instances, np.int32)
    poses = np.zeros((max_instances, 16), np.float64)
    check(lib().rtr_synth_room_boxes(C.byref(p), seed, boxes.ctypes.data, max_boxes, C.byref(nb),
                                     shapes.ctypes.data, poses.ctypes.data, max_instances, C.byref(ni)))
    k = min(ni.value, max_instances)
    return boxes[: nb.value], shapes[:k], poses[:k].reshape(k, 4, 4)


def synth_trajectory(seed: int, n_frames: int, fps: float = 30.0) -> np.ndarray:
    out = np.zeros((n_frames, 16), np.float64)
    lib().rtr_synth_trajectory(seed, n_frames, fps, out.ctypes.data)
    return out.reshape(n_frames, 4, 4)


def room_default_params() -> RoomParams:
    p = RoomParams()
    lib().rtr_room_default_params(C.byref(p))
    return p


def synth_room(seed: int, params: RoomParams | None = None, max_instances: int = 16):
    p = params or room_default_params()
    out = np.empty((p.n_points, 4), dtype=np.float32)
    shapes = np.zeros(max_instances, dtype=np.int32)
    poses = np.zeros((max_instances, 16), dtype=np.float64)
    n = C.c_int(0)
    check(lib().rtr_synth_room(C.byref(p), seed, out.ctypes.data, max_instances,
                               shapes.ctypes.data, poses.ctypes.data, C.byref(n)))
    k = min(n.value, max_instances)
    return out, shapes[:k].copy(), poses[:k].reshape(k, 4, 4).copy()


def config0_pair(seed: int, n: int = 20000):
    """Config-0 ICP pair: chair (n points) and its copy under a seeded rigid
    transform (axis uniform on S^2, angle U[0,15 deg], t U[+-0.1 m]^3) plus
    N(0, 2 mm) noise.  Returns (source, target, T_true)."""
    src = synth_shape(CHAIR, n, seed)
    T = synth_rigid(seed, 15.0, 0.1)
    tgt = synth_transform_noise(src, T, 0.002, seed + 7)
    return src, tgt, T
