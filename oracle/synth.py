"""Seeded synthetic inputs for the CPU baseline (test infrastructure).

Wraps oracle/libsynth.so: the generator source that librtr.so also compiles
(realtime_robot_gb300/csrc/synth.cpp, same compiler and flags), built
host-only so that the timed CPU baseline makes the same clouds as the GPU
path without loading the CUDA library.  Functions and arguments mirror the
package's synth_* helpers; tests/test_lib_cpu.py checks that both give
identical clouds.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libsynth.so"
CHAIR, DESK, SOFA = 0, 1, 2
_lib = None

_P, _I, _D, _U64 = C.c_void_p, C.c_int, C.c_double, C.c_uint64


class RoomParams(C.Structure):
    _fields_ = [("n_points", C.c_int), ("n_chairs", C.c_int), ("n_desks", C.c_int),
                ("n_sofas", C.c_int), ("sigma", C.c_double), ("cam", C.c_double * 3),
                ("look_at", C.c_double * 3), ("width", C.c_int), ("height", C.c_int),
                ("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double), ("cy", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import build
            build()
        L = C.CDLL(str(LIB_PATH))
        L.rtr_synth_shape.restype = _I
        L.rtr_synth_shape.argtypes = [_I, _U64, _I, _P]
        L.rtr_synth_rigid.restype = None
        L.rtr_synth_rigid.argtypes = [_U64, _D, _D, _P]
        L.rtr_synth_transform_noise.restype = None
        L.rtr_synth_transform_noise.argtypes = [_P, _I, _P, _D, _U64, _P]
        L.rtr_synth_crop.restype = _I
        L.rtr_synth_crop.argtypes = [_P, _I, _D, _U64, _P]
        L.rtr_room_default_params.restype = None
        L.rtr_room_default_params.argtypes = [C.POINTER(RoomParams)]
        L.rtr_synth_room.restype = _I
        L.rtr_synth_room.argtypes = [C.POINTER(RoomParams), _U64, _P, _I, _P, _P, C.POINTER(C.c_int)]
        _lib = L
    return _lib


def synth_shape(shape: int, n: int, seed: int) -> np.ndarray:
    out = np.empty((n, 4), dtype=np.float32)
    if lib().rtr_synth_shape(shape, seed, n, out.ctypes.data) != 0:
        raise ValueError("rtr_synth_shape failed")
    return out


def synth_rigid(seed: int, max_angle_deg: float, max_t: float) -> np.ndarray:
    T = np.empty(16, dtype=np.float64)
    lib().rtr_synth_rigid(seed, max_angle_deg, max_t, T.ctypes.data)
    return T.reshape(4, 4)


def synth_transform_noise(pts: np.ndarray, T: np.ndarray, sigma: float, seed: int) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    out = np.empty_like(pts)
    Tc = np.ascontiguousarray(T, dtype=np.float64).reshape(16)
    lib().rtr_synth_transform_noise(pts.ctypes.data, pts.shape[0], Tc.ctypes.data, sigma, seed, out.ctypes.data)
    return out


def synth_crop(pts: np.ndarray, max_frac: float, seed: int) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    out = np.empty_like(pts)
    m = lib().rtr_synth_crop(pts.ctypes.data, pts.shape[0], max_frac, seed, out.ctypes.data)
    return out[:m].copy()


def room_default_params() -> RoomParams:
    p = RoomParams()
    lib().rtr_room_default_params(C.byref(p))
    return p


def synth_room(seed: int, params: RoomParams | None = None, max_instances: int = 16):
    """(points [n, 4], shape per furniture piece, object->world poses [k, 4, 4])."""
    p = params or room_default_params()
    out = np.empty((p.n_points, 4), dtype=np.float32)
    shapes = np.zeros(max_instances, dtype=np.int32)
    poses = np.zeros((max_instances, 16), dtype=np.float64)
    n = C.c_int(0)
    if lib().rtr_synth_room(C.byref(p), seed, out.ctypes.data, max_instances, shapes.ctypes.data,
                            poses.ctypes.data, C.byref(n)) != 0:
        raise ValueError("rtr_synth_room failed")
    k = min(n.value, max_instances)
    return out, shapes[:k].copy(), poses[:k].reshape(k, 4, 4).copy()


def config0_pair(seed: int, n: int = 20000):
    """Config-0 ICP pair (same calls as the package's config0_pair)."""
    src = synth_shape(CHAIR, n, seed)
    T = synth_rigid(seed, 15.0, 0.1)
    tgt = synth_transform_noise(src, T, 0.002, seed + 7)
    return src, tgt, T
