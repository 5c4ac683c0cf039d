"""Seeded synthetic BA scenes (sgba_synth_generate in libsgba_synth.so, host
code; include/sgba_synth.h).  The generator is a separate small library, not
part of libsgba.so."""
import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsgba_synth.so")
_libs = {}


def _lib(path=None):
    path = path or LIB_PATH
    L = _libs.get(path)
    if L is None:
        if not os.path.exists(path):
            raise RuntimeError("scene generator library not built: %s" % path)
        L = C.CDLL(path)
        L.sgba_synth_generate.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                          C.POINTER(C.POINTER(_SynthC))]
        L.sgba_synth_generate.restype = C.c_int
        L.sgba_synth_free.argtypes = [C.POINTER(_SynthC)]
        _libs[path] = L
    return L

CIRCLE = 0
SPHERE = 1
LOOP = 2
WINDOW = 3

BASE_SEED = 20261203


class _SynthC(C.Structure):
    _fields_ = [
        ("n_cam", C.c_int32),
        ("n_pt", C.c_int32),
        ("n_obs", C.c_int64),
        ("intrinsics", C.c_double * 4),
        ("huber_delta", C.c_double),
        ("initial_lm_damping", C.c_double),
        ("num_iterations", C.c_int32),
        ("poses", C.POINTER(C.c_double)),
        ("poses_true", C.POINTER(C.c_double)),
        ("pose_const", C.POINTER(C.c_uint8)),
        ("points", C.POINTER(C.c_double)),
        ("points_true", C.POINTER(C.c_double)),
        ("obs_cam", C.POINTER(C.c_int32)),
        ("obs_pt", C.POINTER(C.c_int32)),
        ("obs_uv", C.POINTER(C.c_double)),
    ]


@dataclass
class BAProblem:
    """Host arrays of one bundle-adjustment problem."""

    poses: np.ndarray          # (n_cam, 7) world_from_camera
    points: np.ndarray         # (n_pt, 3)
    intrinsics: np.ndarray     # (4,) fx fy cx cy
    obs_cam: np.ndarray        # (n_obs,) int32
    obs_pt: np.ndarray         # (n_obs,) int32
    obs_uv: np.ndarray         # (n_obs, 2)
    huber_delta: float = 1.0
    pose_const: np.ndarray = None
    point_const: np.ndarray = None
    poses_true: np.ndarray = None
    points_true: np.ndarray = None
    initial_lm_damping: float = 1e-4
    num_iterations: int = 10
    intrinsics_free: bool = False  # the camera params are optimised too (a Free camera family)
    camera_model: int = 0          # 0 pinhole, 1 enhanced unified camera model (EUCM)
    eucm_alpha_beta: np.ndarray = None  # (2,) EUCM alpha beta (camera_model 1)

    @property
    def n_cam(self):
        return self.poses.shape[0]

    @property
    def n_pt(self):
        return self.points.shape[0]

    @property
    def n_obs(self):
        return self.obs_cam.shape[0]

    def copy(self):
        return BAProblem(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items()})


def generate(kind, n_cam=0, n_pt=0, seed=BASE_SEED, lib_path=None):
    """One seeded scene.  lib_path selects another library that exports the
    same generator (the CPU reference arm of the benchmark uses the oracle's)."""
    L = _lib(lib_path)
    ptr = C.POINTER(_SynthC)()
    st = L.sgba_synth_generate(int(kind), int(n_cam), int(n_pt), C.c_uint64(seed), C.byref(ptr))
    if st != 0:
        raise ValueError("sgba_synth_generate failed with %d" % st)
    try:
        s = ptr.contents
        nc, npt, no = s.n_cam, s.n_pt, s.n_obs

        def arr(p, n, dt):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n > 0 else np.zeros(0, dt)

        prob = BAProblem(
            poses=arr(s.poses, 7 * nc, np.float64).reshape(nc, 7),
            points=arr(s.points, 3 * npt, np.float64).reshape(npt, 3),
            intrinsics=np.array(list(s.intrinsics), dtype=np.float64),
            obs_cam=arr(s.obs_cam, no, np.int32),
            obs_pt=arr(s.obs_pt, no, np.int32),
            obs_uv=arr(s.obs_uv, 2 * no, np.float64).reshape(no, 2),
            huber_delta=s.huber_delta,
            pose_const=arr(s.pose_const, nc, np.uint8),
            point_const=None,
            poses_true=arr(s.poses_true, 7 * nc, np.float64).reshape(nc, 7),
            points_true=arr(s.points_true, 3 * npt, np.float64).reshape(npt, 3),
            initial_lm_damping=s.initial_lm_damping,
            num_iterations=s.num_iterations,
        )
    finally:
        L.sgba_synth_free(ptr)
    return prob
