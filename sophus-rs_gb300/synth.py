"""Seeded synthetic BA scenes (sgba_synth_generate in libsgba_synth.so, host
code; include/sgba_synth.h).  The generator is a separate small library, not
part of libsgba.so.  ring_box_eucm builds the scene of the reference's own BA
example problem and benchmark (EUCM camera) in numpy."""
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
    intrinsics_true: np.ndarray = None  # ground-truth camera params, where the scene has them

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


# ---- the reference's BA example problem (ba_problem.rs:115-346) ------------
EUCM_TRUE = np.array([300.0, 300.0, 320.0, 240.0, 0.5, 1.0])   # TRUE_FOCAL, cx, cy, alpha, beta
EUCM_INIT = np.array([297.0, 297.0, 321.0, 241.0, 0.495, 1.0])  # 0.99 TRUE_FOCAL, 321, 241, 0.495, 1.0
RING_RADIUS = 8.0
BOX_CENTER_Z = 10.0


def _quat_exp(w):
    """Unit quaternion (w x y z) of exp(hat(w)), w a rotation vector."""
    th = float(np.linalg.norm(w))
    if th < 1e-12:
        return np.array([1.0, 0.5 * w[0], 0.5 * w[1], 0.5 * w[2]])
    s = np.sin(0.5 * th) / th
    return np.array([np.cos(0.5 * th), s * w[0], s * w[1], s * w[2]])


def _quat_mul(a, b):
    return np.array([a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3],
                     a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2],
                     a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1],
                     a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0]])


def _quat_rot(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _se3_exp_left(xi, pose):
    """exp(xi) * T for the tangent xi = [rotation; translation] (the
    reference's Isometry3 tangent order) and T = (q w x y z, t)."""
    w, v = np.asarray(xi[:3], float), np.asarray(xi[3:], float)
    th = float(np.linalg.norm(w))
    h = np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])
    if th < 1e-8:
        V = np.eye(3) + 0.5 * h
    else:
        V = np.eye(3) + (1 - np.cos(th)) / th ** 2 * h + (th - np.sin(th)) / th ** 3 * (h @ h)
    dq = _quat_exp(w)
    q = _quat_mul(dq, pose[:4])
    q /= np.linalg.norm(q)
    if q[0] < 0:
        q = -q
    t = _quat_rot(dq) @ pose[4:] + V @ v
    return np.concatenate([q, t])


def eucm_project(params, x_cam):
    """EUCM projection of camera-frame points (n, 3): the z = 1 projection
    divided by alpha rho + (1 - alpha), rho = sqrt(beta r^2 + 1), then the
    affine map (enhanced_unified.rs:59-88)."""
    fx, fy, cx, cy, alpha, beta = params
    x, y = x_cam[:, 0] / x_cam[:, 2], x_cam[:, 1] / x_cam[:, 2]
    rho = np.sqrt(beta * (x * x + y * y) + 1.0)
    norm = alpha * rho + (1.0 - alpha)
    return np.stack([fx * x / norm + cx, fy * y / norm + cy], axis=1)


def ring_box_eucm(n_cam=10, n_pt=500, seed=BASE_SEED, intrinsics_free=True):
    """The scene of the reference's BaProblem::new(num_cameras, num_points)
    (crates/sophus_opt/src/example_problems/ba_problem.rs:154-346), the problem
    its BA benchmark runs (crates/sophus_opt/src/bin/ba_bench.rs: 10 cameras,
    500 points): cameras on a radius-8 m ring in the XZ plane looking inward at
    an open box of points (x in [-3, 3], y in [-2, 2], z in [8, 12], five faces,
    open towards z = 8), one shared EUCM camera (TRUE_FOCAL 300, alpha 0.5,
    beta 1.0), a camera sees a point when it lies in front (z > 0.1), inside the
    640x480 image and, with 20 or more cameras, within 8 m; pixel noise uniform
    +-0.075 px; points with fewer than two views dropped; initial params
    EUCM_INIT; poses 0 and 1 fixed at the truth, the others moved by
    exp(noise) with uniform noise of +-(0.04, 0.04, 0.02) rad and
    +-(0.03, 0.03, 0.01) m; points moved by +-0.2 m per coordinate.  No robust
    kernel; 20 LM iterations at initial damping 1.0 (ba_problem.rs:420-440).
    The random numbers come from numpy's generator seeded with `seed` (the
    reference uses ChaCha12 with a zero seed): the same shapes and
    distributions, not the same draws."""
    rng = np.random.default_rng(seed)
    u = rng.random
    poses_true = np.empty((n_cam, 7))
    for j in range(n_cam):
        th = 2.0 * np.pi * j / n_cam
        poses_true[j, :4] = _quat_exp(np.array([0.0, -th, 0.0]))
        poses_true[j, 4:] = [RING_RADIUS * np.sin(th), 0.0, BOX_CENTER_Z - RING_RADIUS * np.cos(th)]
    bw, bh, z_near, z_far = 3.0, 2.0, 8.0, 12.0
    pts = np.empty((n_pt, 3))
    for k in range(n_pt):
        f = k % 5
        if f == 0:
            pts[k] = [(u() - 0.5) * 2 * bw, (u() - 0.5) * 2 * bh, z_far]
        elif f == 1:
            pts[k] = [-bw, (u() - 0.5) * 2 * bh, z_near + u() * (z_far - z_near)]
        elif f == 2:
            pts[k] = [bw, (u() - 0.5) * 2 * bh, z_near + u() * (z_far - z_near)]
        elif f == 3:
            pts[k] = [(u() - 0.5) * 2 * bw, bh, z_near + u() * (z_far - z_near)]
        else:
            pts[k] = [(u() - 0.5) * 2 * bw, -bh, z_near + u() * (z_far - z_near)]
    max_vis = RING_RADIUS if n_cam >= 20 else np.inf
    cams, pids, uvs = [], [], []
    for j in range(n_cam):
        R = _quat_rot(poses_true[j, :4])
        c = poses_true[j, 4:]
        xc = (pts - c) @ R  # R^T (p - c) per row
        uv = eucm_project(EUCM_TRUE, xc)
        for k in range(n_pt):
            if np.linalg.norm(c - pts[k]) > max_vis or xc[k, 2] <= 0.1:
                continue
            if not (0.0 <= uv[k, 0] < 640.0 and 0.0 <= uv[k, 1] < 480.0):
                continue
            cams.append(j)
            pids.append(k)
            uvs.append(uv[k] + 0.15 * np.array([u() - 0.5, u() - 0.5]))
    cams, pids, uvs = np.array(cams, np.int32), np.array(pids, np.int64), np.array(uvs).reshape(-1, 2)
    counts = np.bincount(pids, minlength=n_pt)
    keep = counts >= 2
    remap = np.cumsum(keep) - 1
    sel = keep[pids]
    points_true = pts[keep]
    poses = poses_true.copy()
    for j in range(2, n_cam):
        noise = np.array([(u() - 0.5) * 0.08, (u() - 0.5) * 0.08, (u() - 0.5) * 0.04,
                          (u() - 0.5) * 0.06, (u() - 0.5) * 0.06, (u() - 0.5) * 0.02])
        poses[j] = _se3_exp_left(noise, poses_true[j])
    points = points_true + np.array([[(u() - 0.5) * 0.4 for _ in range(3)] for _ in range(len(points_true))]
                                    ).reshape(-1, 3)
    pose_const = np.zeros(n_cam, np.uint8)
    pose_const[:2] = 1
    return BAProblem(poses=poses, points=points, intrinsics=EUCM_INIT[:4].copy(), obs_cam=cams[sel],
                     obs_pt=remap[pids[sel]].astype(np.int32), obs_uv=uvs[sel], huber_delta=0.0,
                     pose_const=pose_const, point_const=None, poses_true=poses_true, points_true=points_true,
                     initial_lm_damping=1.0, num_iterations=20, intrinsics_free=intrinsics_free, camera_model=1,
                     eucm_alpha_beta=EUCM_INIT[4:].copy(), intrinsics_true=EUCM_TRUE.copy())
