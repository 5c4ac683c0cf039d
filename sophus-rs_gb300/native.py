"""ctypes binding of the C ABI in include/sgba.h (libsgba.so).

The library is the product: there is no CPU fallback.  If libsgba.so is
missing or cannot reach a CUDA device, every entry point raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libsgba.so")
_lib = None

# sgba_status
OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_INVALID_PARAMS = -2
ERR_SCHUR_MISSING_FREE_OR_MARG = -3
ERR_UNSUPPORTED = -4
ERR_CUDA = -5
ERR_OUT_OF_MEMORY = -6
ERR_STATE = -7
ERR_DEVICE_TIMEOUT = -8
ERR_FACTORIZATION = -9

CAMERA_PINHOLE = 0
CAMERA_EUCM = 1

# sgba_termination
TERM_NONE = 0
TERM_FUNCTION_TOLERANCE = 1
TERM_GRADIENT_TOLERANCE = 2
TERM_PARAMETER_TOLERANCE = 3
TERM_MAX_ITERATIONS = 4
TERM_MAX_CONSECUTIVE_REJECTS = 5

# sgba_layout.solver
SOLVER_DENSE_CLUSTER = 0
SOLVER_BAND = 1
SOLVER_DENSE_PANELS = 2
SOLVER_DENSE_SMALL = 3


class ProblemDesc(C.Structure):
    _fields_ = [
        ("n_cam", C.c_int32),
        ("poses", C.POINTER(C.c_double)),
        ("pose_const", C.POINTER(C.c_uint8)),
        ("n_pt", C.c_int32),
        ("points", C.POINTER(C.c_double)),
        ("point_const", C.POINTER(C.c_uint8)),
        ("intrinsics", C.c_double * 4),
        ("n_obs", C.c_int64),
        ("obs_cam", C.POINTER(C.c_int32)),
        ("obs_pt", C.POINTER(C.c_int32)),
        ("obs_uv", C.POINTER(C.c_double)),
        ("huber_delta", C.c_double),
    ]


class OptParamsC(C.Structure):
    _fields_ = [
        ("num_iterations", C.c_int32),
        ("initial_lm_damping", C.c_double),
        ("function_tolerance", C.c_double),
        ("gradient_tolerance", C.c_double),
        ("parameter_tolerance", C.c_double),
        ("max_consecutive_rejects", C.c_int64),
        ("skip_final_hessian", C.c_int32),
    ]


class IterRecord(C.Structure):
    _fields_ = [
        ("merit", C.c_double),
        ("new_merit", C.c_double),
        ("lm_damping", C.c_double),
        ("gain_ratio", C.c_double),
        ("max_step", C.c_double),
        ("max_grad", C.c_double),
        ("accepted", C.c_int32),
        ("termination", C.c_int32),
    ]


class Layout(C.Structure):
    _fields_ = [
        ("n_free_poses", C.c_int32),
        ("n_marg_points", C.c_int32),
        ("n_terms", C.c_int64),
        ("n_h_blocks", C.c_int64),
        ("n_s_blocks", C.c_int64),
        ("n_schur_pairs", C.c_int64),
        ("solver", C.c_int32),
        ("band_width", C.c_int32),
        ("border_rows", C.c_int32),
        ("float_float_lin", C.c_int32),
        ("intrinsics_rows", C.c_int32),
    ]


class ProblemOptions(C.Structure):
    _fields_ = [("intrinsics_free", C.c_int32), ("camera_model", C.c_int32),
                ("eucm_alpha_beta", C.c_double * 2), ("reserved", C.c_int32 * 2)]


class PoseGraph(C.Structure):
    _fields_ = [("n_edge", C.c_int32), ("edge_pose", C.POINTER(C.c_int32)), ("edge_m_from_n", C.POINTER(C.c_double))]


class Profile(C.Structure):
    _fields_ = [
        ("kernel_launches", C.c_int64),
        ("ms_total", C.c_double),
        ("ms_linearize", C.c_double),
        ("ms_schur", C.c_double),
        ("ms_factor", C.c_double),
        ("ms_update", C.c_double),
        ("ms_cost", C.c_double),
    ]


class WindowResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("termination", C.c_int32),
        ("n_records", C.c_int32),
        ("ms", C.c_float),
        ("final_cost", C.c_double),
    ]


class BatchStats(C.Structure):
    _fields_ = [
        ("batched_windows", C.c_int32),
        ("schedule", C.c_int32),
        ("groups", C.c_int32),
        ("order", C.c_int32),
        ("tuned", C.c_int32),
        ("pad", C.c_int32),
        ("kernel_launches", C.c_int64),
        ("ms", C.c_float),
        ("schedule_ms", C.c_float * 4),
    ]


class LinearSolverC(C.Structure):
    _fields_ = [("mode", C.c_int32), ("max_iterations", C.c_int32), ("tolerance", C.c_double)]


class PcgStats(C.Structure):
    _fields_ = [
        ("solves", C.c_int64),
        ("fallbacks", C.c_int64),
        ("iterations", C.c_int64),
        ("last_iterations", C.c_int32),
        ("last_status", C.c_int32),
        ("last_relative_residual", C.c_double),
    ]


# sgba_linsolve_mode
LINSOLVE_EXACT = 0
LINSOLVE_PCG_BLOCK_JACOBI = 1
LINSOLVE_PCG_LEARNED = 2

EXPORTED = [
    "sgba_abi_version", "sgba_last_error", "sgba_problem_create", "sgba_problem_create_ex", "sgba_problem_create_graph",
    "sgba_get_intrinsics", "sgba_problem_destroy",
    "sgba_optimizer_init", "sgba_optimizer_step", "sgba_optimize", "sgba_get_variables",
    "sgba_get_cost", "sgba_set_variables", "sgba_get_layout", "sgba_export_pattern",
    "sgba_debug_last_system", "sgba_debug_jacobians", "sgba_state_save", "sgba_state_load", "sgba_get_profile",
    "sgba_set_profiling", "sgba_bench_iterations", "sgba_bench_kernel", "sgba_batch_optimize", "sgba_batch_last_stats", "sgba_set_pose_priors", "sgba_set_eq_constraints",
    "sgba_set_linear_solver", "sgba_get_pcg_stats", "sgba_pcg_num_params", "sgba_pcg_model_create",
    "sgba_pcg_model_destroy", "sgba_pcg_model_set_params", "sgba_pcg_model_get_params",
    "sgba_pcg_trainset_create", "sgba_pcg_trainset_destroy", "sgba_pcg_trainset_size", "sgba_pcg_trainset_add",
    "sgba_pcg_collect", "sgba_pcg_loss_grad", "sgba_pcg_train", "sgba_pcg_evaluate",
    "sgba_covariance_prepare", "sgba_covariance_release", "sgba_covariance_blocks",
]

# covariance queries (sgba_covariance_blocks)
VAR_INTRINSICS = 0
VAR_POSE = 1
VAR_POINT = 2
QUERY_COVARIANCE = 0
QUERY_PRECISION = 1


class CovInfo(C.Structure):
    _fields_ = [("n", C.c_int32), ("rank", C.c_int32), ("kernel_launches", C.c_int32), ("pad", C.c_int32),
                ("ms_assemble", C.c_double), ("ms_factor", C.c_double), ("ms_inverse", C.c_double)]


class CovQuery(C.Structure):
    _fields_ = [("row_kind", C.c_int32), ("row_index", C.c_int32), ("col_kind", C.c_int32), ("col_index", C.c_int32)]


class PcgTrainParams(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("learning_rate", C.c_double), ("seed", C.c_uint64)]

# sgba_kernel_id
KERNEL_ITERATION = 0
KERNEL_SCHUR = 1
KERNEL_LANDMARK = 2
KERNEL_CAMERA = 3
KERNEL_COST = 4
KERNEL_FACTOR = 5
KERNEL_BACKSUB = 6


class SgbaError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("sgba status %d: %s" % (status, message))
        self.status = status
        self.message = message


def lib_path():
    return _LIB_PATH


def lib():
    """Load libsgba.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise RuntimeError("libsgba.so is not built (%s); run `python __graft_entry__.py` first" % _LIB_PATH)
    L = C.CDLL(_LIB_PATH)
    dp = C.POINTER(C.c_double)
    L.sgba_abi_version.restype = C.c_int32
    L.sgba_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.sgba_last_error.restype = C.c_size_t
    L.sgba_problem_create.argtypes = [C.POINTER(ProblemDesc), C.c_int32, C.POINTER(C.c_void_p)]
    L.sgba_problem_create_graph.argtypes = [C.POINTER(ProblemDesc), C.POINTER(ProblemOptions), C.POINTER(PoseGraph),
                                            C.c_int32, C.POINTER(C.c_void_p)]
    L.sgba_problem_create_ex.argtypes = [C.POINTER(ProblemDesc), C.POINTER(ProblemOptions), C.c_int32,
                                         C.POINTER(C.c_void_p)]
    L.sgba_get_intrinsics.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    L.sgba_problem_destroy.argtypes = [C.c_void_p]
    L.sgba_optimizer_init.argtypes = [C.c_void_p, C.POINTER(OptParamsC)]
    L.sgba_optimizer_step.argtypes = [C.c_void_p, C.POINTER(IterRecord)]
    L.sgba_optimize.argtypes = [C.c_void_p, C.POINTER(OptParamsC), C.POINTER(IterRecord), C.c_int32,
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.sgba_get_variables.argtypes = [C.c_void_p, dp, dp]
    L.sgba_set_variables.argtypes = [C.c_void_p, dp, dp]
    L.sgba_get_cost.argtypes = [C.c_void_p, dp]
    L.sgba_get_layout.argtypes = [C.c_void_p, C.POINTER(Layout)]
    ip = C.POINTER(C.c_int32)
    L.sgba_export_pattern.argtypes = [C.c_void_p, ip, ip, ip, ip]
    L.sgba_debug_last_system.argtypes = [C.c_void_p, dp, dp, dp]
    L.sgba_debug_jacobians.argtypes = [C.c_void_p, C.c_int64, ip, ip, C.c_int32, dp, dp]
    L.sgba_state_save.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_size_t)]
    L.sgba_state_load.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    L.sgba_get_profile.argtypes = [C.c_void_p, C.POINTER(Profile)]
    L.sgba_set_profiling.argtypes = [C.c_void_p, C.c_int32]
    L.sgba_bench_iterations.argtypes = [C.c_void_p, C.c_int32, C.c_int32, dp, C.POINTER(C.c_int64)]
    L.sgba_bench_kernel.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, dp]
    L.sgba_batch_optimize.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(OptParamsC),
                                      C.POINTER(IterRecord), C.c_int32, C.POINTER(WindowResult)]
    L.sgba_batch_last_stats.argtypes = [C.POINTER(BatchStats)]
    L.sgba_set_pose_priors.argtypes = [C.c_void_p, C.c_int32, ip, dp, dp]
    L.sgba_set_eq_constraints.argtypes = [C.c_void_p, C.c_int32, ip, dp]
    L.sgba_set_linear_solver.argtypes = [C.c_void_p, C.POINTER(LinearSolverC), C.c_void_p]
    L.sgba_get_pcg_stats.argtypes = [C.c_void_p, C.POINTER(PcgStats)]
    L.sgba_pcg_num_params.restype = C.c_int32
    L.sgba_pcg_model_create.argtypes = [C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]
    L.sgba_pcg_model_destroy.argtypes = [C.c_void_p]
    fp = C.POINTER(C.c_float)
    L.sgba_pcg_model_set_params.argtypes = [C.c_void_p, fp, C.c_int32]
    L.sgba_pcg_model_get_params.argtypes = [C.c_void_p, fp, C.c_int32]
    L.sgba_pcg_trainset_create.argtypes = [C.c_int32, C.POINTER(C.c_void_p)]
    L.sgba_pcg_trainset_destroy.argtypes = [C.c_void_p]
    L.sgba_pcg_trainset_size.argtypes = [C.c_void_p]
    L.sgba_pcg_trainset_size.restype = C.c_int32
    L.sgba_pcg_trainset_add.argtypes = [C.c_void_p, C.c_int32, C.c_int64, ip, ip, dp, dp, dp]
    L.sgba_pcg_collect.argtypes = [C.c_void_p, C.c_void_p]
    L.sgba_pcg_loss_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, dp, fp, C.c_int32]
    L.sgba_pcg_train.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(PcgTrainParams), dp]
    L.sgba_pcg_evaluate.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                    C.POINTER(C.c_int32), dp, C.POINTER(C.c_int32)]
    L.sgba_covariance_prepare.argtypes = [C.c_void_p, C.POINTER(CovInfo)]
    L.sgba_covariance_release.argtypes = [C.c_void_p]
    L.sgba_covariance_blocks.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(CovQuery), dp, ip]
    _lib = L
    return L


def last_error():
    L = lib()
    buf = C.create_string_buffer(1024)
    L.sgba_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status):
    if status != OK:
        raise SgbaError(status, last_error())
    return status


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ipt(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _u8p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def opt_params_c(p):
    """Convert an OptParams-like object into the C struct."""
    mr = p.max_consecutive_rejects
    if mr is None or mr > (1 << 62):
        mr = 1 << 62
    return OptParamsC(int(p.num_iterations), float(p.initial_lm_damping), float(p.function_tolerance),
                      float(p.gradient_tolerance), float(p.parameter_tolerance), int(mr),
                      int(bool(getattr(p, "skip_final_hessian", False))))


class Problem:
    """One device-resident BA problem (sgba_problem handle).

    `data` needs poses (n,7), points (m,3), intrinsics (4,), obs_cam, obs_pt,
    obs_uv (k,2), huber_delta and optionally pose_const / point_const.
    """

    def __init__(self, data, device=-1, intrinsics_free=None):
        """intrinsics_free (default: data.intrinsics_free, else False): the
        camera params are a Free family, optimised with the poses.  The camera
        is data.camera_model (CAMERA_PINHOLE when absent; CAMERA_EUCM with
        data.eucm_alpha_beta)."""
        L = lib()
        if intrinsics_free is None:
            intrinsics_free = bool(getattr(data, "intrinsics_free", False))
        self.camera_model = int(getattr(data, "camera_model", CAMERA_PINHOLE))
        self._keep = []
        poses = np.ascontiguousarray(data.poses, dtype=np.float64).reshape(-1, 7)
        points = np.ascontiguousarray(data.points, dtype=np.float64).reshape(-1, 3)
        self.n_cam = poses.shape[0]
        self.n_pt = points.shape[0]
        obs_cam = np.ascontiguousarray(data.obs_cam, dtype=np.int32)
        obs_pt = np.ascontiguousarray(data.obs_pt, dtype=np.int32)
        obs_uv = np.ascontiguousarray(data.obs_uv, dtype=np.float64).reshape(-1, 2)
        pc = getattr(data, "pose_const", None)
        qc = getattr(data, "point_const", None)
        pc = None if pc is None else np.ascontiguousarray(pc, dtype=np.uint8)
        qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.uint8)
        self._keep += [poses, points, obs_cam, obs_pt, obs_uv, pc, qc]
        d = ProblemDesc()
        d.n_cam = self.n_cam
        d.poses = _dptr(poses)
        d.pose_const = _u8p(pc) if pc is not None else None
        d.n_pt = self.n_pt
        d.points = _dptr(points)
        d.point_const = _u8p(qc) if qc is not None else None
        for k in range(4):
            d.intrinsics[k] = float(data.intrinsics[k])
        d.n_obs = obs_cam.shape[0]
        d.obs_cam = _ipt(obs_cam)
        d.obs_pt = _ipt(obs_pt)
        d.obs_uv = _dptr(obs_uv)
        d.huber_delta = float(data.huber_delta) if data.huber_delta is not None else 0.0
        h = C.c_void_p()
        edges = getattr(data, "edge_pose", None)
        if edges is not None and len(edges):
            ep = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
            mn = np.ascontiguousarray(data.edge_mn, dtype=np.float64).reshape(ep.shape[0], 7)
            self._keep += [ep, mn]
            g = PoseGraph()
            g.n_edge = ep.shape[0]
            g.edge_pose = ep.ctypes.data_as(C.POINTER(C.c_int32))
            g.edge_m_from_n = _dptr(mn)
            opts = ProblemOptions()
            opts.intrinsics_free = 1 if intrinsics_free else 0
            opts.camera_model = self.camera_model
            if self.camera_model == CAMERA_EUCM:
                opts.eucm_alpha_beta[0] = float(data.eucm_alpha_beta[0])
                opts.eucm_alpha_beta[1] = float(data.eucm_alpha_beta[1])
            check(L.sgba_problem_create_graph(C.byref(d), C.byref(opts), C.byref(g), int(device), C.byref(h)))
        elif intrinsics_free or self.camera_model != CAMERA_PINHOLE:
            opts = ProblemOptions()
            opts.intrinsics_free = 1 if intrinsics_free else 0
            opts.camera_model = self.camera_model
            if self.camera_model == CAMERA_EUCM:
                ab = data.eucm_alpha_beta
                opts.eucm_alpha_beta[0] = float(ab[0])
                opts.eucm_alpha_beta[1] = float(ab[1])
            check(L.sgba_problem_create_ex(C.byref(d), C.byref(opts), int(device), C.byref(h)))
        else:
            check(L.sgba_problem_create(C.byref(d), int(device), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().sgba_problem_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, params):
        check(lib().sgba_optimizer_init(self._h, C.byref(opt_params_c(params))))

    def step(self):
        r = IterRecord()
        check(lib().sgba_optimizer_step(self._h, C.byref(r)))
        return r

    def optimize(self, params):
        cap = max(1, int(params.num_iterations))
        recs = (IterRecord * cap)()
        n = C.c_int32()
        term = C.c_int32()
        check(lib().sgba_optimize(self._h, C.byref(opt_params_c(params)), recs, cap, C.byref(n), C.byref(term)))
        return [recs[i] for i in range(min(n.value, cap))], term.value

    def variables(self):
        poses = np.empty((self.n_cam, 7))
        points = np.empty((self.n_pt, 3))
        check(lib().sgba_get_variables(self._h, _dptr(poses), _dptr(points)))
        return poses, points

    def set_variables(self, poses=None, points=None):
        pp = None if poses is None else np.ascontiguousarray(poses, dtype=np.float64)
        qq = None if points is None else np.ascontiguousarray(points, dtype=np.float64)
        check(lib().sgba_set_variables(self._h, _dptr(pp) if pp is not None else None,
                                       _dptr(qq) if qq is not None else None))

    def set_pose_priors(self, pose, mean, precision):
        """sgba_set_pose_priors: Isometry3 priors (pose indices, n x 7 means, n x 6 x 6
        precisions); an empty set removes them."""
        pose = np.ascontiguousarray(pose, dtype=np.int32).reshape(-1)
        n = pose.shape[0]
        mean = np.ascontiguousarray(mean, dtype=np.float64).reshape(n, 7)
        precision = np.ascontiguousarray(precision, dtype=np.float64).reshape(n, 6, 6)
        check(lib().sgba_set_pose_priors(self._h, n, pose.ctypes.data_as(C.POINTER(C.c_int32)) if n else None,
                                         _dptr(mean) if n else None, _dptr(precision) if n else None))

    def set_eq_constraints(self, pose, radius):
        """sgba_set_eq_constraints: |t(pose[k])| = radius[k]; an empty set removes them."""
        pose = np.ascontiguousarray(pose, dtype=np.int32).reshape(-1)
        radius = np.ascontiguousarray(radius, dtype=np.float64).reshape(-1)
        n = pose.shape[0]
        check(lib().sgba_set_eq_constraints(self._h, n, pose.ctypes.data_as(C.POINTER(C.c_int32)) if n else None,
                                            _dptr(radius) if n else None))

    def covariance_prepare(self):
        """sgba_covariance_prepare: the undamped H at the current variables, S,
        its LDL^T and its inverse (or min-norm pseudo-inverse) on the device."""
        info = CovInfo()
        check(lib().sgba_covariance_prepare(self._h, C.byref(info)))
        return info

    def covariance_release(self):
        check(lib().sgba_covariance_release(self._h))

    def covariance_blocks(self, queries, mode=QUERY_COVARIANCE):
        """Block queries ((row_kind, row_index), (col_kind, col_index)) in one
        launch: a (rows, cols) array per query, None where the reference
        returns None (constant variable, index out of range)."""
        n = len(queries)
        qs = (CovQuery * max(n, 1))()
        for k, ((rk, ri), (ck, ci)) in enumerate(queries):
            qs[k] = CovQuery(int(rk), int(ri), int(ck), int(ci))
        out = np.zeros((max(n, 1), 36))
        dims = np.zeros((max(n, 1), 2), dtype=np.int32)
        check(lib().sgba_covariance_blocks(self._h, int(mode), n, qs, _dptr(out), _ipt(dims)))
        res = []
        for k in range(n):
            r, c = int(dims[k, 0]), int(dims[k, 1])
            res.append(None if r <= 0 else out[k, :r * c].reshape(r, c).copy())
        return res

    def covariance_block(self, row, col):
        return self.covariance_blocks([(row, col)])[0]

    def precision_block(self, row, col):
        return self.covariance_blocks([(row, col)], QUERY_PRECISION)[0]

    def cost(self):
        c = C.c_double()
        check(lib().sgba_get_cost(self._h, C.byref(c)))
        return c.value

    def layout(self):
        lay = Layout()
        check(lib().sgba_get_layout(self._h, C.byref(lay)))
        return lay

    def export_pattern(self):
        lay = self.layout()
        hr = np.empty(lay.n_h_blocks, dtype=np.int32)
        hc = np.empty(lay.n_h_blocks, dtype=np.int32)
        sr = np.empty(lay.n_s_blocks, dtype=np.int32)
        sc = np.empty(lay.n_s_blocks, dtype=np.int32)
        check(lib().sgba_export_pattern(self._h, _ipt(hr), _ipt(hc), _ipt(sr), _ipt(sc)))
        return (hr, hc), (sr, sc)

    def intrinsics(self):
        """Current fx fy cx cy (then alpha beta for the EUCM camera)."""
        out = np.empty(6 if self.camera_model == CAMERA_EUCM else 4)
        check(lib().sgba_get_intrinsics(self._h, _dptr(out)))
        return out

    def last_system(self):
        lay = self.layout()
        n6 = 6 * lay.n_free_poses + lay.intrinsics_rows
        S = np.empty((n6, n6))
        rhs = np.empty(n6)
        delta = np.empty(n6 + 3 * lay.n_marg_points)
        check(lib().sgba_debug_last_system(self._h, _dptr(S), _dptr(rhs), _dptr(delta)))
        return S, rhs, delta

    def jacobians(self, cam, pt, precision=0):
        """Per-term J_pose (n, 2, 6) and J_point (n, 2, 3) at the current
        variables, as the linearization kernels evaluate them (precision 0:
        FP32, 1: float-float)."""
        cam = np.ascontiguousarray(cam, dtype=np.int32)
        pt = np.ascontiguousarray(pt, dtype=np.int32)
        n = cam.shape[0]
        jp = np.empty((n, 2, 6))
        jm = np.empty((n, 2, 3))
        ip = C.POINTER(C.c_int32)
        check(lib().sgba_debug_jacobians(self._h, n, cam.ctypes.data_as(ip), pt.ctypes.data_as(ip),
                                         int(precision), _dptr(jp), _dptr(jm)))
        return jp, jm

    def set_linear_solver(self, mode, max_iterations=50, tolerance=1e-8, model=None):
        """Reduced-system solver: LINSOLVE_EXACT, LINSOLVE_PCG_BLOCK_JACOBI or
        LINSOLVE_PCG_LEARNED (needs a PcgModel); PCG falls back to the exact
        factorization when it misses the tolerance within max_iterations."""
        cfg = LinearSolverC(int(mode), int(max_iterations), float(tolerance))
        self._model = model  # kept alive while the problem uses it
        check(lib().sgba_set_linear_solver(self._h, C.byref(cfg), model._h if model is not None else None))

    def collect(self, trainset):
        """Append the reduced system of the latest LM step (scaled, with its
        exact solution) to a PcgTrainSet."""
        check(lib().sgba_pcg_collect(self._h, trainset._h))

    def pcg_stats(self):
        st = PcgStats()
        check(lib().sgba_get_pcg_stats(self._h, C.byref(st)))
        return st

    def state_save(self):
        size = C.c_size_t(0)
        check(lib().sgba_state_save(self._h, None, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        check(lib().sgba_state_save(self._h, buf, C.byref(size)))
        return bytes(buf.raw[: size.value])

    def state_load(self, blob):
        buf = C.create_string_buffer(blob, len(blob))
        check(lib().sgba_state_load(self._h, buf, len(blob)))

    def set_profiling(self, on):
        check(lib().sgba_set_profiling(self._h, 1 if on else 0))

    def profile(self):
        p = Profile()
        check(lib().sgba_get_profile(self._h, C.byref(p)))
        return p

    def bench_iterations(self, iters, flush_l2=True):
        """Device ms summed over `iters` LM iterations, and the kernel launch count."""
        ms = C.c_double()
        n = C.c_int64()
        check(lib().sgba_bench_iterations(self._h, int(iters), 1 if flush_l2 else 0, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def bench_kernel(self, kernel, reps, flush_l2=True):
        """Mean device ms of one launch of `kernel` (sgba_kernel_id) on the current data."""
        ms = C.c_double()
        check(lib().sgba_bench_kernel(self._h, int(kernel), int(reps), 1 if flush_l2 else 0, C.byref(ms)))
        return ms.value


def create_problems(datas, device=0, threads=None, **kw):
    """Problem for each of many inputs (local windows), created concurrently on
    host threads: sgba_problem_create is thread-safe, and each problem's set-up
    (host plan, uploads, the Schur pattern on its own stream) is independent.
    The problems come back in input order; if one fails, the others are closed
    and the first error is raised."""
    import concurrent.futures as cf

    datas = list(datas)
    if threads is None:
        threads = min(16, os.cpu_count() or 1)
    if threads <= 1 or len(datas) < 2:
        return [Problem(d, device=device, **kw) for d in datas]
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        futs = [ex.submit(Problem, d, device, **kw) for d in datas]
        out, err = [], None
        for f in futs:
            try:
                out.append(f.result())
            except Exception as e:  # noqa: BLE001 (re-raised below)
                out.append(None)
                err = err or e
    if err is not None:
        for p in out:
            if p is not None:
                p.close()
        raise err
    return out


def batch_optimize(problems, params):
    """sgba_batch_optimize over Problem handles (independent windows).

    Returns one (records, termination, device_ms, final_cost, status) tuple per
    window.  Eligible windows run batched (each kernel of an LM iteration
    launched once for all of them); the others concurrently, one stream each."""
    n = len(problems)
    cap = max(1, int(params.num_iterations))
    handles = (C.c_void_p * n)(*[p._h for p in problems])
    recs = (IterRecord * (n * cap))()
    res = (WindowResult * n)()
    check(lib().sgba_batch_optimize(handles, n, C.byref(opt_params_c(params)), recs, cap, res))
    out = []
    for w in range(n):
        r = res[w]
        k = min(r.n_records, cap)
        out.append(([recs[w * cap + i] for i in range(k)], r.termination, r.ms, r.final_cost, r.status))
    return out


def batch_last_stats():
    """sgba_batch_last_stats: the batched path of the last batch_optimize call
    (windows, schedule, autotuner state, kernel launches, device time)."""
    st = BatchStats()
    check(lib().sgba_batch_last_stats(C.byref(st)))
    return dict(batched_windows=st.batched_windows, schedule=st.schedule, groups=st.groups, order=st.order,
                tuned=bool(st.tuned), kernel_launches=int(st.kernel_launches), ms=float(st.ms),
                schedule_ms=[float(x) for x in st.schedule_ms])


TRAINED_WEIGHTS = os.path.join(_HERE, "weights", "pcg_mpnn_loop.npz")


class PcgModel:
    """Parameters of the learned block preconditioner (sgba_pcg_model)."""

    @classmethod
    def load(cls, path=TRAINED_WEIGHTS, device=0):
        """A model with the parameters saved by pcg_train.py (an .npz with
        `params`, FP32)."""
        with np.load(path) as z:
            params = np.asarray(z["params"], dtype=np.float32)
        return cls(device=device, params=params)

    def __init__(self, device=0, seed=20261203, params=None):
        h = C.c_void_p()
        check(lib().sgba_pcg_model_create(int(device), C.c_uint64(seed), C.byref(h)))
        self._h = h
        if params is not None:
            self.set_params(params)

    @staticmethod
    def num_params():
        return int(lib().sgba_pcg_num_params())

    def set_params(self, params):
        w = np.ascontiguousarray(params, dtype=np.float32).ravel()
        check(lib().sgba_pcg_model_set_params(self._h, w.ctypes.data_as(C.POINTER(C.c_float)), w.shape[0]))

    def params(self):
        w = np.empty(self.num_params(), np.float32)
        check(lib().sgba_pcg_model_get_params(self._h, w.ctypes.data_as(C.POINTER(C.c_float)), w.shape[0]))
        return w

    def close(self):
        if getattr(self, "_h", None):
            lib().sgba_pcg_model_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PcgTrainSet:
    """Reduced systems with exact solutions for training the preconditioner
    (sgba_pcg_trainset)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().sgba_pcg_trainset_create(int(device), C.byref(h)))
        self._h = h

    def __len__(self):
        return int(lib().sgba_pcg_trainset_size(self._h))

    def add(self, nf, s_rows, s_cols, blocks, b, x):
        """A Jacobi-scaled system from host arrays (lower blocks, n x 36)."""
        r = np.ascontiguousarray(s_rows, dtype=np.int32)
        c = np.ascontiguousarray(s_cols, dtype=np.int32)
        bl = np.ascontiguousarray(blocks, dtype=np.float64).reshape(-1, 36)
        bv = np.ascontiguousarray(b, dtype=np.float64)
        xv = np.ascontiguousarray(x, dtype=np.float64)
        check(lib().sgba_pcg_trainset_add(self._h, int(nf), r.shape[0], _ipt(r), _ipt(c), _dptr(bl), _dptr(bv),
                                          _dptr(xv)))

    def loss_grad(self, model, index, with_grad=True):
        loss = C.c_double()
        if with_grad:
            g = np.empty(PcgModel.num_params(), np.float32)
            check(lib().sgba_pcg_loss_grad(model._h, self._h, int(index), C.byref(loss),
                                           g.ctypes.data_as(C.POINTER(C.c_float)), g.shape[0]))
            return loss.value, g
        check(lib().sgba_pcg_loss_grad(model._h, self._h, int(index), C.byref(loss), None, 0))
        return loss.value

    def train(self, model, epochs, batch=8, learning_rate=1e-3, seed=1):
        losses = np.zeros(int(epochs))
        tp = PcgTrainParams(int(epochs), int(batch), float(learning_rate), C.c_uint64(seed))
        check(lib().sgba_pcg_train(model._h, self._h, C.byref(tp), _dptr(losses)))
        return losses

    def evaluate(self, index, mode, model=None, max_iterations=50, tolerance=1e-8):
        """PCG on stored system `index`: (iterations, relative residual, status)."""
        it = C.c_int32()
        rr = C.c_double()
        st = C.c_int32()
        check(lib().sgba_pcg_evaluate(model._h if model is not None else None, self._h, int(index), int(mode),
                                      int(max_iterations), float(tolerance), C.byref(it), C.byref(rr), C.byref(st)))
        return it.value, rr.value, st.value

    def close(self):
        if getattr(self, "_h", None):
            lib().sgba_pcg_trainset_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
