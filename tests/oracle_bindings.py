"""ctypes bindings of the CPU oracle (oracle/sgba_oracle.h).

Test infrastructure only: used by the tests, smoke() and the CPU-baseline
leg of bench.py as the checker / timed CPU restatement of the reference.
"""
import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "libsgba_oracle.so")
_lib = None


class OraParams(C.Structure):
    _fields_ = [
        ("num_iterations", C.c_int32),
        ("initial_lm_damping", C.c_double),
        ("function_tolerance", C.c_double),
        ("gradient_tolerance", C.c_double),
        ("parameter_tolerance", C.c_double),
        ("max_consecutive_rejects", C.c_int64),
        ("emulate_fp32", C.c_int32),
    ]


class OraRecord(C.Structure):
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


class OraProblem(C.Structure):
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
        ("intrinsics_free", C.c_int32),
        ("camera_model", C.c_int32),
        ("eucm_alpha_beta", C.c_double * 2),
        ("n_eq", C.c_int32),
        ("eq_pose", C.POINTER(C.c_int32)),
        ("eq_radius", C.POINTER(C.c_double)),
        ("n_prior", C.c_int32),
        ("prior_pose", C.POINTER(C.c_int32)),
        ("prior_mean", C.POINTER(C.c_double)),
        ("prior_precision", C.POINTER(C.c_double)),
        ("n_edge", C.c_int32),
        ("edge_pose", C.POINTER(C.c_int32)),
        ("edge_mn", C.POINTER(C.c_double)),
    ]


CAMERA_PINHOLE = 0
CAMERA_EUCM = 1


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("oracle library not built: %s" % LIB)
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        L.ora_se3_exp.argtypes = [dp, dp]
        L.ora_se3_mul.argtypes = [dp, dp, dp]
        L.ora_se3_inverse.argtypes = [dp, dp]
        L.ora_eval_term.argtypes = [dp, dp, dp, dp, C.c_double, dp, dp, dp, dp, dp]
        L.ora_eval_term_dual.argtypes = [dp, dp, dp, dp, dp, dp]
        L.ora_block_ldlt_solve.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        L.ora_total_cost.argtypes = [C.POINTER(OraProblem), C.c_int]
        L.ora_total_cost.restype = C.c_double
        L.ora_dense_system.argtypes = [C.POINTER(OraProblem), C.c_double, dp, dp]
        L.ora_dense_system.restype = C.c_int64
        L.ora_schur_step.argtypes = [C.POINTER(OraProblem), C.c_double, C.c_int, C.c_int, dp, dp, dp]
        L.ora_optimize.argtypes = [C.POINTER(OraProblem), C.POINTER(OraParams), C.c_int,
                                   C.POINTER(OraRecord), C.c_int, C.POINTER(C.c_int), dp, dp]
        L.ora_optimize_ex.argtypes = [C.POINTER(OraProblem), C.POINTER(OraParams), C.c_int,
                                      C.POINTER(OraRecord), C.c_int, C.POINTER(C.c_int), dp, dp, dp]
        L.ora_eval_term_intrinsics.argtypes = [dp, dp, dp, dp]
        L.ora_eval_term_ex.argtypes = [dp, dp, dp, C.c_int32, dp, dp, dp, dp, dp]
        L.ora_covariance_block.argtypes = [C.POINTER(OraProblem), C.c_int32, C.c_int32, C.c_int32, C.c_int32, dp,
                                           C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.ora_eq_eval.argtypes = [C.POINTER(OraProblem), dp, dp, dp]
        L.ora_eval_prior.argtypes = [dp, dp, dp, dp, dp, dp]
        L.ora_se3_log.argtypes = [dp, dp]
        L.ora_eval_edge.argtypes = [dp, dp, dp, dp, dp, dp, dp]
        L.ora_min_norm_pinv.argtypes = [C.c_int, C.c_int, dp, dp]
        L.ora_schur_kkt_step.argtypes = [C.POINTER(OraProblem), C.c_double, dp, C.c_int, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Keep:
    pass


def problem_struct(prob):
    k = _Keep()
    k.poses = np.ascontiguousarray(prob.poses, dtype=np.float64)
    k.points = np.ascontiguousarray(prob.points, dtype=np.float64)
    k.obs_cam = np.ascontiguousarray(prob.obs_cam, dtype=np.int32)
    k.obs_pt = np.ascontiguousarray(prob.obs_pt, dtype=np.int32)
    k.obs_uv = np.ascontiguousarray(prob.obs_uv, dtype=np.float64)
    pc = getattr(prob, "pose_const", None)
    qc = getattr(prob, "point_const", None)
    k.pc = None if pc is None else np.ascontiguousarray(pc, dtype=np.uint8)
    k.qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.uint8)
    s = OraProblem()
    s.n_cam = k.poses.shape[0]
    s.poses = _d(k.poses)
    s.pose_const = k.pc.ctypes.data_as(C.POINTER(C.c_uint8)) if k.pc is not None else None
    s.n_pt = k.points.shape[0]
    s.points = _d(k.points)
    s.point_const = k.qc.ctypes.data_as(C.POINTER(C.c_uint8)) if k.qc is not None else None
    for i in range(4):
        s.intrinsics[i] = float(prob.intrinsics[i])
    s.n_obs = k.obs_cam.shape[0]
    s.obs_cam = k.obs_cam.ctypes.data_as(C.POINTER(C.c_int32))
    s.obs_pt = k.obs_pt.ctypes.data_as(C.POINTER(C.c_int32))
    s.obs_uv = _d(k.obs_uv)
    s.huber_delta = float(prob.huber_delta or 0.0)
    s.intrinsics_free = 1 if getattr(prob, "intrinsics_free", False) else 0
    s.camera_model = int(getattr(prob, "camera_model", CAMERA_PINHOLE))
    ab = getattr(prob, "eucm_alpha_beta", None)
    if ab is None:
        ab = (0.0, 0.0)
    s.eucm_alpha_beta[0] = float(ab[0])
    s.eucm_alpha_beta[1] = float(ab[1])
    # TranslationNormConstraint terms: prob.eq_pose (indices), prob.eq_radius
    ep = getattr(prob, "eq_pose", None)
    k.eq_pose = np.ascontiguousarray(ep if ep is not None else [], dtype=np.int32)
    k.eq_radius = np.ascontiguousarray(getattr(prob, "eq_radius", None) if ep is not None else [], dtype=np.float64)
    assert k.eq_pose.shape == k.eq_radius.shape
    s.n_eq = k.eq_pose.shape[0]
    s.eq_pose = k.eq_pose.ctypes.data_as(C.POINTER(C.c_int32)) if s.n_eq else None
    s.eq_radius = _d(k.eq_radius) if s.n_eq else None
    # Isometry3PriorCostTerm terms: prob.prior_pose, prob.prior_mean (n x 7), prob.prior_precision (n x 6 x 6)
    pp = getattr(prob, "prior_pose", None)
    k.prior_pose = np.ascontiguousarray(pp if pp is not None else [], dtype=np.int32)
    k.prior_mean = np.ascontiguousarray(prob.prior_mean if pp is not None else np.zeros((0, 7)), dtype=np.float64)
    k.prior_precision = np.ascontiguousarray(prob.prior_precision if pp is not None else np.zeros((0, 6, 6)),
                                             dtype=np.float64)
    assert k.prior_mean.shape == (k.prior_pose.shape[0], 7)
    assert k.prior_precision.shape == (k.prior_pose.shape[0], 6, 6)
    s.n_prior = k.prior_pose.shape[0]
    s.prior_pose = k.prior_pose.ctypes.data_as(C.POINTER(C.c_int32)) if s.n_prior else None
    s.prior_mean = _d(k.prior_mean) if s.n_prior else None
    s.prior_precision = _d(k.prior_precision) if s.n_prior else None
    # PoseGraph3CostTerm terms: prob.edge_pose (n x 2), prob.edge_mn (n x 7)
    ee = getattr(prob, "edge_pose", None)
    k.edge_pose = np.ascontiguousarray(ee if ee is not None else np.zeros((0, 2)), dtype=np.int32)
    k.edge_mn = np.ascontiguousarray(prob.edge_mn if ee is not None else np.zeros((0, 7)), dtype=np.float64)
    assert k.edge_pose.shape == (k.edge_pose.shape[0], 2) and k.edge_mn.shape == (k.edge_pose.shape[0], 7)
    s.n_edge = k.edge_pose.shape[0]
    s.edge_pose = k.edge_pose.ctypes.data_as(C.POINTER(C.c_int32)) if s.n_edge else None
    s.edge_mn = _d(k.edge_mn) if s.n_edge else None
    s._keep = k
    return s


def optimize(prob, params, n_threads=1, emulate_fp32=False, with_intrinsics=False):
    """Records, final poses and points (and the final intrinsics when
    with_intrinsics: fx fy cx cy alpha beta, alpha and beta zero for a
    pinhole; they change only when prob.intrinsics_free)."""
    L = lib()
    s = problem_struct(prob)
    mr = params.max_consecutive_rejects
    if mr is None or mr > (1 << 62):
        mr = 1 << 62
    p = OraParams(int(params.num_iterations), float(params.initial_lm_damping), float(params.function_tolerance),
                  float(params.gradient_tolerance), float(params.parameter_tolerance), int(mr),
                  1 if emulate_fp32 else 0)
    cap = max(1, int(params.num_iterations)) + 1
    recs = (OraRecord * cap)()
    n = C.c_int()
    poses = np.empty((s.n_cam, 7))
    points = np.empty((s.n_pt, 3))
    intr = np.empty(6)
    rc = L.ora_optimize_ex(C.byref(s), C.byref(p), int(n_threads), recs, cap, C.byref(n), _d(poses), _d(points),
                           _d(intr))
    if rc != 0:
        raise RuntimeError("oracle optimize failed with %d" % rc)
    out = [recs[i] for i in range(min(n.value, cap))], poses, points
    return out + (intr,) if with_intrinsics else out


def total_cost(prob, n_threads=1):
    s = problem_struct(prob)
    return lib().ora_total_cost(C.byref(s), int(n_threads))


def dense_system(prob, nu):
    L = lib()
    s = problem_struct(prob)
    n = L.ora_dense_system(C.byref(s), float(nu), None, None)
    H = np.zeros((n, n))
    b = np.zeros(n)
    L.ora_dense_system(C.byref(s), float(nu), _d(H), _d(b))
    return H, b


def schur_step(prob, nu, n_threads=1):
    """One Schur solve: returns (delta, S, rhs_bar); raises on failure.
    With free intrinsics S and rhs_bar start with their block, padded to 6."""
    L = lib()
    s = problem_struct(prob)
    n = L.ora_dense_system(C.byref(s), float(nu), None, None)
    nf6 = 6 * int(np.sum(1 - (np.asarray(prob.pose_const) if getattr(prob, "pose_const", None) is not None
                              else np.zeros(prob.poses.shape[0], np.uint8))))
    nf6 += 6 if getattr(prob, "intrinsics_free", False) else 0
    delta = np.zeros(n)
    S = np.zeros((nf6, nf6))
    rhs = np.zeros(nf6)
    rc = L.ora_schur_step(C.byref(s), float(nu), int(n_threads), 0, _d(delta), _d(S), _d(rhs))
    if rc != 0:
        raise RuntimeError("oracle Schur step failed with %d" % rc)
    return delta, S, rhs


def se3_exp(xi):
    out = np.zeros(7)
    lib().ora_se3_exp(_d(np.ascontiguousarray(xi, dtype=np.float64)), _d(out))
    return out


def se3_mul(a, b):
    out = np.zeros(7)
    lib().ora_se3_mul(_d(np.ascontiguousarray(a, float)), _d(np.ascontiguousarray(b, float)), _d(out))
    return out


def se3_inverse(a):
    out = np.zeros(7)
    lib().ora_se3_inverse(_d(np.ascontiguousarray(a, float)), _d(out))
    return out


def eval_term(pose, point, intr, uv, huber):
    r = np.zeros(2)
    jp = np.zeros(12)
    jm = np.zeros(6)
    w = C.c_double()
    c = C.c_double()
    lib().ora_eval_term(_d(np.ascontiguousarray(pose, float)), _d(np.ascontiguousarray(point, float)),
                        _d(np.ascontiguousarray(intr, float)), _d(np.ascontiguousarray(uv, float)),
                        float(huber), _d(r), _d(jp), _d(jm), C.byref(w), C.byref(c))
    return r, jp.reshape(2, 6), jm.reshape(2, 3), w.value, c.value


def eval_term_dual(pose, point, intr, uv):
    jp = np.zeros(12)
    jm = np.zeros(6)
    lib().ora_eval_term_dual(_d(np.ascontiguousarray(pose, float)), _d(np.ascontiguousarray(point, float)),
                             _d(np.ascontiguousarray(intr, float)), _d(np.ascontiguousarray(uv, float)),
                             _d(jp), _d(jm))
    return jp.reshape(2, 6), jm.reshape(2, 3)


def block_ldlt_solve(A, b, bs=6):
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    rc = lib().ora_block_ldlt_solve(A.shape[0], bs, _d(A), _d(b), _d(x))
    if rc != 0:
        raise RuntimeError("block LDLT failed with %d" % rc)
    return x


def eval_term_intrinsics(pose, point, intr):
    """d residual / d (fx, fy, cx, cy), 2x4."""
    j = np.zeros(8)
    lib().ora_eval_term_intrinsics(_d(np.ascontiguousarray(pose, float)), _d(np.ascontiguousarray(point, float)),
                                   _d(np.ascontiguousarray(intr, float)), _d(j))
    return j.reshape(2, 4)


def eval_term_ex(pose, point, intr6, camera_model, uv):
    """Residual, J_pose (2x6), J_point (2x3), J_cam (2 x 4 or 6) of one term."""
    r = np.zeros(2)
    jp = np.zeros(12)
    jm = np.zeros(6)
    jc = np.zeros(12)
    lib().ora_eval_term_ex(_d(np.ascontiguousarray(pose, float)), _d(np.ascontiguousarray(point, float)),
                           _d(np.ascontiguousarray(intr6, float)), int(camera_model),
                           _d(np.ascontiguousarray(uv, float)), _d(r), _d(jp), _d(jm), _d(jc))
    nc = 6 if camera_model == CAMERA_EUCM else 4
    return r, jp.reshape(2, 6), jm.reshape(2, 3), jc[:2 * nc].reshape(2, nc)


VAR_INTRINSICS, VAR_POSE, VAR_POINT = 0, 1, 2


def covariance_block(prob, row, col):
    """Covariance block between row = (kind, index) and col = (kind, index)
    (SchurFactor::inverse_block), or None for a variable without a block."""
    s = problem_struct(prob)
    out = np.zeros(36)
    nr, nc = C.c_int32(), C.c_int32()
    rc = lib().ora_covariance_block(C.byref(s), int(row[0]), int(row[1]), int(col[0]), int(col[1]), _d(out),
                                    C.byref(nr), C.byref(nc))
    if rc == -1:
        return None
    if rc != 0:
        raise RuntimeError("oracle covariance failed with %d" % rc)
    return out[:nr.value * nc.value].reshape(nr.value, nc.value)


def eq_eval(prob, poses=None):
    """Residuals c_k = |t(T_k)| - r_k of the problem's TranslationNormConstraint
    terms and their 1x6 Jacobians (left perturbation), at poses (default: the
    problem's)."""
    s = problem_struct(prob)
    P = np.ascontiguousarray(prob.poses if poses is None else poses, dtype=np.float64)
    c = np.zeros(s.n_eq)
    J = np.zeros((s.n_eq, 6))
    lib().ora_eq_eval(C.byref(s), _d(P), _d(c), _d(J))
    return c, J


def schur_kkt_step(prob, nu, lam, n_threads=1):
    """One damped step with the equality constraints: [dx; dlam] (dx in the
    layout of dense_system); raises on failure."""
    L = lib()
    s = problem_struct(prob)
    n = L.ora_dense_system(C.byref(s), float(nu), None, None)
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    assert lam.shape == (s.n_eq,)
    delta = np.zeros(n + s.n_eq)
    rc = L.ora_schur_kkt_step(C.byref(s), float(nu), _d(lam), int(n_threads), _d(delta))
    if rc != 0:
        raise RuntimeError("oracle KKT step failed with %d" % rc)
    return delta


def eval_prior(pose, mean, precision):
    """One Isometry3PriorCostTerm: residual (6), Jacobian (6x6), cost."""
    r = np.zeros(6)
    J = np.zeros((6, 6))
    cost = C.c_double()
    lib().ora_eval_prior(_d(np.ascontiguousarray(pose, dtype=np.float64)),
                         _d(np.ascontiguousarray(mean, dtype=np.float64)),
                         _d(np.ascontiguousarray(precision, dtype=np.float64)), _d(r), _d(J), C.byref(cost))
    return r, J, cost.value


def se3_log(params):
    out = np.zeros(6)
    lib().ora_se3_log(_d(np.ascontiguousarray(params, dtype=np.float64)), _d(out))
    return out


def eval_edge(pose_m, pose_n, m_from_n):
    """One PoseGraph3CostTerm: residual (6), J_m, J_n (6x6 each), cost."""
    r = np.zeros(6)
    Jm = np.zeros((6, 6))
    Jn = np.zeros((6, 6))
    cost = C.c_double()
    f = lambda a: _d(np.ascontiguousarray(a, dtype=np.float64))  # noqa: E731
    lib().ora_eval_edge(f(pose_m), f(pose_n), f(m_from_n), _d(r), _d(Jm), _d(Jn), C.byref(cost))
    return r, Jm, Jn, cost.value


def min_norm_pinv(A, bs=6):
    """(pseudo-inverse, rank) of a symmetric PSD matrix by the min-norm LDL^T."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    out = np.zeros_like(A)
    r = lib().ora_min_norm_pinv(A.shape[0], int(bs), _d(A), _d(out))
    if r < 0:
        raise RuntimeError("oracle pseudo-inverse failed with %d" % r)
    return out, r
