"""The LM step of the GPU path against an FP64 LDL^T solve of the same reduced
camera system (test and benchmark infrastructure).

For each step the GPU exports its reduced system S, the reduced right-hand
side and its step (sgba_debug_last_system).  The FP64 reference step solves
S x = rhs by a sparse LU in double precision (SuperLU through scipy; numpy's
dense solve for small systems).  With one constant camera and no constant
point the scale gauge is free: the exact damped step is defined only up to
the gauge projection the GPU applies, so the error is measured outside the
gauge direction v = [0; t_j - c] of the free poses (c the constant camera's
centre):

    err = |P(dx_gpu) - P(dx_f64)| / |P(dx_f64)|,   P(x) = x - v (v . x)

The reference solves this system with its block LDL^T
(crates/sophus_solver/src/ldlt/schur_ldlt.rs:756-812,
 crates/sophus_solver/src/ldlt/block_sparse_ldlt.rs:99-190).
"""
import numpy as np


def f64_solve(S, rhs):
    n = S.shape[0]
    if n <= 1200:
        return np.linalg.solve(S, rhs)
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    A = sp.csc_matrix(S)
    return spla.splu(A, permc_spec="COLAMD").solve(rhs)


def gauge_direction(prob, poses, n6):
    const = np.where(prob.pose_const == 1)[0]
    if len(const) != 1 or (prob.point_const is not None and np.any(prob.point_const)):
        return None
    free = np.where(prob.pose_const == 0)[0]
    c = poses[const[0], 4:]
    v = np.zeros(n6)
    for k, j in enumerate(free):
        v[6 * k + 3:6 * k + 6] = poses[j, 4:] - c
    return v / np.linalg.norm(v)


def step_errors(gp, prob, n_steps):
    """Run n_steps LM iterations on an initialised native.Problem and return
    the step error of each (steps whose solve was skipped are left out)."""
    errs = []
    for _ in range(n_steps):
        poses, _ = gp.variables()
        rec = gp.step()
        if not np.isfinite(rec.max_step):
            continue
        S, rhs, delta = gp.last_system()
        n6 = S.shape[0]
        x64 = f64_solve(S, rhs)
        v = gauge_direction(prob, poses, n6)
        xf = delta[:n6]
        if v is not None:
            xf = xf - v * (v @ xf)
            x64 = x64 - v * (v @ x64)
        errs.append(float(np.linalg.norm(xf - x64) / np.linalg.norm(x64)))
        del S
    return errs
