"""Reduced systems for the learned-preconditioner tests: small random SPD
block systems (CPU) and the Jacobi-scaled reduced system of a GPU problem's
latest LM step (through sgba_debug_last_system and sgba_export_pattern)."""
import numpy as np


def random_system(nf, seed, band=2):
    """A Jacobi-scaled SPD block system with a band of `band` blocks plus a
    loop closure, its lower blocks (pattern order), b and the solution."""
    rng = np.random.default_rng(seed)
    pat = set()
    for j in range(nf):
        for k in range(max(0, j - band), j + 1):
            pat.add((j, k))
    pat.add((nf - 1, 0))
    pat = sorted(pat)
    n6 = 6 * nf
    A = np.zeros((n6, n6))
    for (j, k) in pat:
        if j != k:
            X = rng.normal(size=(6, 6)) * 0.3
            A[6 * j:6 * j + 6, 6 * k:6 * k + 6] = X
            A[6 * k:6 * k + 6, 6 * j:6 * j + 6] = X.T
    for j in range(nf):
        Q = rng.normal(size=(6, 6))
        A[6 * j:6 * j + 6, 6 * j:6 * j + 6] = Q @ Q.T + 6.0 * np.eye(6)
    # diagonally dominant enough to be SPD, then Jacobi-scaled
    w = np.linalg.eigvalsh(A)
    if w[0] <= 0:
        A += (1e-2 - w[0]) * np.eye(n6)
    d = 1.0 / np.sqrt(np.diag(A))
    A = A * d[:, None] * d[None, :]
    rows = np.array([j for j, k in pat], np.int32)
    cols = np.array([k for j, k in pat], np.int32)
    blocks = np.stack([A[6 * j:6 * j + 6, 6 * k:6 * k + 6].ravel() for j, k in pat])
    b = rng.normal(size=n6)
    x = np.linalg.solve(A, b)
    return rows, cols, blocks, b, x


def scaled_system(gp):
    """The latest step's reduced system of a native.Problem, Jacobi-scaled:
    (nf, lower block rows, cols, blocks, b~, x~ solved in f64)."""
    S, rhs, _ = gp.last_system()
    lay = gp.layout()
    _, (sr, sc) = gp.export_pattern()
    d = 1.0 / np.sqrt(np.diag(S))
    A = S * d[:, None] * d[None, :]
    b = rhs * d
    x = np.linalg.solve(A, b)
    blocks = np.stack([A[6 * j:6 * j + 6, 6 * k:6 * k + 6].ravel() for j, k in zip(sr, sc)])
    return lay.n_free_poses, sr, sc, blocks, b, x
