"""The FP64 restatement of the learned preconditioner (oracle/pcg_mpnn.py):
its hand-written backward pass against central differences, and the loss at
the block-Jacobi point.  CPU only."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pcg_mpnn as M  # noqa: E402
from pcg_systems import random_system  # noqa: E402


def _params(seed, scale=0.2):
    rng = np.random.default_rng(seed)
    _, n = M.layout()
    return rng.normal(size=n) * scale


def test_gradient_matches_central_differences():
    nf = 6
    rows, cols, blocks, b, x = random_system(nf, seed=3)
    p = _params(5)
    loss, g = M.gradient(p, nf, rows, cols, blocks, b, x, bf16=False)
    rng = np.random.default_rng(7)
    idx = rng.choice(p.shape[0], size=60, replace=False)
    lay, _ = M.layout()
    # every parameter block is probed at least once
    for name, (o, s) in lay.items():
        idx = np.append(idx, o + int(np.prod(s)) // 2)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = M.forward(p + e, nf, rows, cols, blocks, b, x, bf16=False)
        lm, _ = M.forward(p - e, nf, rows, cols, blocks, b, x, bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])


def test_block_jacobi_point_and_perfect_preconditioner():
    """L = 0 gives block-Jacobi; for a block-diagonal S block-Jacobi is exact
    (loss 0), and the loss does not change when P is scaled."""
    nf = 4
    rows, cols, blocks, b, x = random_system(nf, seed=11, band=0)
    keep = rows == cols  # drop the loop closure: block-diagonal
    rows, cols, blocks = rows[keep], cols[keep], blocks[keep]
    A = np.zeros((6 * nf, 6 * nf))
    for j, bl in zip(rows, blocks):
        A[6 * j:6 * j + 6, 6 * j:6 * j + 6] = bl.reshape(6, 6)
    x = np.linalg.solve(A, b)
    p = np.zeros(M.layout()[1])
    loss, _ = M.forward(p, nf, rows, cols, blocks, b, x, bf16=False)
    assert abs(loss) < 1e-12
    # L = t I for every pose: P = (1 + t^2) x block-Jacobi, same loss
    rows2, cols2, blocks2, b2, x2 = random_system(nf, seed=12)
    lay, _ = M.layout()
    o, _ = lay["b_o"]
    l0, _ = M.forward(p, nf, rows2, cols2, blocks2, b2, x2, bf16=False)
    p2 = p.copy()
    p2[o + np.array([0, 2, 5, 9, 14, 20])] = 0.7
    l1, _ = M.forward(p2, nf, rows2, cols2, blocks2, b2, x2, bf16=False)
    assert abs(l0 - l1) < 1e-12 and 0.0 < l0 < 1.0
