"""FP64 CPU restatement of the learned block preconditioner and its training
loss (test infrastructure: the checker of the GPU forward and backward
kernels in sophus-rs_gb300/csrc/sgba_pcg_net.cu; never on the product path).

The reference has no learned preconditioner: it solves the reduced camera
system only exactly (crates/sophus_solver/src/ldlt/schur_ldlt.rs:536-812).
This file restates, in numpy float64, what the library computes on the GPU:

  node features f_j from the Jacobi-scaled reduced system S~ (lower 6x6
  blocks): the 15 strictly-upper entries of the diagonal block B_j, the log of
  the diagonal of B_j^-1, log(1 + degree), and the sum, maximum, Euclidean
  norm and mean of the neighbouring blocks' Frobenius norms w_jk;
  h0 = relu(W_in f + b_in);  m_j = sum_k w_jk h_k / sum_k w_jk;
  h' = h + relu(W_s h + W_m m + b)  (3 layers);  L_j = W_o h + b_o;
  P_j = Ci_j^T (I + L_j L_j^T) Ci_j,  Ci_j = chol(B_j)^-1;
  y = P b,  loss = min_a |x* - a y|^2_S~ / x*^T b = 1 - (y^T b)^2 / (x*^T b  y^T S~ y)
  (the error left by one preconditioned step of optimal length from 0).

gradient() is a hand-written backward pass of the same graph; it is itself
checked against central differences in the tests.
"""
import numpy as np

F = 32
H = 64
LAYERS = 3
OUT = 21


def layout():
    """Offsets (start, shape) of the parameter blocks, in the library's order."""
    off = 0
    out = {}

    def take(name, shape):
        nonlocal off
        n = int(np.prod(shape))
        out[name] = (off, shape)
        off += n

    take("W_in", (H, F))
    take("b_in", (H,))
    for l in range(LAYERS):
        take("W_s%d" % l, (H, H))
        take("W_m%d" % l, (H, H))
        take("b%d" % l, (H,))
    take("W_o", (OUT, H))
    take("b_o", (OUT,))
    return out, off


def unpack(params):
    lay, n = layout()
    params = np.asarray(params, dtype=np.float64)
    assert params.shape == (n,)
    return {k: params[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def bf16_round(params):
    """Round FP32 parameters to BF16 (nearest even), as the kernels read them."""
    u = np.ascontiguousarray(params, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def rows(nf, s_rows, s_cols):
    """Full block rows: per row, (column, block id, transposed) by column."""
    out = [[] for _ in range(nf)]
    for b, (j, k) in enumerate(zip(s_rows, s_cols)):
        out[j].append((k, b, False))
        if j != k:
            out[k].append((j, b, True))
    return [sorted(r) for r in out]


def block(blocks, b, tr):
    B = blocks[b].reshape(6, 6)
    return B.T if tr else B


def features(nf, R, blocks):
    f = np.zeros((nf, F))
    W = []  # per row: [(neighbour, w)]
    for j in range(nf):
        nb = [(k, np.sqrt(np.sum(blocks[b] ** 2))) for (k, b, tr) in R[j] if k != j]
        W.append(nb)
        B = [block(blocks, b, tr) for (k, b, tr) in R[j] if k == j][0]
        iu = np.triu_indices(6, 1)
        f[j, :15] = B[iu]
        Ci = np.linalg.inv(np.linalg.cholesky(B))
        f[j, 15:21] = np.log(np.maximum(np.sum(Ci ** 2, axis=0), 1e-30))
        w = np.array([x for _, x in nb])
        deg = len(nb)
        f[j, 21] = np.log1p(deg)
        f[j, 22] = w.sum() if deg else 0.0
        f[j, 23] = w.max() if deg else 0.0
        f[j, 24] = np.sqrt(np.sum(w ** 2)) if deg else 0.0
        f[j, 25] = w.sum() / deg if deg else 0.0
    return f.astype(np.float32).astype(np.float64), W


def forward(params, nf, s_rows, s_cols, blocks, b, xs, bf16=True):
    """Loss and the intermediates of the backward pass."""
    p = unpack(bf16_round(params) if bf16 else params)
    blocks = np.asarray(blocks, dtype=np.float64).reshape(-1, 36)
    R = rows(nf, s_rows, s_cols)
    f, W = features(nf, R, blocks)
    pre0 = f @ p["W_in"].T + p["b_in"]
    h = [np.maximum(pre0, 0.0)]
    Ms, Us = [], []
    for l in range(LAYERS):
        M = np.zeros((nf, H))
        for j in range(nf):
            ws = sum(w for _, w in W[j])
            if ws > 0:
                M[j] = sum(w * h[l][k] for k, w in W[j]) / ws
        U = h[l] @ p["W_s%d" % l].T + M @ p["W_m%d" % l].T + p["b%d" % l]
        Ms.append(M)
        Us.append(U)
        h.append(h[l] + np.maximum(U, 0.0))
    Lv = h[-1] @ p["W_o"].T + p["b_o"]
    tril = np.tril_indices(6)
    Ps, Cis, Ls = [], [], []
    y = np.zeros(6 * nf)
    for j in range(nf):
        B = [block(blocks, bb, tr) for (k, bb, tr) in R[j] if k == j][0]
        Ci = np.linalg.inv(np.linalg.cholesky(B))
        L = np.zeros((6, 6))
        L[tril] = Lv[j]
        P = Ci.T @ (np.eye(6) + L @ L.T) @ Ci
        Ps.append(P)
        Cis.append(Ci)
        Ls.append(L)
        y[6 * j:6 * j + 6] = P @ b[6 * j:6 * j + 6]
    Sy = matvec(nf, R, blocks, y)
    den = float(xs @ b)
    q = float(y @ Sy)
    nn = float(y @ b)
    loss = 1.0 - nn * nn / (den * q)
    ctx = dict(p=p, R=R, W=W, f=f, h=h, Ms=Ms, Us=Us, Ls=Ls, Cis=Cis, Sy=Sy, den=den, q=q, nn=nn, b=b, nf=nf)
    return loss, ctx


def matvec(nf, R, blocks, x):
    y = np.zeros(6 * nf)
    for j in range(nf):
        for (k, bb, tr) in R[j]:
            y[6 * j:6 * j + 6] += block(blocks, bb, tr) @ x[6 * k:6 * k + 6]
    return y


def gradient(params, nf, s_rows, s_cols, blocks, b, xs, bf16=True):
    """Loss and d loss / d params (float64), by the chain rule of forward()."""
    loss, c = forward(params, nf, s_rows, s_cols, blocks, b, xs, bf16)
    p, W, h, Ms, Us = c["p"], c["W"], c["h"], c["Ms"], c["Us"]
    lay, n = layout()
    g = {k: np.zeros(s) for k, (o, s) in lay.items()}
    tril = np.tril_indices(6)
    dLv = np.zeros((nf, OUT))
    cc = 2.0 * c["nn"] / (c["den"] * c["q"])
    astar = c["nn"] / c["q"]
    for j in range(nf):
        bj = b[6 * j:6 * j + 6]
        gj = cc * (astar * c["Sy"][6 * j:6 * j + 6] - bj)
        Ci = c["Cis"][j]
        Gm = Ci @ np.outer(gj, bj) @ Ci.T
        D = (Gm + Gm.T) @ c["Ls"][j]
        dLv[j] = D[tril]
    g["W_o"] += dLv.T @ h[-1]
    g["b_o"] += dLv.sum(axis=0)
    dH = dLv @ p["W_o"]
    for l in range(LAYERS - 1, -1, -1):
        dU = dH * (Us[l] > 0)
        g["W_s%d" % l] += dU.T @ h[l]
        g["W_m%d" % l] += dU.T @ Ms[l]
        g["b%d" % l] += dU.sum(axis=0)
        dM = dU @ p["W_m%d" % l]
        dHl = dH + dU @ p["W_s%d" % l]
        for i in range(nf):  # M_i = sum_k w_ik h_k / sum_k w_ik
            ws = sum(w for _, w in W[i])
            if ws > 0:
                for k, w in W[i]:
                    dHl[k] += (w / ws) * dM[i]
        dH = dHl
    dpre = dH * (h[0] > 0)
    g["W_in"] += dpre.T @ c["f"]
    g["b_in"] += dpre.sum(axis=0)
    out = np.zeros(n)
    for k, (o, s) in lay.items():
        out[o:o + int(np.prod(s))] = g[k].ravel()
    return loss, out
