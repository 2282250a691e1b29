"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the learned preconditioner
(forward, loss, backward) used to check the CUDA kernels' outputs and gradients.  The
reference has no learned component, so this oracle is pinned by its own central finite
differences and by symmetry / positivity checks (tests/test_gnn_oracle.py), not by the
reference.

Network, the same definition as the library (free nodes, width 64, 3 layers):
  x = D^-1/2 r
  S x:  h0 = x We^T;   h <- h + [h ; A h] Wl^T   (A: mean over mesh-graph neighbours)
  M(r) = D^-1/2 (c x + S^T S x),   c = exp(log c)
S is linear, so M is a fixed symmetric positive definite operator.  Layer weights may be
rounded to BF16 to match the device's weight copies.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

H, FIN, NL = 64, 3, 3
AIN = 2 * H
OFF_WE = 0
OFF_L = OFF_WE + H * FIN
L_STRIDE = H * AIN
OFF_C = OFF_L + NL * L_STRIDE
NPARAM = OFF_C + 1


def bf16_round(a):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def free_graph(tets_shuffled, n_bcs, n_nodes):
    """Mean-aggregation matrix over the free-node graph (edges of the tets), in the
    reference's reshuffled free-node order."""
    t = np.asarray(tets_shuffled, dtype=np.int64)
    a = t[:, [0, 0, 0, 1, 1, 2]].ravel()
    b = t[:, [1, 2, 3, 2, 3, 3]].ravel()
    n = n_nodes - n_bcs
    keep = (a >= n_bcs) & (b >= n_bcs)
    i, j = a[keep] - n_bcs, b[keep] - n_bcs
    A = sp.coo_matrix((np.ones(2 * i.size), (np.concatenate([i, j]), np.concatenate([j, i]))), shape=(n, n)).tocsr()
    A.sum_duplicates()
    A.data[:] = 1.0  # duplicates collapse to one edge
    deg = np.asarray(A.sum(axis=1)).ravel()
    return (sp.diags(1.0 / np.maximum(deg, 1.0)) @ A).tocsr()


def unpack(p, bf16_layers=True):
    p = np.asarray(p, dtype=np.float64)
    We = p[OFF_WE:OFF_L].reshape(H, FIN)
    Ws = []
    for l in range(NL):
        W = p[OFF_L + l * L_STRIDE:OFF_L + (l + 1) * L_STRIDE].reshape(H, AIN)
        Ws.append(bf16_round(W) if bf16_layers else W)
    return We, Ws, float(np.exp(p[OFF_C]))


def s_forward(We, Ws, Am, x):
    """h3 = S x and the layer inputs a_l = [h_l ; A h_l]."""
    h = x @ We.T
    acts = []
    for W in Ws:
        a = np.concatenate([h, Am @ h], axis=1)
        acts.append(a)
        h = h + a @ W.T
    return h, acts


def s_transpose(We, Ws, Am, g):
    """S^T g (g: n x H) -> n x 3."""
    for W in reversed(Ws):
        ga = g @ W
        g = g + ga[:, :H] + Am.T @ ga[:, H:]
    return g @ We


def s_weight_grad(We, Ws, Am, x, cot):
    """Gradient of <cot, S x> with respect to (We, W_1..W_NL), flattened like the parameters."""
    _, acts = s_forward(We, Ws, Am, x)
    g = np.zeros(OFF_C)
    G = cot
    for l in reversed(range(NL)):
        W = Ws[l]
        g[OFF_L + l * L_STRIDE:OFF_L + (l + 1) * L_STRIDE] = (G.T @ acts[l]).ravel()
        ga = G @ W
        G = G + ga[:, :H] + Am.T @ ga[:, H:]
    g[OFF_WE:OFF_L] = (G.T @ x).ravel()
    return g


def forward(p, Am, r, dinv, bf16_layers=True):
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    sd = np.sqrt(np.asarray(dinv, dtype=np.float64).reshape(-1, 3))
    We, Ws, c = unpack(p, bf16_layers)
    x = sd * r
    h3, _ = s_forward(We, Ws, Am, x)
    return (sd * (c * x + s_transpose(We, Ws, Am, h3))).ravel()


def loss_grad(p, Am, r, dinv, e, Kmul, bf16_layers=True, mode="energy"):
    """Loss and gradient; Kmul(v) = K v (flat).
    energy:   ||M(r) - e||_K^2 / (e.r);   residual: ||K M(r) - r||^2 / (r.r)."""
    r = np.asarray(r, dtype=np.float64).ravel()
    out = forward(p, Am, r, dinv, bf16_layers)
    if mode == "energy":
        d = out - np.ravel(e)
        q = Kmul(d)
        cc = float(np.ravel(e) @ r)
        L = float(d @ q) / cc
        Go = 2.0 * q / cc
    else:
        d = Kmul(out) - r
        cc = float(r @ r)
        L = float(d @ d) / cc
        Go = 2.0 * Kmul(d) / cc
    We, Ws, c = unpack(p, bf16_layers)
    sd = np.sqrt(np.asarray(dinv, dtype=np.float64).reshape(-1, 3))
    x = sd * r.reshape(-1, 3)
    gy = sd * Go.reshape(-1, 3)
    hx, _ = s_forward(We, Ws, Am, x)
    hg, _ = s_forward(We, Ws, Am, gy)
    g = np.zeros(NPARAM)
    g[:OFF_C] = s_weight_grad(We, Ws, Am, x, hg) + s_weight_grad(We, Ws, Am, gy, hx)
    g[OFF_C] = c * float(np.sum(gy * x))
    return L, g


def poly_coefficients(p, bf16_layers=True):
    """The network folded into its polynomial form.  S is linear and the feature maps act on
    the right while A acts on the node index, so they commute:
        S x = sum_k (A^k x) T_k,   T_k = We^T C_k,   prod_l (P_l + A Q_l) = sum_k A^k C_k,
        P_l = I + Wa_l^T,  Q_l = Wb_l^T  (Wl = [Wa | Wb]),
    and  S^T S x = sum_{j,k} (A^T)^j (A^k x) G_kj  with  G_kj = T_k T_j^T  (3 x 3).
    Returns G (4, 4, 3, 3) and c."""
    We, Ws, c = unpack(p, bf16_layers)
    C = [np.eye(H)]
    for W in Ws:
        P = np.eye(H) + W[:, :H].T
        Q = W[:, H:].T
        nxt = [np.zeros((H, H)) for _ in range(len(C) + 1)]
        for k, Ck in enumerate(C):
            nxt[k] += Ck @ P
            nxt[k + 1] += Ck @ Q
        C = nxt
    T = [We.T @ Ck for Ck in C]
    G = np.array([[T[k] @ T[j].T for j in range(NL + 1)] for k in range(NL + 1)])
    return G, c


def forward_poly(p, Am, r, dinv, bf16_layers=True):
    """M(r) evaluated through the folded polynomial (equal to ``forward`` in exact arithmetic)."""
    G, c = poly_coefficients(p, bf16_layers)
    sd = np.sqrt(np.asarray(dinv, dtype=np.float64).reshape(-1, 3))
    x = sd * np.asarray(r, dtype=np.float64).reshape(-1, 3)
    y = [x]
    for _ in range(NL):
        y.append(Am @ y[-1])
    w = [sum(y[k] @ G[k, j] for k in range(NL + 1)) for j in range(NL + 1)]
    u = w[NL]
    for j in range(NL - 1, -1, -1):
        u = Am.T @ u + w[j]
    return (sd * (c * x + u)).ravel()
