"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the learned preconditioner
(forward, energy-norm loss, backward) used to check the CUDA kernels' outputs and
gradients.  The reference has no learned component, so this oracle is pinned by
its own central finite differences (tests/test_gnn_oracle.py), not by the reference.

Network (free node i, width 64, 3 layers), the same definition as the library:
  z = D^-1 r,  s = rms(z),  x_i = [z_i/s, -log D_i^-1 - mean(-log D^-1), fixed_nb_i, 1]
  h0 = relu(We x + be);  h <- h + relu(Wl [h ; mean_{j~i} h_j] + bl);  M(r) = z + s (Wd h + bd)
Layer weights may be rounded to BF16 to match the device's weight copies.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

H, FIN, NL = 64, 8, 3
AIN = 2 * H
OFF_WE = 0
OFF_BE = OFF_WE + H * FIN
OFF_L = OFF_BE + H
L_STRIDE = H * AIN + H
OFF_WD = OFF_L + NL * L_STRIDE
OFF_BD = OFF_WD + 3 * H
NPARAM = OFF_BD + 3


def bf16_round(a):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def free_graph(tets_shuffled, n_bcs, n_nodes):
    """Mean-aggregation matrix over the free-node graph (edges of the tets) and the
    fixed-neighbour flags, in the reference's reshuffled free-node order."""
    t = np.asarray(tets_shuffled, dtype=np.int64)
    a = t[:, [0, 0, 0, 1, 1, 2]].ravel()
    b = t[:, [1, 2, 3, 2, 3, 3]].ravel()
    n = n_nodes - n_bcs
    fixed_nb = np.zeros(n, dtype=bool)
    af, bf = a >= n_bcs, b >= n_bcs
    fixed_nb[a[af & ~bf] - n_bcs] = True
    fixed_nb[b[bf & ~af] - n_bcs] = True
    keep = af & bf
    i, j = a[keep] - n_bcs, b[keep] - n_bcs
    A = sp.coo_matrix((np.ones(2 * i.size), (np.concatenate([i, j]), np.concatenate([j, i]))), shape=(n, n)).tocsr()
    A.data[:] = 1.0  # duplicates collapse to one edge
    A.sum_duplicates()
    A.data[:] = 1.0
    deg = np.asarray(A.sum(axis=1)).ravel()
    Am = sp.diags(1.0 / np.maximum(deg, 1.0)) @ A
    return Am.tocsr(), fixed_nb


def unpack(p, bf16_layers=True):
    p = np.asarray(p, dtype=np.float64)
    We = p[OFF_WE:OFF_BE].reshape(H, FIN)
    be = p[OFF_BE:OFF_L]
    Ws, bs = [], []
    for l in range(NL):
        o = OFF_L + l * L_STRIDE
        W = p[o:o + H * AIN].reshape(H, AIN)
        Ws.append(bf16_round(W) if bf16_layers else W)
        bs.append(p[o + H * AIN:o + L_STRIDE])
    Wd = p[OFF_WD:OFF_BD].reshape(3, H)
    bd = p[OFF_BD:NPARAM]
    return We, be, Ws, bs, Wd, bd


def forward(p, Am, fixed_nb, r, dinv, bf16_layers=True):
    r = r.reshape(-1, 3)
    dinv = dinv.reshape(-1, 3)
    We, be, Ws, bs, Wd, bd = unpack(p, bf16_layers)
    z = r * dinv
    s = np.sqrt(np.mean(z ** 2))
    ld = -np.log(dinv)
    x = np.concatenate([z / s, ld - ld.mean(), fixed_nb[:, None].astype(float), np.ones((z.shape[0], 1))], axis=1)
    u0 = x @ We.T + be
    h = np.maximum(u0, 0)
    cache = {"x": x, "u": [u0], "h": [h], "a": [], "s": s, "z": z}
    for l in range(NL):
        a = np.concatenate([h, Am @ h], axis=1)
        u = a @ Ws[l].T + bs[l]
        h = h + np.maximum(u, 0)
        cache["a"].append(a)
        cache["u"].append(u)
        cache["h"].append(h)
    y = h @ Wd.T + bd
    return z + s * y, cache


def loss_grad(p, Am, fixed_nb, r, dinv, e, Kmul, bf16_layers=True, mode="energy"):
    """Loss and gradient; Kmul(v) = K v (flat).
    energy:   ||M(r) - e||_K^2 / (e.r);   residual: ||K M(r) - r||^2 / (r.r)."""
    out, c = forward(p, Am, fixed_nb, r, dinv, bf16_layers)
    if mode == "energy":
        e = e.reshape(-1, 3)
        d = out - e
        q = Kmul(d.ravel()).reshape(-1, 3)
        cc = float(e.ravel() @ r.ravel())
        L = float(d.ravel() @ q.ravel()) / cc
        Go = 2.0 * q / cc
    else:
        d = Kmul(out.ravel()) - r.ravel()
        cc = float(r.ravel() @ r.ravel())
        L = float(d @ d) / cc
        Go = (2.0 * Kmul(d) / cc).reshape(-1, 3)
    We, be, Ws, bs, Wd, bd = unpack(p, bf16_layers)
    g = np.zeros(NPARAM)
    gy = c["s"] * Go
    h3 = c["h"][-1]
    g[OFF_WD:OFF_BD] = (gy.T @ h3).ravel()
    g[OFF_BD:NPARAM] = gy.sum(axis=0)
    gh = gy @ Wd
    for l in reversed(range(NL)):
        gu = gh * (c["u"][l + 1] > 0)
        o = OFF_L + l * L_STRIDE
        g[o:o + H * AIN] = (gu.T @ c["a"][l]).ravel()
        g[o + H * AIN:o + L_STRIDE] = gu.sum(axis=0)
        ga = gu @ Ws[l]
        gh = gh + ga[:, :H] + Am.T @ ga[:, H:]
    gu0 = gh * (c["u"][0] > 0)
    g[OFF_WE:OFF_BE] = (gu0.T @ c["x"]).ravel()
    g[OFF_BE:OFF_L] = gu0.sum(axis=0)
    return L, g
