"""FP64 restatement of the warm-start network — TEST INFRASTRUCTURE ONLY.

The same network, parameter layout, BF16 rounding of the weight matrices and
head vectors, loss and analytic backward pass as the GPU kernels
(include/sps_gnn.h describes them); used to check the GPU gradients.  The
analytic backward is itself checked against central finite differences with
exact (unrounded) weights, where the loss is smooth.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def bf16_round(a) -> np.ndarray:
    """FP32 -> nearest BF16 (ties to even), returned as float64."""
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


class Layout:
    """Offsets of the parameter vector (order of include/sps_gnn.h)."""

    def __init__(self, H: int, L: int, Fv: int, Fc: int):
        self.H, self.L, self.Fv, self.Fc = H, L, Fv, Fc
        self.items = []
        o = 0

        def add(name, shape, mat):
            nonlocal o
            size = int(np.prod(shape))
            self.items.append((name, o, shape, mat))
            o += size

        add("Wv", (H, Fv), True); add("bv", (H,), False)
        add("Wc", (H, Fc), True); add("bc", (H,), False)
        for l in range(L):
            add(f"Uc{l}", (H, H), True); add(f"Mc{l}", (H, H), True); add(f"bc{l}", (H,), False)
            add(f"Uv{l}", (H, H), True); add(f"Mv{l}", (H, H), True); add(f"bv{l}", (H,), False)
        add("wx", (H,), True); add("bx", (1,), False)
        add("wy", (H,), True); add("by", (1,), False)
        add("wo", (2 * H,), True); add("bo", (1,), False)
        self.size = o

    def unpack(self, p, bf16=True) -> dict:
        out = {}
        for name, o, shape, mat in self.items:
            v = np.asarray(p[o:o + int(np.prod(shape))], dtype=np.float64)
            if mat and bf16:
                v = bf16_round(np.asarray(p[o:o + int(np.prod(shape))], dtype=np.float32))
            out[name] = v.reshape(shape)
        return out

    def pack(self, d: dict) -> np.ndarray:
        p = np.zeros(self.size)
        for name, o, shape, _ in self.items:
            p[o:o + int(np.prod(shape))] = np.asarray(d[name]).ravel()
        return p


def graph_mats(ptr, idx, val, n):
    """Ac = A / deg(row) (m x n), Av = A^T / deg(column) (n x m)."""
    m = len(ptr) - 1
    A = sp.csr_matrix((np.asarray(val, float), np.asarray(idx), np.asarray(ptr)), shape=(m, n))
    degc = np.diff(A.indptr).astype(float)
    degv = np.bincount(A.indices, minlength=n).astype(float)
    Ac = sp.diags(1.0 / np.maximum(degc, 1)) @ A
    Av = sp.diags(1.0 / np.maximum(degv, 1)) @ A.T.tocsr()
    return Ac.tocsr(), Av.tocsr()


def relu(z):
    return np.maximum(z, 0.0)


def forward(P: dict, L: int, Ac, Av, fv, fc):
    hv = [relu(fv @ P["Wv"].T + P["bv"])]
    hc = [relu(fc @ P["Wc"].T + P["bc"])]
    ac, av = [], []
    for l in range(L):
        ac.append(Ac @ hv[l])
        hc.append(relu(hc[l] @ P[f"Uc{l}"].T + ac[l] @ P[f"Mc{l}"].T + P[f"bc{l}"]))
        av.append(Av @ hc[l + 1])
        hv.append(relu(hv[l] @ P[f"Uv{l}"].T + av[l] @ P[f"Mv{l}"].T + P[f"bv{l}"]))
    x0 = hv[L] @ P["wx"] + P["bx"][0]
    y0 = hc[L] @ P["wy"] + P["by"][0]
    pool = np.concatenate([hc[L].mean(0), hv[L].mean(0)])
    lw = pool @ P["wo"] + P["bo"][0]
    return {"hv": hv, "hc": hc, "ac": ac, "av": av, "x0": x0, "y0": y0, "pool": pool, "lw": lw}


def loss_grad(p, lay: Layout, ptr, idx, val, fvs, fcs, xts, yts, lts, ax=1.0, ay=1.0, ao=0.1, bf16=True):
    """Mean loss over the instances and its gradient (FP64)."""
    n, m = fvs[0].shape[0], fcs[0].shape[0]
    Ac, Av = graph_mats(ptr, idx, val, n)
    P = lay.unpack(p, bf16)
    G = {k: np.zeros_like(v) for k, v in P.items()}
    B = len(fvs)
    H, L = lay.H, lay.L
    total = 0.0
    for fv, fc, xt, yt, lt in zip(fvs, fcs, xts, yts, lts):
        c = forward(P, L, Ac, Av, np.asarray(fv, float), np.asarray(fc, float))
        dx, dy, dl = c["x0"] - xt, c["y0"] - yt, c["lw"] - lt
        total += ax * np.sum(dx * dx) / n + ay * np.sum(dy * dy) / m + ao * dl * dl
        gx, gy, gl = 2 * ax * dx / (n * B), 2 * ay * dy / (m * B), 2 * ao * dl / B
        hv, hc, ac, av = c["hv"], c["hc"], c["ac"], c["av"]
        G["wx"] += gx @ hv[L]; G["bx"] += gx.sum()
        G["wy"] += gy @ hc[L]; G["by"] += gy.sum()
        G["wo"] += gl * c["pool"]; G["bo"] += gl
        dhv = np.outer(gx, P["wx"]) + gl * P["wo"][H:] / n
        dhc = np.outer(gy, P["wy"]) + gl * P["wo"][:H] / m
        for l in range(L - 1, -1, -1):
            dzv = dhv * (hv[l + 1] > 0)
            G[f"Uv{l}"] += dzv.T @ hv[l]; G[f"Mv{l}"] += dzv.T @ av[l]; G[f"bv{l}"] += dzv.sum(0)
            dhv_prev = dzv @ P[f"Uv{l}"]
            dhc = dhc + Av.T @ (dzv @ P[f"Mv{l}"])
            dzc = dhc * (hc[l + 1] > 0)
            G[f"Uc{l}"] += dzc.T @ hc[l]; G[f"Mc{l}"] += dzc.T @ ac[l]; G[f"bc{l}"] += dzc.sum(0)
            dhc = dzc @ P[f"Uc{l}"]
            dhv = dhv_prev + Ac.T @ (dzc @ P[f"Mc{l}"])
        dzv = dhv * (hv[0] > 0)
        G["Wv"] += dzv.T @ np.asarray(fv, float); G["bv"] += dzv.sum(0)
        dzc = dhc * (hc[0] > 0)
        G["Wc"] += dzc.T @ np.asarray(fc, float); G["bc"] += dzc.sum(0)
    return total / B, lay.pack(G)


def predict(p, lay: Layout, ptr, idx, val, fv, fc, bf16=True):
    n = fv.shape[0]
    Ac, Av = graph_mats(ptr, idx, val, n)
    c = forward(lay.unpack(p, bf16), lay.L, Ac, Av, np.asarray(fv, float), np.asarray(fc, float))
    return c["x0"], c["y0"], c["lw"]
