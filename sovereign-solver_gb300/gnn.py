"""Learned warm start for a parametric LP family (new API surface).

``WarmStartGNN`` wraps the network of ``include/sps_gnn.h``: a bipartite
message-passing net over the constraint matrix shared by every instance of a
family (one sparsity pattern; per-instance c and b), trained on PDHG solutions
by the library's own forward / backward / Adam kernels.  ``predict`` gives a
warm start (x0, y0, omega0) for ``PDHGEngine.warm_start`` or
``PDHGBatch.set_warm_starts``; those solves fall back to a cold start
when the prediction is worse than zero (KKT of the start point), and the usual
relative-KKT test judges every answer.

Features (per instance, scaled by fixed family scales; cmin_i = min of c over
the columns of row i):
  variable j:   [c_j, mean over its '<=' rows of (c_j - cmin_i),
                 mean over its '=' rows of (c_j - cmin_i), 1]      (costs / c_scale)
  constraint i: [b_i / b_scale, 1 if '<=' row else 0, cmin_i / c_scale, 1]
The cost gaps tell each variable how far it is from the cheapest column of its
rows, which mean aggregation alone cannot compute.  With ``lp_features``
(default) the network takes only the scaled c and b and the device builds these
features (``k_lp_con_features`` / ``k_lp_var_features``); ``host_features`` is
the same construction in NumPy (the tests compare the two).
Targets: x* / x_scale, y* / y_scale, log omega* (omega in the engine's scaled space).
"""

from __future__ import annotations

import ctypes as C
from typing import Iterable, Sequence

import numpy as np
import scipy.sparse as sp

from . import _native as N

FV, FC = 4, 4


def stacked_rows(problem) -> sp.csr_matrix:
    """K = [A_ub; A_eq] (the engine's row order)."""
    return sp.vstack([problem.A_ub, problem.A_eq]).tocsr()


def rhs(problem) -> np.ndarray:
    return np.concatenate([np.asarray(problem.b_ub, float), np.asarray(problem.b_eq, float)])


class WarmStartGNN:
    """A warm-start predictor for the family of ``template`` (same K pattern)."""

    def __init__(self, template, hidden: int = 64, layers: int = 3, seed: int = 0, lr: float = 1e-3,
                 max_batch: int = 8, device: int = 0, loss_weights=(1.0, 1.0, 0.1), scales: dict | None = None,
                 lp_features: bool = True):
        self.lib = N.load()
        K = stacked_rows(template)
        K.sort_indices()
        self.n, self.m, self.m_ub = K.shape[1], K.shape[0], template.A_ub.shape[0]
        self._ptr = np.ascontiguousarray(K.indptr, dtype=np.int32)
        self._idx = np.ascontiguousarray(K.indices, dtype=np.int32)
        self._val = np.ascontiguousarray(K.data, dtype=np.float32)
        self.nnz = int(self._ptr[-1])
        self.hidden, self.layers, self.max_batch = hidden, layers, max_batch
        if scales is None:
            c = np.abs(np.asarray(template.c, float))
            b = np.abs(rhs(template))
            cs = float(c.mean()) if c.size and c.mean() > 0 else 1.0
            bs = float(b.mean()) if b.size and b.mean() > 0 else 1.0
            scales = {"c": cs, "b": bs, "x": bs, "y": cs}
        self.scales = dict(scales)
        self._kind = np.zeros(self.m, np.float32)
        self._kind[: self.m_ub] = 1.0
        deg = np.diff(self._ptr)
        self._row = np.repeat(np.arange(self.m), deg)
        self._nonempty = deg > 0
        self._starts = self._ptr[:-1][self._nonempty]
        le = self._kind[self._row] > 0
        self._w_le, self._w_eq = le.astype(float), (~le).astype(float)
        self._cnt_le = np.maximum(np.bincount(self._idx, weights=self._w_le, minlength=self.n), 1)
        self._cnt_eq = np.maximum(np.bincount(self._idx, weights=self._w_eq, minlength=self.n), 1)
        self.lp_features = bool(lp_features)
        self._kind8 = np.ascontiguousarray(self._kind.astype(np.int8))
        fin_v, fin_c = (1, 1) if self.lp_features else (FV, FC)
        gr = N.GnnGraph(self.n, self.m, N.i32p(self._ptr), N.i32p(self._idx), N.f32p(self._val), fin_v, fin_c,
                        self._kind8.ctypes.data_as(C.POINTER(C.c_int8)))
        o = N.GnnOptions()
        self.lib.sps_gnn_options_init(C.byref(o))
        o.hidden, o.layers, o.seed, o.lr = hidden, layers, seed, lr
        o.loss_x, o.loss_y, o.loss_omega = loss_weights
        o.max_batch, o.device = max_batch, device
        o.lp_features = 1 if self.lp_features else 0
        h = C.c_void_p()
        rc = self.lib.sps_gnn_create(C.byref(gr), C.byref(o), C.byref(h))
        if rc != 0:
            raise (ValueError if rc == -1 else RuntimeError)(self.lib.sps_gnn_last_error(None).decode())
        self.h = h
        self.num_params = int(self.lib.sps_gnn_num_params(h))

    # ---------------------------------------------------------------- data
    def features_from(self, c, b):
        """The network's inputs for one instance's c and b: scaled (c, b) as columns with
        ``lp_features``, else the expanded features of ``host_features``."""
        if self.lp_features:
            return (np.asarray(c, float) / self.scales["c"]).astype(np.float32)[:, None], \
                   (np.asarray(b, float) / self.scales["b"]).astype(np.float32)[:, None]
        return self.host_features(c, b)

    def host_features(self, c, b):
        """(var features n x 4, constraint features m x 4) from one instance's c and b."""
        c = np.asarray(c, float) / self.scales["c"]
        ce = c[self._idx]
        cmin = np.zeros(self.m)
        if self._starts.size:
            cmin[self._nonempty] = np.minimum.reduceat(ce, self._starts)
        d = ce - cmin[self._row]
        fv = np.empty((self.n, FV), np.float32)
        fv[:, 0] = c
        fv[:, 1] = np.bincount(self._idx, weights=d * self._w_le, minlength=self.n) / self._cnt_le
        fv[:, 2] = np.bincount(self._idx, weights=d * self._w_eq, minlength=self.n) / self._cnt_eq
        fv[:, 3] = 1.0
        fc = np.empty((self.m, FC), np.float32)
        fc[:, 0] = np.asarray(b, float) / self.scales["b"]
        fc[:, 1] = self._kind
        fc[:, 2] = cmin
        fc[:, 3] = 1.0
        return fv, fc

    def features(self, problem):
        return self.features_from(problem.c, rhs(problem))

    def targets(self, x, y, omega):
        return (np.asarray(x, float) / self.scales["x"]).astype(np.float32), \
               (np.asarray(y, float) / self.scales["y"]).astype(np.float32), np.float32(np.log(omega))

    # ---------------------------------------------------------------- network calls
    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"{N.ERRORS.get(rc, rc)}: {self.lib.sps_gnn_last_error(self.h).decode()}")

    @staticmethod
    def _stack(items, dtype=np.float32):
        return np.ascontiguousarray(np.stack(items), dtype=dtype)

    def predict_features(self, fvs: Sequence, fcs: Sequence):
        """Raw network outputs for a list of feature pairs: (x0 [k, n], y0 [k, m], log_omega [k])."""
        k = len(fvs)
        X, Y, Lw = np.empty((k, self.n), np.float32), np.empty((k, self.m), np.float32), np.empty(k, np.float32)
        for s in range(0, k, self.max_batch):
            e = min(k, s + self.max_batch)
            fv, fc = self._stack(fvs[s:e]), self._stack(fcs[s:e])
            self._check(self.lib.sps_gnn_predict(self.h, e - s, N.f32p(fv), N.f32p(fc), N.f32p(X[s:e]),
                                                 N.f32p(Y[s:e]), N.f32p(Lw[s:e])))
        return X, Y, Lw

    def predict(self, problems: Iterable):
        """Warm starts (x0, y0, omega0) in the problems' own units, one per problem."""
        problems = list(problems)
        feats = [self.features(p) for p in problems]
        X, Y, Lw = self.predict_features([f[0] for f in feats], [f[1] for f in feats])
        out = []
        for p, x, y, lw in zip(problems, X, Y, Lw):
            x0 = np.clip(x.astype(float) * self.scales["x"], np.asarray(p.lb, float), np.asarray(p.ub, float))
            y0 = y.astype(float) * self.scales["y"]
            y0[: self.m_ub] = np.minimum(y0[: self.m_ub], 0.0)
            out.append((x0, y0, float(np.exp(np.clip(lw, -30.0, 30.0)))))
        return out

    def loss_grad(self, fvs, fcs, xts, yts, lts):
        fv, fc = self._stack(fvs), self._stack(fcs)
        xt, yt, lt = self._stack(xts), self._stack(yts), np.ascontiguousarray(lts, dtype=np.float32)
        loss = C.c_double()
        g = np.empty(self.num_params, np.float32)
        self._check(self.lib.sps_gnn_loss_grad(self.h, len(fvs), N.f32p(fv), N.f32p(fc), N.f32p(xt), N.f32p(yt),
                                               N.f32p(lt), C.byref(loss), N.f32p(g)))
        return loss.value, g

    def train_step(self, fvs, fcs, xts, yts, lts) -> float:
        fv, fc = self._stack(fvs), self._stack(fcs)
        xt, yt, lt = self._stack(xts), self._stack(yts), np.ascontiguousarray(lts, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.sps_gnn_train_step(self.h, len(fvs), N.f32p(fv), N.f32p(fc), N.f32p(xt), N.f32p(yt),
                                                N.f32p(lt), C.byref(loss)))
        return loss.value

    def params(self) -> np.ndarray:
        p = np.empty(self.num_params, np.float32)
        self._check(self.lib.sps_gnn_get_params(self.h, N.f32p(p)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        self._check(self.lib.sps_gnn_set_params(self.h, N.f32p(p)))

    # ---------------------------------------------------------------- persistence
    def save(self, path: str) -> None:
        np.savez(path, params=self.params(), hidden=self.hidden, layers=self.layers, n=self.n, m=self.m,
                 nnz=self.nnz, scales=np.array([self.scales[k] for k in ("c", "b", "x", "y")]),
                 lp_features=int(self.lp_features))

    @classmethod
    def load(cls, path: str, template, **kw) -> "WarmStartGNN":
        d = np.load(path)
        sc = d["scales"]
        net = cls(template, hidden=int(d["hidden"]), layers=int(d["layers"]),
                  scales={"c": float(sc[0]), "b": float(sc[1]), "x": float(sc[2]), "y": float(sc[3])}, **kw)
        if (net.n, net.m, net.nnz) != (int(d["n"]), int(d["m"]), int(d["nnz"])):
            raise ValueError("saved network was trained on a different constraint pattern")
        net.set_params(d["params"])
        return net

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sps_gnn_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
