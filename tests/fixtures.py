"""Loaders for the committed golden fixtures in ``tests/golden/``."""

import json
import os

import numpy as np
import scipy.sparse as sp

import sovereign_solver_gb300 as sps

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _unpack(z, prefix):
    mats = {}
    for nm in ("A_ub", "A_eq"):
        shape = tuple(int(v) for v in z[f"{prefix}/{nm}/shape"])
        mats[nm] = sp.csr_matrix((z[f"{prefix}/{nm}/data"], z[f"{prefix}/{nm}/indices"],
                                  z[f"{prefix}/{nm}/indptr"]), shape=shape)
    c = z[f"{prefix}/c"]
    return sps.Problem(c=c, A_ub=mats["A_ub"], b_ub=z[f"{prefix}/b_ub"], A_eq=mats["A_eq"],
                       b_eq=z[f"{prefix}/b_eq"], lb=z[f"{prefix}/lb"], ub=z[f"{prefix}/ub"],
                       integer_mask=np.zeros(c.size, dtype=bool),
                       sense=str(z[f"{prefix}/sense"]), name=prefix)


def load_problems():
    """name -> Problem for every fixture problem."""
    out = {}
    for fn in ("netlib_problems.npz", "small_problems.npz"):
        z = np.load(os.path.join(GOLDEN, fn))
        for prefix in sorted({k.split("/")[0] for k in z.files}):
            out[prefix] = _unpack(z, prefix)
    return out


def load_golden():
    with open(os.path.join(GOLDEN, "pdhg_golden.json")) as f:
        return json.load(f)


def load_stress():
    """(name -> Problem, name -> golden entry) for the reference's three
    seeded stress LPs (``tests/golden/make_stress_golden.py``)."""
    z = np.load(os.path.join(GOLDEN, "stress_problems.npz"))
    probs = {prefix: _unpack(z, prefix) for prefix in sorted({k.split("/")[0] for k in z.files})}
    with open(os.path.join(GOLDEN, "stress_golden.json")) as f:
        return probs, json.load(f)
