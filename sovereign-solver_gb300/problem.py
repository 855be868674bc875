"""LP input type, field-for-field the reference's ``Problem`` dataclass.

Mirrors ``solver/problem.py:19-67`` (fields), ``:71-99`` (derived sizes),
``:103-142`` (``validate``), ``:146-158`` (``empty``) and ``:160-169``
(``eval_obj``) of the reference, so a reference ``Problem`` and this one are
interchangeable at the solver boundary (the solver only reads attributes).

    min/max  cᵀx
    s.t.     A_ub x ≤ b_ub      (m_ub rows, CSR)
             A_eq x = b_eq      (m_eq rows, CSR)
             lb ≤ x ≤ ub        (±inf allowed)

``sense == "max"`` problems store c already negated; the reported objective
is flipped back (``problem.py:50-52``).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np
import scipy.sparse as sp


@dataclass
class Problem:
    c: np.ndarray
    A_ub: sp.csr_matrix
    b_ub: np.ndarray
    A_eq: sp.csr_matrix
    b_eq: np.ndarray
    lb: np.ndarray
    ub: np.ndarray
    integer_mask: np.ndarray
    P_qp: Optional[sp.csr_matrix] = None
    sense: str = "min"
    name: str = ""

    @property
    def n_vars(self) -> int:
        return len(self.c)

    @property
    def n_ineq(self) -> int:
        return self.A_ub.shape[0]

    @property
    def n_eq(self) -> int:
        return self.A_eq.shape[0]

    @property
    def n_constraints(self) -> int:
        return self.n_ineq + self.n_eq

    @property
    def is_milp(self) -> bool:
        return bool(np.any(self.integer_mask))

    @property
    def is_qp(self) -> bool:
        return self.P_qp is not None

    def validate(self) -> None:
        """Raise ``ValueError`` listing every inconsistent dimension."""
        n = self.n_vars
        errs = []
        if self.A_ub.shape != (self.n_ineq, n):
            errs.append(f"A_ub shape {self.A_ub.shape} inconsistent with n_vars={n}")
        if np.shape(self.b_ub) != (self.n_ineq,):
            errs.append(f"b_ub shape {np.shape(self.b_ub)} != ({self.n_ineq},)")
        if self.A_eq.shape != (self.n_eq, n):
            errs.append(f"A_eq shape {self.A_eq.shape} inconsistent with n_vars={n}")
        if np.shape(self.b_eq) != (self.n_eq,):
            errs.append(f"b_eq shape {np.shape(self.b_eq)} != ({self.n_eq},)")
        if np.shape(self.lb) != (n,):
            errs.append(f"lb shape {np.shape(self.lb)} != ({n},)")
        if np.shape(self.ub) != (n,):
            errs.append(f"ub shape {np.shape(self.ub)} != ({n},)")
        if np.shape(self.integer_mask) != (n,):
            errs.append(f"integer_mask shape {np.shape(self.integer_mask)} != ({n},)")
        if self.sense not in ("min", "max"):
            errs.append(f"sense must be 'min' or 'max', got '{self.sense}'")
        if self.P_qp is not None and self.P_qp.shape != (n, n):
            errs.append(f"P_qp shape {self.P_qp.shape} inconsistent with n_vars={n}")
        if not errs and np.any(self.lb > self.ub + 1e-12):
            bad = np.where(self.lb > self.ub + 1e-12)[0]
            errs.append(f"lb > ub for variables: {bad[:5].tolist()} ...")
        if errs:
            raise ValueError("Problem validation failed:\n  " + "\n  ".join(errs))

    @classmethod
    def empty(cls, n: int) -> "Problem":
        """An n-variable problem with no constraints, x ≥ 0."""
        return cls(
            c=np.zeros(n),
            A_ub=sp.csr_matrix((0, n), dtype=float),
            b_ub=np.zeros(0),
            A_eq=sp.csr_matrix((0, n), dtype=float),
            b_eq=np.zeros(0),
            lb=np.zeros(n),
            ub=np.full(n, np.inf),
            integer_mask=np.zeros(n, dtype=bool),
        )

    def eval_obj(self, x: np.ndarray) -> float:
        """Objective at x in the problem's own sense."""
        v = float(self.c @ x)
        if self.P_qp is not None:
            v += 0.5 * float(x @ self.P_qp.dot(x))
        return -v if self.sense == "max" else v

    def __repr__(self) -> str:
        kind = "MILP" if self.is_milp else ("QP" if self.is_qp else "LP")
        return (f"Problem(name={self.name!r}, type={kind}, n_vars={self.n_vars}, "
                f"n_ineq={self.n_ineq}, n_eq={self.n_eq})")
