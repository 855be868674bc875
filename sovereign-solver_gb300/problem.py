"""LP input type, field-for-field the reference's ``Problem`` dataclass.

Mirrors ``solver/problem.py:19-67`` (fields), ``:71-99`` (derived sizes),
``:103-142`` (``validate``: ``ValueError`` on the same conditions, in this
module's own wording), ``:146-158`` (``empty``) and ``:160-169``
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
        """Raise ``ValueError`` naming every field whose shape does not fit the
        others (and any variable whose lower bound exceeds its upper bound)."""
        n, mu, me = self.n_vars, self.n_ineq, self.n_eq
        want = [("A_ub", np.shape(self.A_ub), (mu, n)), ("b_ub", np.shape(self.b_ub), (mu,)),
                ("A_eq", np.shape(self.A_eq), (me, n)), ("b_eq", np.shape(self.b_eq), (me,)),
                ("lb", np.shape(self.lb), (n,)), ("ub", np.shape(self.ub), (n,)),
                ("integer_mask", np.shape(self.integer_mask), (n,))]
        if self.P_qp is not None:
            want.append(("P_qp", np.shape(self.P_qp), (n, n)))
        problems = [f"{field}: shape {got}, expected {exp}" for field, got, exp in want if tuple(got) != exp]
        if self.sense not in ("min", "max"):
            problems.append(f"sense: {self.sense!r} is neither 'min' nor 'max'")
        if not problems:
            crossed = np.flatnonzero(self.lb > self.ub + 1e-12)
            if crossed.size:
                problems.append(f"lb above ub at {crossed.size} variable(s), first {crossed[:5].tolist()}")
        if problems:
            raise ValueError(f"invalid Problem {self.name!r}: " + "; ".join(problems))

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
        kind = "MILP" if self.is_milp else "QP" if self.is_qp else "LP"
        return f"Problem({self.name!r}, {kind}, {self.n_vars} vars, {self.n_ineq} <=, {self.n_eq} =)"
