"""MPS reader: a fixed- or free-format MPS file to the engine's ``Problem``.

Counterpart of the reference's ``read_mps`` (``solver/io/mps_reader.py:42-331``)
for feeding real instances to the GPU engine.  Sections: NAME, OBJSENSE
(MIN / MAX, on the same or the next line), ROWS (N / L / G / E; the first N row
is the objective, later N rows are ignored), COLUMNS (with 'MARKER' 'INTORG' /
'INTEND' integer markers), RHS (a value on the objective row is a constant and
is ignored), RANGES, BOUNDS (UP, LO, FX, FR, MI, PL, BV, LI, UI), ENDATA.
Tokens are whitespace separated (names without spaces); text after '$' or a
line starting with '*' is a comment.

Rows become the box form the engine takes:
  L:  a x <= b                 G:  -a x <= -b            E:  a x = b
  range R on L:  b - |R| <= a x <= b       on G:  b <= a x <= b + |R|
  on E:  R > 0: b <= a x <= b + R,  R < 0: b + R <= a x <= b
(a two-sided row is two '<=' rows).  Column bounds default to [0, +inf); an
UP bound below zero with no lower bound given sets the lower bound to -inf, as
the MPS convention has it.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import scipy.sparse as sp

from .problem import Problem


def _tokens(line: str):
    if line[:1] == "*":
        return []
    return line.split("$", 1)[0].split()


def read_mps(path) -> Problem:
    """Parse an MPS file (see the module docstring) into a ``Problem``."""
    path = Path(path)
    sense = "min"
    obj_row = None
    row_kind: dict[str, str] = {}
    row_order: list[str] = []
    col_index: dict[str, int] = {}
    col_names: list[str] = []
    integer: list[bool] = []
    entries: dict[str, list[tuple[int, float]]] = {}
    cost: dict[int, float] = {}
    rhs: dict[str, float] = {}
    ranges: dict[str, float] = {}
    lo: dict[int, float] = {}
    up: dict[int, float] = {}
    section = None
    in_int = False
    pending_objsense = False
    with open(path) as f:
        for raw in f:
            if not raw.strip():
                continue
            head = not raw[:1].isspace()
            t = _tokens(raw)
            if not t:
                continue
            if head:
                section = t[0].upper()
                if section == "OBJSENSE" and len(t) > 1:
                    sense = "max" if t[1].upper() in ("MAX", "MAXIMIZE") else "min"
                else:
                    pending_objsense = section == "OBJSENSE"
                if section == "ENDATA":
                    break
                continue
            if section == "OBJSENSE" or pending_objsense:
                sense = "max" if t[0].upper() in ("MAX", "MAXIMIZE") else "min"
                pending_objsense = False
            elif section == "ROWS":
                kind, name = t[0].upper(), t[1]
                if kind == "N":
                    if obj_row is None:
                        obj_row = name
                    continue
                if kind not in ("L", "G", "E"):
                    raise ValueError(f"{path.name}: unknown row type {kind!r}")
                row_kind[name] = kind
                row_order.append(name)
                entries[name] = []
            elif section == "COLUMNS":
                if len(t) >= 3 and t[1].strip("'\"").upper() == "MARKER":
                    marker = t[2].strip("'\"").upper()
                    in_int = marker == "INTORG"
                    continue
                col = t[0]
                if col not in col_index:
                    col_index[col] = len(col_names)
                    col_names.append(col)
                    integer.append(in_int)
                j = col_index[col]
                for r, v in zip(t[1::2], t[2::2]):
                    v = float(v)
                    if r == obj_row:
                        cost[j] = cost.get(j, 0.0) + v
                    elif r in entries:
                        entries[r].append((j, v))
                    elif r not in row_kind:
                        raise ValueError(f"{path.name}: column {col} names unknown row {r!r}")
            elif section in ("RHS", "RANGES"):
                pairs = t[1:] if len(t) % 2 == 1 else t
                target = rhs if section == "RHS" else ranges
                for r, v in zip(pairs[0::2], pairs[1::2]):
                    if r == obj_row:
                        continue
                    if r not in row_kind:
                        raise ValueError(f"{path.name}: {section} names unknown row {r!r}")
                    target[r] = float(v)
            elif section == "BOUNDS":
                kind = t[0].upper()
                if kind in ("FR", "MI", "PL", "BV"):
                    col = t[-1] if len(t) < 3 else t[2]
                    val = None
                else:
                    col, val = t[2], float(t[3])
                if col not in col_index:
                    raise ValueError(f"{path.name}: bound on unknown column {col!r}")
                j = col_index[col]
                if kind == "UP":
                    up[j] = val
                    if val < 0 and j not in lo:
                        lo[j] = -np.inf
                elif kind == "LO":
                    lo[j] = val
                elif kind == "FX":
                    lo[j] = up[j] = val
                elif kind == "FR":
                    lo[j], up[j] = -np.inf, np.inf
                elif kind == "MI":
                    lo[j] = -np.inf
                elif kind == "PL":
                    up[j] = np.inf
                elif kind == "BV":
                    lo[j], up[j] = 0.0, 1.0
                    integer[j] = True
                elif kind in ("LI", "UI"):
                    (lo if kind == "LI" else up)[j] = val
                    integer[j] = True
                else:
                    raise ValueError(f"{path.name}: unsupported bound type {kind!r}")
            # NAME and unknown sections carry nothing the LP needs
    n = len(col_names)
    ub_rows, ub_rhs, eq_rows, eq_rhs = [], [], [], []
    for name in row_order:
        a, b, k = entries[name], rhs.get(name, 0.0), row_kind[name]
        neg = [(j, -v) for j, v in a]
        r = ranges.get(name)
        if k == "L":
            ub_rows.append(a); ub_rhs.append(b)
            if r is not None:
                ub_rows.append(neg); ub_rhs.append(-(b - abs(r)))
        elif k == "G":
            ub_rows.append(neg); ub_rhs.append(-b)
            if r is not None:
                ub_rows.append(a); ub_rhs.append(b + abs(r))
        else:
            if r is None or r == 0.0:
                eq_rows.append(a); eq_rhs.append(b)
            else:
                lo_b, hi_b = (b, b + r) if r > 0 else (b + r, b)
                ub_rows.append(a); ub_rhs.append(hi_b)
                ub_rows.append(neg); ub_rhs.append(-lo_b)

    def csr(rows):
        ptr = np.zeros(len(rows) + 1, dtype=np.int64)
        idx, val = [], []
        for i, row in enumerate(rows):
            acc: dict[int, float] = {}
            for j, v in row:
                acc[j] = acc.get(j, 0.0) + v
            for j in sorted(acc):
                idx.append(j)
                val.append(acc[j])
            ptr[i + 1] = len(idx)
        return sp.csr_matrix((np.asarray(val, float), np.asarray(idx, np.int64), ptr), shape=(len(rows), n))

    c = np.zeros(n)
    for j, v in cost.items():
        c[j] = v
    lb = np.array([lo.get(j, 0.0) for j in range(n)], float)
    ub = np.array([up.get(j, np.inf) for j in range(n)], float)
    if sense == "max":
        c = -c                               # stored minimisation, reported in the file's sense
    p = Problem(c=c, A_ub=csr(ub_rows), b_ub=np.asarray(ub_rhs, float), A_eq=csr(eq_rows),
                b_eq=np.asarray(eq_rhs, float), lb=lb, ub=ub, integer_mask=np.asarray(integer, bool),
                sense=sense, name=path.stem)
    return p
