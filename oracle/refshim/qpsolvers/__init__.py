"""Stand-in for ``qpsolvers`` (test infrastructure only).

``solve_qp`` routes the reference's GISA quadratic program to the oracle's own
exact active-set solver, so the rest of the reference's GISA loop can run.
"""
import numpy as np


def solve_qp(P, q, G=None, h=None, A=None, b=None, solver=None, initvals=None, **kwargs):
    from oracle.hp_oracle import qp_simplex_nonneg

    q = np.asarray(q, dtype=float).ravel()
    total = float(np.asarray(b, dtype=float).ravel()[0])
    return qp_simplex_nonneg(np.asarray(P, dtype=float), q, total)
