"""gLISA solvers whose iterations run on the host.

horton-part offers, beside its Newton solvers, four solvers of the global
problem that iterate on a handful of vectors of populations: DIIS and CDIIS
acceleration of the self-consistent map ``function_g`` (``glisa.py:883-928,
969-1028`` with ``algo/diis.py:41-137`` and ``algo/cdiis.py:15-357``), a
BFGS quasi-Newton method (``glisa.py:595-615, 617-803`` with
``algo/quasi_newton.py:24-49``) and SciPy's trust-constr minimiser
(``glisa.py:930-991``). Here the iteration logic (the small least-squares
problems, QR updates and rank-two updates on vectors of nparam values) runs
on the host, and every pass over the grid runs on the device through an
*evaluator*:

``evaluate(x, nderiv)``  -> ``(f, grad, hess, int rho0)`` of ``_working_matrix``
``change(x, y, kind)``   -> promolecule change (kind 0) or outer change (kind 1)
``line_search(x, d, k)`` -> ``(t, x + k t d)`` of the valid-promolecule search, t < 0: none

:class:`horton_part_gb300._lib.Job` is the device evaluator. Each solver
returns ``(populations, niter, history)`` with ``history`` the populations
after each iteration as the reference records them.
"""

from __future__ import annotations

import numpy as np

__all__ = ["function_g", "solve_diis", "solve_cdiis", "solve_quasi_newton", "solve_trust_region",
           "fixed_diffuse_shells", "HOST_SOLVERS"]

HOST_SOLVERS = ("diis", "cdiis", "quasi-newton", "trust-region")


def function_g(ev, x):
    """The self-consistent map c_k <- c_k int rho g_k / rho0 (``glisa.py:850-879``):
    ``-grad_k`` of ``_working_matrix`` is the integral."""
    _, grad, _, _ = ev.evaluate(x, 1)
    return x * -grad


def _pulay_combination(points, residuals):
    """Coefficients c (sum c = 1) minimising |sum c_i r_i| by the bordered
    normal equations (Pulay), solved by a sparse LU as the reference's
    ``lstsq_spsolver`` (``algo/diis.py:140-168``); returns sum c_i x_i, or the
    last point when the system is singular."""
    from scipy.sparse import csc_matrix
    from scipy.sparse.linalg import spsolve

    n = len(points)
    r = np.asarray(residuals)
    gram = r @ r.T
    b = np.zeros((n + 1, n + 1))
    b[:n, :n] = 0.5 * (gram + gram.T)
    b[n, :n] = -1.0
    b[:n, n] = -1.0
    rhs = np.zeros(n + 1)
    rhs[n] = -1.0
    coef = spsolve(csc_matrix(b), rhs)
    out = coef[:n] @ np.asarray(points)
    return points[-1] if np.isnan(out).any() else out


def solve_diis(ev, x0, threshold, maxiter=1000, diis_size=8, version="P", use_dmrs=False):
    """Anderson-Pulay DIIS on the fixed point g(x) = x.

    Version P mixes the iterates and applies g to the mixture; version A
    mixes the images. Convergence: the promolecule change between the new
    point and the previous one (or, with ``use_dmrs``, the residual norm)
    below ``threshold``."""
    x = np.array(x0, dtype=float)
    res_hist, x_hist, g_hist = [], [], []
    for it in range(maxiter):
        g = function_g(ev, x)
        r = g - x
        x_prev = x.copy()
        res_hist.append(r)
        depth = min(it + 1, diis_size)
        if version == "P":
            x_hist.append(x.copy())
            x = function_g(ev, _pulay_combination(x_hist[-depth:], res_hist[-depth:]))
        else:
            g_hist.append(g)
            x = _pulay_combination(g_hist[-depth:], res_hist[-depth:])
            x_hist.append(x)
        conv = np.linalg.norm(r) if use_dmrs else ev.change(x, x_prev, 0)
        if conv < threshold:
            return x, it + 1, x_hist
    raise RuntimeError("Error: not converge!")


def solve_cdiis(ev, x0, threshold, maxiter=1000, mode="R-CDIIS", diis_size=5, param=0.1,
                minrestart=1, modeQR="full", slidehole=False):
    """Commutator DIIS with restarts (R-CDIIS, the default), fixed depth
    (FD-CDIIS), adaptive depth (AD-CDIIS) or plain iteration ("Roothaan"),
    after Chupin, Dupuy, Legendre and Sere (2021): the least-squares problem
    for the mixing coefficients is solved through a QR factorisation of the
    matrix of residual differences, updated column by column.

    Returns ``(converged, niter, residual_norms, x_last, history)``."""
    import scipy.linalg as sla

    def resid(v):
        return function_g(ev, v) - v

    use_diis = mode != "Roothaan"
    x = np.array(x0, dtype=float)
    npar = x.size
    diis_size = min(diis_size, npar)
    r = resid(x)
    hist_all = [x]
    xs, rs = [x], [r]
    norms = []
    mk, nbiter = 0, 1
    grown_full = False
    restart = True
    dr = None
    q = rr = q1 = None
    xlast = x
    while np.linalg.norm(rs[-1]) > threshold and nbiter < maxiter:
        norms.append(np.linalg.norm(r))
        if mk > 0 and use_diis:
            if mode == "R-CDIIS":
                if modeQR == "full":
                    if mk == 1 or restart:
                        restart = False
                        q, rr = sla.qr(dr)
                    else:
                        q, rr = sla.qr_insert(q, rr, dr[:, -1], mk - 1, "col")
                else:
                    q, rr = sla.qr(dr, mode="economic")
            elif mode == "AD-CDIIS":
                q, rr = sla.qr(dr, mode="economic")
            elif mode == "FD-CDIIS":
                if modeQR == "full":
                    if mk == 1:
                        q, rr = sla.qr(dr)
                    elif mk < diis_size:
                        q, rr = sla.qr_insert(q, rr, dr[:, -1], mk - 1, "col")
                    else:
                        if grown_full:
                            q, rr = sla.qr_delete(q, rr, 0, which="col")
                        q, rr = sla.qr_insert(q, rr, dr[:, -1], mk - 1, "col")
                        grown_full = True
                else:
                    q, rr = sla.qr(dr, mode="economic")
            q1 = q[:, :mk]
            base = rs[0] if mode == "R-CDIIS" else rs[-1]
            rhs = -(q.T @ base.reshape(-1, 1))
            gamma = sla.solve_triangular(rr[:mk, :mk], rhs[:mk], lower=False).ravel()
            c = np.zeros(mk + 1)
            if mode == "R-CDIIS":
                c[0] = 1.0 - gamma.sum()
                c[1:] = gamma
            else:
                c[0] = -gamma[0]
                for i in range(1, mk):
                    c[i] = gamma[i - 1] - gamma[i]
                c[mk] = 1.0 - c[:mk].sum()
            x_mix = np.zeros_like(x)
            for i in range(mk + 1):
                x_mix = x_mix + c[i] * xs[i]
        else:
            x_mix = x.copy()
        x = function_g(ev, x_mix)
        xs.append(x)
        r = x_new_r = resid(x)
        if mode in ("AD-CDIIS", "FD-CDIIS"):
            s = x_new_r - rs[-1]
        elif mode == "R-CDIIS":
            s = x_new_r - rs[0]
        elif mode == "Roothaan":
            s = x_new_r.copy()
        else:
            raise RuntimeError(f"Unknown mode: {mode}")
        rs.append(x_new_r)
        col = s.reshape(-1, 1)
        dr = col if (mk == 0 or not use_diis) else np.hstack((dr, col))
        if mode == "R-CDIIS":
            if mk > 0:
                last = dr[:, -1]
                if param * np.linalg.norm(last) > np.linalg.norm(last - q1 @ (q1.T @ last)):
                    mk = minrestart - 1
                    dr = dr[:, -minrestart:]
                    rs = rs[-minrestart:]
                    xs = xs[-minrestart:]
                    restart = True
                else:
                    mk += 1
            else:
                mk += 1
        if mode == "AD-CDIIS":
            mk += 1
            drop = []
            for l in range(mk - 1):
                if np.linalg.norm(rs[-1]) < param * np.linalg.norm(rs[l]):
                    drop.append(l)
                elif not slidehole:
                    break
            if drop:
                mk -= len(drop)
                dr = np.delete(dr, drop, axis=1)
                for l in sorted(drop, reverse=True):
                    rs.pop(l)
                    xs.pop(l)
            if mk == npar + 1:
                dr = dr[:, 1:mk + 1]
                xs.pop(0)
                rs.pop(0)
                mk -= 1
        elif mode == "FD-CDIIS":
            if mk == diis_size:
                dr = dr[:, 1:mk + 1]
                xs.pop(0)
                rs.pop(0)
            if mk < diis_size:
                mk += 1
        nbiter += 1
        xlast = x
        hist_all.append(x.copy())
    converged = not (np.linalg.norm(rs[-1]) > threshold and nbiter == maxiter)
    return converged, nbiter - 1, norms, xlast, hist_all


def fixed_diffuse_shells(exponents, c, delta):
    """Shells whose population stays fixed in a Newton line search
    (``utils.py:556-577``): walking from the most diffuse shell, those with
    |c| < 1e-4 and a negative step, up to the first that is not."""
    fixed = []
    for idx in np.argsort(exponents):
        if abs(c[idx]) < 1e-4 and delta[idx] < 0.0:
            fixed.append(int(idx))
        else:
            break
    return fixed


def _bfgs_inverse(df, s, df_old, h_old):
    """BFGS update of the inverse Hessian from the step s and the gradient
    change y = df - df_old (Nocedal and Wright, eq. 6.17)."""
    y = df - df_old
    sy = s @ y
    hy = h_old @ y
    return (h_old + (sy + y @ hy) * np.outer(s, s) / sy**2
            - (np.outer(hy, s) + np.outer(s, y @ h_old)) / sy)


def solve_quasi_newton(ev, x0, threshold, exponents, ranges, maxiter=1000, niter_exact_newton=0):
    """BFGS on the extended KL objective with the valid-promolecule line
    search of the Newton solvers. ``exponents``/``ranges``: each atom's shell
    exponents and population range (for the fixed diffuse shells).

    Returns ``(x, niter, history, entropies, changes)``; raises
    ``RuntimeError`` when the line search or the iteration fails."""
    x = np.array(x0, dtype=float)
    history, entropies, changes = [], [], []
    h_inv = df_old = s = None
    for it in range(maxiter):
        x_old = x.copy()
        if it == 0 or it <= niter_exact_newton - 1:
            if niter_exact_newton == 0:
                f, df, _, _ = ev.evaluate(x, 1)
                h_inv = np.identity(df.size)
            else:
                f, df, hess, _ = ev.evaluate(x, 2)
                h_inv = np.linalg.inv(hess)
        else:
            f, df, _, _ = ev.evaluate(x, 1)
            h_inv = _bfgs_inverse(df, s, df_old, h_inv)
        delta = h_inv @ (-1.0 - df)
        keep = np.ones_like(delta)
        for a in range(len(ranges) - 1):
            sl = slice(ranges[a], ranges[a + 1])
            for i in fixed_diffuse_shells(np.asarray(exponents[a]), x[sl], delta[sl]):
                keep[ranges[a] + i] = 0.0
        t, x_new = ev.line_search(x, delta, keep)
        if t < 0:
            raise RuntimeError("Line search failed!")
        s = t * delta
        x = x_new
        change = ev.change(x, x_old, 1)
        entropies.append(f)
        history.append(x.copy())
        changes.append(change)
        if change < threshold:
            return x, it + 1, history, entropies, changes
        df_old = df
    raise RuntimeError("Not converged!")


def solve_trust_region(ev, x0, threshold, maxiter, mol_pop, allow_neg_pars=False):
    """SciPy's trust-constr minimiser with SR1 Hessian approximations on
    f(c) + int rho0 - int rho (``glisa.py:930-991``): populations in
    [0, 200], or a population constraint sum c = int rho when negative
    populations are allowed. Returns ``(x, niter)``."""
    from scipy.optimize import SR1, LinearConstraint, minimize

    nb = len(x0)

    def cost_grad(x):
        f, df, _, pro_pop = ev.evaluate(x, 1)
        return f + pro_pop - mol_pop, df + 1.0

    if allow_neg_pars:
        bounds, constraint = None, LinearConstraint(np.ones((1, nb)), mol_pop, mol_pop)
    else:
        bounds, constraint = [(0.0, 200)] * nb, None
    seen = []

    def callback(xk, state):
        seen.append(np.array(xk, dtype=float))
        if len(seen) >= 2:
            change = ev.change(seen[-1], seen[-2], 0)
            return change < threshold and state["status"]
        return None

    res = minimize(cost_grad, np.array(x0, dtype=float), method="trust-constr", jac=True, hess=SR1(),
                   bounds=bounds, constraints=constraint, callback=callback,
                   options={"gtol": threshold, "maxiter": maxiter, "verbose": 0})
    if not res.success:
        raise RuntimeError("Convergence failure.")
    return res.x, int(res.nit)
