"""CPU oracle: an FP64 NumPy restatement of horton-part's iterative
stockholder loop on the molecular grid (MBIS, GISA, aLISA, gLISA).

TEST INFRASTRUCTURE ONLY. This module is the checker for the GPU path and the
timed CPU baseline of ``bench.py``; the product never imports it. It follows
the reference algorithm step by step (file:line citations are to the
reference package ``src/horton_part``), on plain arrays instead of the
reference's class hierarchy:

* inputs: ``points (N,3)``, ``weights (N,)``, ``rho (N,)``, ``coordinates
  (A,3)``, ``numbers (A,)``, ``pseudo_numbers (A,)``;
* results: a dict with the keys the reference stores in ``part.cache``.

Parity of this restatement is pinned against the reference itself: the
fixtures in ``tests/golden`` were produced by running the unmodified
reference (through ``oracle/refshim``) on the same inputs, and
``tests/test_oracle_golden.py`` checks the restatement against them. Two reference solvers need packages that are absent here
(quadprog for GISA, cvxopt for the aLISA/gLISA class defaults); GISA's QP is
restated as an exact active-set solver (:func:`qp_simplex_nonneg`), so GISA
parity at that boundary is unpinned.

Vectorised NumPy (BLAS for the gLISA Hessian) replaces a few of the
reference's Python loops; the arithmetic is the same, and the CPU baseline
timed from this module is therefore at least as fast as the reference.
"""

from __future__ import annotations

import math
import warnings

import numpy as np

DENSITY_CUTOFF = 1e-15  # data/constants.yaml:27
NEGATIVE_CUTOFF = -1e-12  # data/constants.yaml:28
POPULATION_CUTOFF = 1e-4  # data/constants.yaml:29


class OracleError(RuntimeError):
    """Raised where the reference raises ``RuntimeError``."""


# ---------------------------------------------------------------------------
# shared pieces
# ---------------------------------------------------------------------------


def radial_distances(points, coordinates):
    """|p - R_a| for every atom (``core/base.py:630-635``)."""
    return [np.linalg.norm(points - c, axis=1) for c in coordinates]


def integrate(weights, *arrays):
    prod = arrays[0]
    for a in arrays[1:]:
        prod = prod * a
    return float(np.dot(weights, prod))


def entropy(weights, rho, rho0, density_cutoff=DENSITY_CUTOFF):
    """Integral of rho ln(rho/rho0) with the sick mask (``core/stockholder.py:145-151``)."""
    sick = (rho0 < density_cutoff) | (rho < density_cutoff)
    with np.errstate(all="ignore"):
        ratio = np.divide(rho, rho0, out=np.zeros_like(rho), where=~sick)
        ln_ratio = np.log(ratio, out=np.zeros_like(rho), where=~sick)
    return integrate(weights, rho, ln_ratio)


def stockholder_weights(proatoms):
    """Promolecule and clipped at_weights (``core/stockholder.py:153-175, 352-384``).

    The promolecule accumulates each pro-atom and then 1e-100, atom by atom.
    """
    promol = np.zeros_like(proatoms[0])
    for work in proatoms:
        promol += work
        promol += 1e-100
    at_weights = [np.clip(work / promol, 0.0, 1.0) for work in proatoms]
    return promol, at_weights


def finalize(res, numbers, pseudo_numbers):
    """``finalize_propars`` (``core/iterstock.py:48-58``)."""
    charges = res["charges"]
    res["history_propars"] = np.array(res["history_propars"])
    res["history_charges"] = np.array(res["history_charges"])
    res["history_entropies"] = np.array(res["history_entropies"])
    res["history_changes"] = np.array(res["history_changes"])
    res["populations"] = numbers - charges
    res["pseudo_populations"] = pseudo_numbers - charges
    return res


# ---------------------------------------------------------------------------
# MBIS  (mbis.py)
# ---------------------------------------------------------------------------


def mbis_nshell(number):
    """Number of Slater shells (``mbis.py:36-46``)."""
    noble = np.array([2, 10, 18, 36, 54, 86, 118])
    return int(noble.searchsorted(number) + 1)


def mbis_initial_propars(number):
    """Initial (N_k, S_k) pairs (``mbis.py:49-78``)."""
    nshell = mbis_nshell(number)
    propars = np.zeros(2 * nshell)
    s0 = 2.0 * number
    alpha = (2.0 / s0) ** (1.0 / (nshell - 1)) if nshell > 1 else 1.0
    nel = np.array([2.0, 8.0, 8.0, 18.0, 18.0, 32.0, 32.0])
    for k in range(nshell):
        propars[2 * k] = nel[k]
        propars[2 * k + 1] = s0 * alpha**k
    propars[-2] = number - propars[:-2:2].sum()
    return propars


def mbis_proatom(propars_a, r):
    """sum_k N_k S_k^3 exp(-S_k r) / (8 pi) (``mbis.py:234-289``)."""
    y = np.zeros(len(r))
    for k in range(len(propars_a) // 2):
        n, s = propars_a[2 * k], propars_a[2 * k + 1]
        y += n * s**3 * np.exp(-s * r) / (8 * np.pi)
    return y


def opt_mbis_propars(rho, propars, weights, r, threshold, density_cutoff=DENSITY_CUTOFF,
                     maxiter=2000):
    """Inner MBIS fixed point for one atom (``mbis.py:81-163``).

    Returns ``(propars, n_inner, converged)``.
    """
    nshell = len(propars) // 2
    terms = np.zeros((nshell, len(r)))
    oldpro = None
    for irep in range(maxiter):
        for k in range(nshell):
            n, s = propars[2 * k], propars[2 * k + 1]
            terms[k] = n * s**3 * np.exp(-s * r) / (8 * np.pi)
        pro = terms.sum(axis=0)
        sick = (rho < density_cutoff) | (pro < density_cutoff)
        with np.errstate(all="ignore"):
            ratio = rho / pro
        ratio[sick] = 0.0
        terms *= ratio
        for k in range(nshell):
            m0 = np.einsum("p,p->", weights, terms[k])
            m1 = np.einsum("p,p,p->", weights, terms[k], r)
            propars[2 * k] = m0
            propars[2 * k + 1] = 3 * m0 / m1
        if oldpro is None:
            change = 1e100
        else:
            err = oldpro - pro
            change = np.sqrt(np.einsum("p,p,p->", weights, err, err))
        if change < threshold:
            return propars, irep + 1, True
        oldpro = pro
    return propars, maxiter, False


def spherical_average(values, shell, wsph, nrad):
    """Angular average of ``values`` over each radial shell of one atom grid:
    sum_j wsph_j f_j per shell, wsph = Lebedev weight / 4 pi (the node values
    of the spline that qc-grid's ``AtomGrid.spherical_average`` returns;
    ``mbis.py:179-184`` evaluates it at the radial nodes)."""
    return np.bincount(shell, weights=wsph * values, minlength=nrad)


def mbis(coordinates, numbers, pseudo_numbers, points, weights, rho, threshold=1e-6,
         maxiter=500, inner_threshold=1e-8, density_cutoff=DENSITY_CUTOFF, local=None):
    """MBIS on the molecular grid (``core/iterstock.py:159-193``, ``mbis.py:167-203``,
    ``mbis.py:291-362``).

    ``local`` selects the atom-grid form (grid_type 1): a dict with
    ``indices`` (atom a owns points indices[a]:indices[a+1]), per-atom radial
    nodes ``rpoints`` and weights ``rweights`` (lists), and per point its
    shell index within its atom grid (``shell``) and its angular weight / 4 pi
    (``wsph``). The at_weights then act on each atom's own points, the inner
    solve runs on the spherical average over the atom's radial grid
    (``mbis.py:174-187``) and the change is a radial integral
    (``core/iterstock.py:43-44``)."""
    natom = len(numbers)
    inner = inner_threshold if inner_threshold < threshold else threshold  # iterstock.py:101
    rs = radial_distances(points, coordinates)
    ranges = [0]
    for z in numbers:
        ranges.append(ranges[-1] + 2 * mbis_nshell(z))
    propars = np.concatenate([mbis_initial_propars(z) for z in numbers])
    res = dict(history_propars=[], history_charges=[], history_entropies=[], history_changes=[],
               inner_iterations=[])
    charges = np.zeros(natom)
    counter = 0
    while True:
        counter += 1
        old = propars.copy()
        pros = [mbis_proatom(propars[ranges[a]:ranges[a + 1]], rs[a]) for a in range(natom)]
        promol, at_weights = stockholder_weights(pros)
        inner_its = []
        for a in range(natom):
            sl = slice(ranges[a], ranges[a + 1])
            if local is None:
                rhoa, wa, ra = at_weights[a] * rho, weights, rs[a]
            else:
                own = slice(local["indices"][a], local["indices"][a + 1])
                ra = local["rpoints"][a]
                rhoa = spherical_average(at_weights[a][own] * rho[own], local["shell"][own],
                                         local["wsph"][own], len(ra))
                wa = 4 * np.pi * ra**2 * local["rweights"][a]
            new, nit, _ = opt_mbis_propars(rhoa, propars[sl].copy(), wa, ra, inner,
                                           density_cutoff)
            propars[sl] = new
            inner_its.append(nit)
            charges[a] = pseudo_numbers[a] - np.einsum("p,p->", wa, rhoa)
        res["inner_iterations"].append(inner_its)
        res["history_propars"].append(propars.copy())
        res["history_charges"].append(charges.copy())
        res["history_entropies"].append(entropy(weights, rho, promol, density_cutoff))
        msd = 0.0
        for a in range(natom):
            if local is None:
                ra, wa = rs[a], weights
            else:
                ra = local["rpoints"][a]
                wa = 4 * np.pi * ra**2 * local["rweights"][a]
            d = (mbis_proatom(propars[ranges[a]:ranges[a + 1]], ra)
                 - mbis_proatom(old[ranges[a]:ranges[a + 1]], ra))
            msd += integrate(wa, d, d)
        change = np.sqrt(msd)
        res["history_changes"].append(change)
        if change < threshold or counter >= maxiter:
            break
    res.update(charges=charges, propars=propars, niter=counter, change=change,
               promoldens=promol, at_weights=np.array(at_weights), ranges=np.array(ranges))
    finalize(res, np.asarray(numbers), np.asarray(pseudo_numbers, dtype=float))
    valence = np.array([-propars[ranges[a + 1] - 2] for a in range(natom)])
    widths = np.array([1.0 / propars[ranges[a + 1] - 1] for a in range(natom)])
    res["valence_charges"] = valence
    res["valence_widths"] = widths
    res["core_charges"] = charges - valence
    return res


# ---------------------------------------------------------------------------
# NLIS / GMBIS  (nlis.py, gmbis.py): MBIS with shells exp(-S r^n)
# ---------------------------------------------------------------------------


def nlis_nshell(number, nshell_dict):
    """Shells of an element (``nlis.py:23-35``)."""
    return nshell_dict.get(number, mbis_nshell(number))


def nlis_initial_propars(number, exp_n_dict, nshell_dict):
    """Initial (N, S, n) triples (``nlis.py:38-96``)."""
    nbs = nlis_nshell(number, nshell_dict)
    propars = np.ones(3 * nbs)
    s0 = 2.0 * number
    alpha = (0.5 / s0) ** (1.0 / (nbs - 1)) if nbs > 1 else 1.0
    for k in range(nbs):
        propars[3 * k] = number / nbs
        propars[3 * k + 1] = s0 * alpha**k
        propars[3 * k + 2] = exp_n_dict[(number, k)] if (number, k) in exp_n_dict else 1.0
    return propars


def gmbis_initial_propars(number, exp_n_dict):
    """Initial (N, S, n) triples of GMBIS (``gmbis.py:17-52``)."""
    nshell = mbis_nshell(number)
    propars = np.zeros(3 * nshell)
    s0 = 2.0 * number
    alpha = (2.0 / s0) ** (1.0 / (nshell - 1)) if nshell > 1 else 1.0
    nel = np.array([2.0, 8.0, 8.0, 18.0, 18.0, 32.0, 32.0])
    for k in range(nshell):
        propars[3 * k] = nel[k]
        propars[3 * k + 1] = s0 * alpha**k
        propars[3 * k + 2] = exp_n_dict[(number, k)] if (number, k) in exp_n_dict else 1.0
    propars[-3] = number - propars[:-3:3].sum()
    return propars


def nlis_unit_shell(s, n, r):
    """n S^(3/n) exp(-S r^n) / (4 pi Gamma(3/n)) (``nlis.py:148``)."""
    return n * s ** (3.0 / n) * np.exp(-s * r**n) / (4 * np.pi * math.gamma(3.0 / n))


def nlis_proatom(propars_a, r):
    """sum_k N_k g_k(r) (``nlis.py:281-296``)."""
    y = np.zeros(len(r))
    for k in range(len(propars_a) // 3):
        nk, s, n = propars_a[3 * k:3 * k + 3]
        y += nk * nlis_unit_shell(s, n, r)
    return y


def opt_nlis_propars(rho, propars, weights, r, threshold, density_cutoff=DENSITY_CUTOFF,
                     maxiter=2000):
    """Inner NLIS fixed point for one atom (``nlis.py:99-195``): N_k <- m0_k,
    S_k <- 3 / (n_k m1_k) with m1_k = int w g_k (rho / pro) r^n (the unit shell,
    without N_k), S_k = 1e-5 where m1_k is within 1e-8 of zero.

    Returns ``(propars, n_inner, converged)``.
    """
    nshell = len(propars) // 3
    terms = np.zeros((nshell, len(r)))
    oldpro = None
    for irep in range(maxiter):
        for k in range(nshell):
            terms[k] = nlis_unit_shell(propars[3 * k + 1], propars[3 * k + 2], r)
        pro = np.sum(terms * propars[::3, None], axis=0)
        sick = (rho < density_cutoff) | (pro < density_cutoff)
        with np.errstate(all="ignore"):
            ratio = rho / pro
        ratio[sick] = 0.0
        terms_ratio = terms * ratio
        for k in range(nshell):
            nk, n = propars[3 * k], propars[3 * k + 2]
            m0 = np.einsum("p,p->", weights, terms_ratio[k] * nk)
            m1 = np.einsum("p,p,p->", weights, terms_ratio[k], r**n)
            propars[3 * k] = m0
            propars[3 * k + 1] = 1e-5 if np.isclose(m1, 0.0) else 3 / (m1 * n)
        if oldpro is None:
            change = 1e100
        else:
            err = oldpro - pro
            change = np.sqrt(np.einsum("p,p,p->", weights, err, err))
        if change < threshold:
            return propars, irep + 1, True
        oldpro = pro
    return propars, maxiter, False


def nlis(coordinates, numbers, pseudo_numbers, points, weights, rho, initial, ranges,
         threshold=1e-6, maxiter=500, inner_threshold=1e-8, density_cutoff=DENSITY_CUTOFF,
         local=None):
    """NLIS / GMBIS (``nlis.py:198-367``, ``gmbis.py:55-156``): the outer loop of
    ``mbis`` (``core/iterstock.py:159-193``, ``mbis.py:167-203``) with the
    pro-atoms of ``nlis_proatom`` and the inner solver ``opt_nlis_propars``.
    ``initial`` holds the atoms' initial (N, S, n) triples
    (``nlis_initial_propars`` or ``gmbis_initial_propars``) and ``ranges`` their
    offsets; ``local`` as in ``mbis``."""
    natom = len(numbers)
    inner = inner_threshold if inner_threshold < threshold else threshold
    rs = radial_distances(points, coordinates)
    propars = np.asarray(initial, dtype=float).copy()
    res = dict(history_propars=[], history_charges=[], history_entropies=[], history_changes=[],
               inner_iterations=[])
    charges = np.zeros(natom)
    counter = 0
    while True:
        counter += 1
        old = propars.copy()
        pros = [nlis_proatom(propars[ranges[a]:ranges[a + 1]], rs[a]) for a in range(natom)]
        promol, at_weights = stockholder_weights(pros)
        its = []
        for a in range(natom):
            sl = slice(ranges[a], ranges[a + 1])
            if local is None:
                rhoa, wa, ra = at_weights[a] * rho, weights, rs[a]
            else:
                ra, wa, _ = _radial_view(local, a)
                rhoa = _local_average(local, a, at_weights[a] * rho)
            new, nit, _ = opt_nlis_propars(rhoa, propars[sl].copy(), wa, ra, inner, density_cutoff)
            propars[sl] = new
            its.append(nit)
            charges[a] = pseudo_numbers[a] - np.einsum("p,p->", wa, rhoa)
        res["inner_iterations"].append(its)
        res["history_propars"].append(propars.copy())
        res["history_charges"].append(charges.copy())
        res["history_entropies"].append(entropy(weights, rho, promol, density_cutoff))
        msd = 0.0
        for a in range(natom):
            ra, wa = (rs[a], weights) if local is None else _radial_view(local, a)[:2]
            d = (nlis_proatom(propars[ranges[a]:ranges[a + 1]], ra)
                 - nlis_proatom(old[ranges[a]:ranges[a + 1]], ra))
            msd += integrate(wa, d, d)
        change = np.sqrt(msd)
        res["history_changes"].append(change)
        if change < threshold or counter >= maxiter:
            break
    res.update(charges=charges, propars=propars, niter=counter, change=change,
               promoldens=promol, at_weights=np.array(at_weights), ranges=np.array(ranges))
    finalize(res, np.asarray(numbers), np.asarray(pseudo_numbers, dtype=float))
    res["valence_charges"] = np.array([-propars[ranges[a + 1] - 3] for a in range(natom)])
    res["valence_widths"] = np.array([1.0 / propars[ranges[a + 1] - 2] for a in range(natom)])
    res["core_charges"] = charges - res["valence_charges"]
    return res


# ---------------------------------------------------------------------------
# basis-function schemes: shared  (gisa.py)
# ---------------------------------------------------------------------------


def shell_prefactor(n, alpha):
    """N(alpha, n) (``core/basis.py:161``)."""
    return n * alpha ** (3.0 / n) / (4.0 * math.pi * math.gamma(3.0 / n))


def basis_functions(orders, exponents, r):
    """(K, N) array of unit-population shells (``gisa.py:91-106``)."""
    return np.array([shell_prefactor(n, a) * np.exp(-a * r**n) for n, a in zip(orders, exponents)])


def init_basis_propars(initials, pseudo_numbers, weights, rho):
    """Initial coefficients (``gisa.py:68-88``): initials below 1e-4 raised
    to 1e-4, each atom normalised to its pseudo number, then all rescaled to
    the integrated density."""
    parts = []
    for inits, zp in zip(initials, pseudo_numbers):
        inits = np.array(inits, dtype=float)
        inits[inits < 1e-4] = 1e-4
        parts.append(inits / np.sum(inits) * zp)
    propars = np.concatenate(parts)
    nelec = integrate(weights, rho)
    return propars / np.sum(propars) * nelec


def compute_quantities(density, propars, bs_funcs, density_cutoff):
    """pro-shells, pro-atom, sick mask, ratio, ln ratio (``utils.py:198-252``)."""
    pro_shells = bs_funcs * np.asarray(propars).ravel()[:, None]
    pro = np.einsum("ij->j", pro_shells)
    sick = (density < density_cutoff) | (pro < density_cutoff)
    with np.errstate(all="ignore"):
        ratio = np.divide(density, pro, out=np.zeros_like(density), where=~sick)
        ln_ratio = np.log(ratio, out=np.zeros_like(density), where=~sick)
    return pro_shells, pro, sick, ratio, ln_ratio


def _population_warning(propars, pop, population_cutoff):
    if abs(np.sum(propars) - pop) > population_cutoff:  # utils.py:418-456
        warnings.warn("The sum of pro-atom parameters is not equal to reference population.")


def _negativity_error(dens, negative_cutoff):
    if (dens < negative_cutoff).any():  # utils.py:491-520
        raise OracleError("Negative pro-atom density found!")


# ---------------------------------------------------------------------------
# GISA  (gisa.py:348-421) - quadratic program
# ---------------------------------------------------------------------------


def qp_simplex_nonneg(P, q, total, maxiter=200):
    """min 1/2 x^T P x + q^T x  subject to  x >= 0, sum(x) = total.

    Exact primal active-set method (Nocedal & Wright, Algorithm 16.3) started
    from the feasible point x = total/K. Restates the problem the reference
    hands to quadprog (``gisa.py:387-421``); quadprog itself is not available.
    """
    K = len(q)
    x = np.full(K, total / K)
    work = np.zeros(K, dtype=bool)  # True: x_i fixed at 0
    at_min = False  # x minimises the objective on the current free set
    for _ in range(maxiter):
        free = ~work
        nf = int(free.sum())
        g = P @ x + q
        if at_min:
            # multiplier check at the subspace minimiser (lambda = -mean g_F)
            lam = -g[free].mean() if nf else 0.0
            mu = g + lam
            if not work.any() or mu[work].min() >= -1e-12 * max(1.0, np.abs(g).max()):
                return x
            work[np.where(work)[0][np.argmin(mu[work])]] = False
            at_min = False
            continue
        kkt = np.zeros((nf + 1, nf + 1))
        kkt[:nf, :nf] = P[np.ix_(free, free)]
        kkt[:nf, nf] = 1.0
        kkt[nf, :nf] = 1.0
        rhs = np.concatenate([-g[free], [0.0]])
        sol = np.linalg.solve(kkt, rhs)
        p = np.zeros(K)
        p[free] = sol[:nf]
        if np.max(np.abs(p)) <= 1e-14 * max(1.0, np.max(np.abs(x))):
            at_min = True
            continue
        alpha, block = 1.0, -1
        for i in np.where(free & (p < 0))[0]:
            a = -x[i] / p[i]
            if a < alpha:
                alpha, block = a, i
        x = x + alpha * p
        if block >= 0:
            x[block] = 0.0
            work[block] = True
        else:
            at_min = True
    raise OracleError("QP active-set solver did not converge")


def gisa_qp(bs_funcs, rho, weights, alphas):
    """One atom's GISA update (``gisa.py:348-421``)."""
    a = np.asarray(alphas, dtype=float)
    P = 2 / np.pi**1.5 * (a[:, None] * a[None, :]) ** 1.5 / (a[:, None] + a[None, :]) ** 1.5
    P = (P + P.T) / 2
    q = -2 * np.einsum("i,ni,i->n", weights, bs_funcs, rho)
    pop = np.einsum("i,i", weights, rho)
    x = qp_simplex_nonneg(P, q, pop)
    _population_warning(x, pop, POPULATION_CUTOFF)
    return x


# ---------------------------------------------------------------------------
# aLISA inner solvers  (alisa.py)
# ---------------------------------------------------------------------------


def lisa_solver_sc(bs_funcs, rho, propars, weights, threshold, density_cutoff=DENSITY_CUTOFF,
                   max_niter_inner=100000):
    """Self-consistent update c_k <- int w c_k g_k rho/pro (``alisa.py:193-291``)."""
    oldpro = None
    for irep in range(int(max_niter_inner)):
        pro_shells, pro, sick, ratio, _ = compute_quantities(rho, propars, bs_funcs,
                                                            density_cutoff)
        propars[:] = np.einsum("p,ip->i", weights, pro_shells * ratio)
        if oldpro is None:
            change = 1e100
        else:
            err = oldpro - pro
            change = np.sqrt(np.einsum("i,i,i", weights, err, err))
        if change < threshold:
            _population_warning(propars, np.einsum("i,i", weights, rho), POPULATION_CUTOFF)
            return propars, irep + 1
        oldpro = pro
    warnings.warn("Warning: Inner iteration is not converge!")
    return propars, int(max_niter_inner)


def lisa_solver_newton(bs_funcs, rho, propars, weights, threshold, mode="exact",
                       density_cutoff=DENSITY_CUTOFF, negative_cutoff=NEGATIVE_CUTOFF,
                       tau=1.0, linspace_size=20, niter=10000):
    """Newton / modified Newton / BFGS quasi-Newton (``mode="bfgs"``) on one
    atom (``alisa.py:753-938``, BFGS update of ``algo/quasi_newton.py:24-49``)."""
    from scipy.linalg import solve

    oldpro = None
    change = 1e100
    pop = np.einsum("i,i", weights, rho)
    H = olddf = step = None
    for irep in range(niter):
        _, pro, sick, ratio, _ = compute_quantities(rho, propars, bs_funcs, density_cutoff)
        if oldpro is not None:
            err = oldpro - pro
            change = np.sqrt(np.einsum("i,i,i", weights, err, err))
        if change < threshold:
            _negativity_error(pro, negative_cutoff)
            _population_warning(propars, pop, POPULATION_CUTOFF)
            return propars, irep + 1
        integrand = bs_funcs * ratio
        with np.errstate(all="ignore"):
            grad_integrand = integrand / pro
        grad_integrand[:, sick] = 0.0
        df = -np.einsum("kp,p->k", integrand, weights)
        if mode == "bfgs":
            if irep == 0:
                H = np.identity(len(propars))
            else:
                y = df - olddf
                sy = step @ y
                H = (H + (sy + y @ H @ y) * np.outer(step, step) / sy ** 2
                     - (H @ np.outer(y, step) + np.outer(step, y) @ H) / sy)
            delta = H @ (-1 - df)
        else:
            hess = np.einsum("kp,jp,p->kj", grad_integrand, bs_funcs, weights)
            delta = solve(hess, -1 - df, assume_a="sym")
        if mode == "exact":
            propars[:] = propars + delta
        else:
            for x in np.linspace(tau, 0, linspace_size):
                new = propars + x * delta
                new_pro = np.einsum("ij->j", bs_funcs * new[:, None])
                if (new_pro > negative_cutoff).all():
                    step = x * delta
                    propars[:] = new
                    break
            else:
                raise OracleError("Line search failed!")
        oldpro = pro
        olddf = df
    raise OracleError("Inner loop: Newton does not converge!")


# ---------------------------------------------------------------------------
# GISA / aLISA outer loop  (core/iterstock.py:159-193, gisa.py:251-279)
# ---------------------------------------------------------------------------


def _radial_view(local, a, bs_orders=None, bs_exponents=None):
    """Atom a's radial nodes, the weights 4 pi r^2 w_r and (optionally) its
    unit-population shells at the nodes (``gisa.py:91-106`` with
    ``rgrid.points``; ``gisa.py:281-318``)."""
    ra = np.asarray(local["rpoints"][a], dtype=float)
    wa = 4 * np.pi * ra**2 * np.asarray(local["rweights"][a], dtype=float)
    g = None if bs_orders is None else basis_functions(bs_orders, bs_exponents, ra)
    return ra, wa, g


def _local_average(local, a, values):
    """Spherical average of ``values`` (molecular-grid array) over atom a's
    own points (``gisa.py:283-289``, ``mbis.py:174-187``)."""
    own = slice(local["indices"][a], local["indices"][a + 1])
    return spherical_average(values[own], local["shell"][own], local["wsph"][own],
                             len(local["rpoints"][a]))


def basis_scheme(scheme, coordinates, numbers, pseudo_numbers, points, weights, rho, orders,
                 exponents, initials, threshold=1e-6, maxiter=500, inner_threshold=1e-8,
                 solver="sc", density_cutoff=DENSITY_CUTOFF, negative_cutoff=NEGATIVE_CUTOFF,
                 local=None):
    """GISA (``scheme='gisa'``) or aLISA (``scheme='lisa'``) on the molecular grid,
    or with ``local`` (the atom-grid description of ``mbis``) on atom grids
    (grid_type 1): each atom's update works on the spherical average of its
    AIM density over its radial grid with the shells evaluated at the radial
    nodes and the weights 4 pi r^2 w_r, the charges are radial integrals, and
    the change is the radial integral of the squared pro-atom difference
    (``gisa.py:281-318``, ``core/iterstock.py:32-45``).

    ``orders/exponents/initials`` are per-atom lists of arrays.
    """
    natom = len(numbers)
    inner = inner_threshold if inner_threshold < threshold else threshold
    rs = radial_distances(points, coordinates)
    bs = [basis_functions(orders[a], exponents[a], rs[a]) for a in range(natom)]
    rad = [_radial_view(local, a, orders[a], exponents[a]) for a in range(natom)] if local else None
    ranges = np.concatenate([[0], np.cumsum([len(e) for e in exponents])])
    propars = init_basis_propars(initials, pseudo_numbers, weights, rho)
    res = dict(history_propars=[], history_charges=[], history_entropies=[], history_changes=[],
               inner_iterations=[])
    charges = np.zeros(natom)
    counter = 0
    while True:
        counter += 1
        old = propars.copy()
        pros = [propars[ranges[a]:ranges[a + 1]] @ bs[a] for a in range(natom)]
        promol, at_weights = stockholder_weights(pros)
        its = []
        for a in range(natom):
            sl = slice(ranges[a], ranges[a + 1])
            if local is None:
                rhoa, wa, ga = at_weights[a] * rho, weights, bs[a]
            else:
                _, wa, ga = rad[a]
                rhoa = _local_average(local, a, at_weights[a] * rho)
            if scheme == "gisa":
                propars[sl] = gisa_qp(ga, rhoa, wa, exponents[a])
                its.append(1)
            elif solver == "sc":
                new, nit = lisa_solver_sc(ga, rhoa, propars[sl].copy(), wa, inner,
                                          density_cutoff)
                propars[sl] = new
                its.append(nit)
            elif solver == "sc-1-iter":  # alisa.py:294-353: one update, no test
                pro_shells, _, _, ratio, _ = compute_quantities(rhoa, propars[sl], ga,
                                                                density_cutoff)
                propars[sl] = np.einsum("p,ip->i", wa, pro_shells * ratio)
                its.append(1)
            elif solver in ("newton", "m-newton", "quasi-newton"):
                new, nit = lisa_solver_newton(
                    ga, rhoa, propars[sl].copy(), wa, inner,
                    mode={"newton": "exact", "m-newton": "modified"}.get(solver, "bfgs"),
                    density_cutoff=density_cutoff, negative_cutoff=negative_cutoff)
                propars[sl] = new
                its.append(nit)
            else:
                raise NotImplementedError(solver)
            charges[a] = pseudo_numbers[a] - integrate(wa, rhoa)
        res["inner_iterations"].append(its)
        res["history_propars"].append(propars.copy())
        res["history_charges"].append(charges.copy())
        res["history_entropies"].append(entropy(weights, rho, promol, density_cutoff))
        msd = 0.0
        for a in range(natom):
            ga, wa = (bs[a], weights) if local is None else (rad[a][2], rad[a][1])
            d = (propars[ranges[a]:ranges[a + 1]] - old[ranges[a]:ranges[a + 1]]) @ ga
            msd += integrate(wa, d, d)
        change = np.sqrt(msd)
        res["history_changes"].append(change)
        if change < threshold or counter >= maxiter:
            break
    res.update(charges=charges, propars=propars, niter=counter, change=change,
               promoldens=promol, at_weights=np.array(at_weights), ranges=ranges)
    return finalize(res, np.asarray(numbers), np.asarray(pseudo_numbers, dtype=float))


# ---------------------------------------------------------------------------
# gLISA  (glisa.py)
# ---------------------------------------------------------------------------


def _fix_propars(exp_array, propars, delta):
    """Indices of the most diffuse shells to freeze (``utils.py:556-577``)."""
    fixed = []
    check = True
    for idx in np.argsort(exp_array):
        if check and np.abs(propars[idx]) < 1e-4 and delta[idx] < 0.0:
            fixed.append(idx)
        else:
            check = False
    return fixed


def glisa(coordinates, numbers, pseudo_numbers, points, weights, rho, orders, exponents,
          initials, threshold=1e-6, maxiter=100, solver="newton",
          density_cutoff=DENSITY_CUTOFF, negative_cutoff=NEGATIVE_CUTOFF, linspace_size=40,
          tau=1.0, local=None):
    """gLISA on the molecular grid (``glisa.py:248-281``) with the ``newton``,
    ``m-newton`` (``glisa.py:617-803``) or ``sc`` (``glisa.py:805-879``) solver.
    With ``local`` (grid_type 1) only the change differs: it is the radial
    integral of the squared pro-atom difference on each atom's radial grid
    (``glisa.py:166-168`` through ``core/iterstock.py:32-45``); the solver
    works on the molecular grid for every grid type (``glisa.py:257-270``)."""
    from scipy.linalg import solve

    natom = len(numbers)
    rs = radial_distances(points, coordinates)
    G = np.concatenate([basis_functions(orders[a], exponents[a], rs[a]) for a in range(natom)])
    ranges = np.concatenate([[0], np.cumsum([len(e) for e in exponents])])
    propars = init_basis_propars(initials, pseudo_numbers, weights, rho)
    pop = integrate(weights, rho)
    res = dict(history_propars=[], history_charges=[], history_entropies=[], history_changes=[])

    rad = ([_radial_view(local, a, orders[a], exponents[a]) for a in range(natom)]
           if local else None)

    def change_of(p1, p2):
        msd = 0.0
        for a in range(natom):
            if local is None:
                ga, wa = G[ranges[a]:ranges[a + 1]], weights
            else:
                ga, wa = rad[a][2], rad[a][1]
            d = (p1[ranges[a]:ranges[a + 1]] - p2[ranges[a]:ranges[a + 1]]) @ ga
            msd += integrate(wa, d, d)
        return np.sqrt(msd)

    def promol_valid(p):
        for a in range(natom):
            if (p[ranges[a]:ranges[a + 1]] @ G[ranges[a]:ranges[a + 1]] < negative_cutoff).any():
                return False
        return True

    niter = None
    if solver in ("newton", "m-newton"):
        for irep in range(maxiter):
            old = propars.copy()
            pro = propars @ G
            sick = (rho < density_cutoff) | (pro < density_cutoff)
            with np.errstate(all="ignore"):
                d1 = np.where(sick, 0.0, rho / pro)  # rho / rho0
            df = -(G @ (weights * d1))
            hess = (G * (weights * np.where(sick, 0.0, d1 / np.where(sick, 1.0, pro)))) @ G.T
            try:
                delta = solve(hess, -1 - df, assume_a="sym")
            except np.linalg.LinAlgError as e:
                raise OracleError(str(e))
            if solver == "newton":
                propars = propars + delta
            else:
                keep = np.ones_like(delta)
                for a in range(natom):
                    sl = slice(ranges[a], ranges[a + 1])
                    for i in _fix_propars(np.asarray(exponents[a]), propars[sl], delta[sl]):
                        keep[i + ranges[a]] = 0
                for x in np.linspace(tau, 0, linspace_size, endpoint=False):
                    new = propars + keep * (x * delta)
                    if promol_valid(new):
                        break
                else:
                    raise OracleError("Line search failed!")
                propars = new
            ent = entropy(weights, rho, pro, density_cutoff)
            change = change_of(propars, old)
            res["history_entropies"].append(ent)
            res["history_propars"].append(propars.copy())
            res["history_changes"].append(change)
            if change < threshold:
                _negativity_error(pro, negative_cutoff)
                _population_warning(propars, pop, POPULATION_CUTOFF)
                niter = irep + 1
                break
        else:
            raise OracleError("Not converged!")
    elif solver == "sc":
        it = 0
        while True:
            old = propars.copy()
            rho0 = old @ G
            sick = (rho < density_cutoff) | (rho0 < density_cutoff)
            with np.errstate(all="ignore"):
                f = np.where(sick, 0.0, rho / rho0)
            propars = old * (G @ (weights * f))
            change = change_of(propars, old)
            res["history_entropies"].append(entropy(weights, rho, rho0, density_cutoff))
            res["history_changes"].append(change)
            res["history_propars"].append(propars.copy())
            if change < threshold:
                break
            it += 1
            if it >= maxiter:
                raise OracleError("Not converged!")
        niter = it + 1
    else:
        raise NotImplementedError(solver)

    pros = [propars[ranges[a]:ranges[a + 1]] @ G[ranges[a]:ranges[a + 1]] for a in range(natom)]
    promol, at_weights = stockholder_weights(pros)
    charges = np.array([pseudo_numbers[a] - integrate(weights, at_weights[a] * rho)
                        for a in range(natom)])
    res.update(charges=charges, propars=propars, niter=niter, promoldens=promol,
               at_weights=np.array(at_weights), ranges=ranges)
    return finalize(res, np.asarray(numbers), np.asarray(pseudo_numbers, dtype=float))


# ---------------------------------------------------------------------------
# gLISA with non-negative populations (the reference's cvxopt default)
# ---------------------------------------------------------------------------


def glisa_objective(G, weights, rho, c, density_cutoff=DENSITY_CUTOFF, nderiv=2):
    """Objective, gradient and Hessian of ``_working_matrix`` (``glisa.py:411-479``)
    for the basis matrix ``G`` (M, N), vectorised: f = int rho ln(rho/rho0),
    grad_i = -int rho g_i / rho0, H_ij = int rho g_i g_j / rho0^2, with the
    sick mask rho < cutoff or rho0 < cutoff."""
    rho0 = c @ G
    sick = (rho < density_cutoff) | (rho0 < density_cutoff)
    with np.errstate(all="ignore"):
        ratio = np.where(sick, 0.0, rho / np.where(sick, 1.0, rho0))
        lnr = np.where(sick, 0.0, np.log(np.where(sick, 1.0, ratio)))
    f = integrate(weights, rho, lnr)
    if nderiv == 0:
        return f
    wr = weights * ratio
    grad = -(G @ wr)
    if nderiv == 1:
        return f, grad
    d2 = wr * np.where(sick, 0.0, 1.0 / np.where(sick, 1.0, rho0))
    hess = (G * d2) @ G.T
    return f, grad, hess


def glisa_kkt(G, weights, rho, c, density_cutoff=DENSITY_CUTOFF, zero=0.0):
    """KKT residuals of the cvxopt problem of ``glisa.py:488-571`` (minimise
    int rho ln(rho/rho0) subject to sum c = int rho and c >= 0) at ``c``.

    Its multiplier of the equality is 1 (sum_i c_i grad_i = -int rho at any
    c), so the optimality conditions read e_i = 1 + grad_i = 0 where
    c_i > ``zero`` and e_i >= 0 where c_i <= ``zero``. Returns the largest
    |e_i| over the positive populations, the most negative e_i over the zero
    ones (0 when none is negative), the smallest population and
    |sum c - int rho|."""
    _, grad = glisa_objective(G, weights, rho, c, density_cutoff, nderiv=1)
    e = 1.0 + grad
    pos = c > zero
    stat = float(np.abs(e[pos]).max()) if pos.any() else 0.0
    dual = float(min(0.0, e[~pos].min())) if (~pos).any() else 0.0
    return {"stationarity": stat, "dual_infeasibility": -dual, "min_population": float(c.min()),
            "population_error": float(abs(c.sum() - integrate(weights, rho)))}


def glisa_nonneg(coordinates, numbers, pseudo_numbers, points, weights, rho, orders, exponents,
                 initials, gtol=1e-12, maxiter=200, density_cutoff=DENSITY_CUTOFF,
                 raise_on_maxiter=True):
    """The optimum of the reference's default gLISA solver (cvxopt,
    ``glisa.py:488-571``; cvxopt is absent here) on the molecular grid.

    The same convex problem is solved by a projected Newton method on the
    extended objective F(c) = int rho ln(rho/rho0) + sum c over c >= 0
    (Bertsekas 1982), whose KKT points are those of the cvxopt problem
    (:func:`glisa_kkt`): free set {c_i > 0 or dF/dc_i < 0}, Newton step on the
    free block (FP64 Cholesky), step lengths 2^-t on the projection
    max(c + 2^-t d, 0) with the Armijo rule. Stops when every KKT residual
    is below ``gtol``. Starts from the reference's initial populations
    (``gisa.py:68-88``). Returns the reference's result keys plus ``kkt``
    and ``G``. With ``raise_on_maxiter=False`` it returns after ``maxiter``
    iterations without reaching the tolerance (a bounded timing sample)."""
    from scipy.linalg import cho_factor, cho_solve

    natom = len(numbers)
    rs = radial_distances(points, coordinates)
    G = np.concatenate([basis_functions(orders[a], exponents[a], rs[a]) for a in range(natom)])
    ranges = np.concatenate([[0], np.cumsum([len(e) for e in exponents])])
    c = init_basis_propars(initials, pseudo_numbers, weights, rho)

    def F(x):
        return glisa_objective(G, weights, rho, x, density_cutoff, nderiv=0) + x.sum()

    niter = 0
    for niter in range(1, maxiter + 1):
        f, grad, hess = glisa_objective(G, weights, rho, c, density_cutoff)
        e = 1.0 + grad
        kkt = max(np.abs(e[c > 0]).max(initial=0.0), max(0.0, -e[c <= 0].min(initial=0.0)))
        if kkt < gtol:
            break
        free = (c > 0) | (e < 0)
        idx = np.flatnonzero(free)
        d = np.zeros_like(c)
        d[idx] = -cho_solve(cho_factor(hess[np.ix_(idx, idx)]), e[idx])
        f0 = f + c.sum()
        for t in range(40):
            x = np.maximum(c + 0.5**t * d, 0.0)
            if F(x) <= f0 + 1e-4 * e @ (x - c):
                break
        else:
            raise OracleError("projected Newton: no descent step")
        c = x
    else:
        if raise_on_maxiter:
            raise OracleError("projected Newton did not reach the KKT tolerance")
    pros = [c[ranges[a]:ranges[a + 1]] @ G[ranges[a]:ranges[a + 1]] for a in range(natom)]
    _, at_weights = stockholder_weights(pros)
    charges = np.array([pseudo_numbers[a] - integrate(weights, at_weights[a] * rho)
                        for a in range(natom)])
    return {"charges": charges, "propars": c, "niter": niter, "ranges": ranges, "G": G,
            "populations": np.asarray(numbers) - charges,
            "kkt": glisa_kkt(G, weights, rho, c, density_cutoff)}
