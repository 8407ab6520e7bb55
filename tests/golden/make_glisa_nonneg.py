"""Write the fixtures of gLISA with non-negative populations (the reference's
default ``cvxopt`` solver) on the benchmarked molecule and on two larger
shell counts, from the oracle.

    python tests/golden/make_glisa_nonneg.py [case ...]

cvxopt is absent, so the target is the optimum of the same convex problem
(``glisa.py:488-571``), found by :func:`oracle.hp_oracle.glisa_nonneg` and
certified by its KKT residuals (stationarity where a population is positive,
dual feasibility where it is zero; the objective and gradient restate
``_working_matrix``, ``glisa.py:411-479``, pinned to the reference through the
golden Newton cases). One step of the reference's own self-consistent
update (``glisa.py:805-879``) from that optimum is stored beside it: a KKT
point is a fixed point of that update.

Each ``<case>.npz`` holds the charges, populations, iteration count, KKT
residuals, the self-consistent step residual and input fingerprints (sums of
weights, density and points), a few KB per case. The inputs themselves are
regenerated by :mod:`horton_part_gb300.synthetic` on any machine.
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from horton_part_gb300 import synthetic  # noqa: E402
from oracle import hp_oracle as O  # noqa: E402

# (molecule composition, radial, angular, seed), basis shells per element
NONNEG_CASES = {
    # the benchmarked workload: C6H10N2O2, 100 x Lebedev-302 (604,000 points),
    # 6 s-Gaussians per H and 9 per C/N/O, exponents geometric 0.05..300: 150 shells
    "glisa_nonneg_c6h10n2o2_100x302": dict(mol=({6: 6, 1: 10, 7: 2, 8: 2}, 100, 302, 2024),
                                           shells={1: 6, 6: 9, 7: 9, 8: 9}),
    # 30 atoms, 222 shells: above the fused-pass limit (192)
    "glisa_nonneg_chain30_40x50": dict(mol=({6: 10, 1: 16, 7: 2, 8: 2}, 40, 50, 31),
                                       shells={1: 6, 6: 9, 7: 9, 8: 9}),
    # 38 atoms, 282 shells: the tiled tensor-core Hessian (above 256)
    "glisa_nonneg_chain38_40x50": dict(mol=({6: 14, 1: 20, 8: 4}, 40, 50, 38),
                                       shells={1: 6, 6: 9, 8: 9}),
}


def build_nonneg_inputs(case):
    """(molecule, basis helper) of a case."""
    counts, nrad, nang, seed = case["mol"]
    mol = synthetic.chain_molecule(counts, nrad, nang, seed=seed)
    helper = synthetic.geometric_gaussian_basis(case["shells"], 0.05, 300.0)
    return mol, helper


def fingerprint(mol):
    return np.array([mol.grid.weights.sum(), mol.density.sum(), mol.grid.points.sum(),
                     float(mol.npoint)])


def solve(mol, helper):
    args = (mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points, mol.grid.weights,
            mol.density, [helper.get_order(z) for z in mol.numbers],
            [helper.get_exponent(z) for z in mol.numbers],
            [helper.get_initial(z) for z in mol.numbers])
    return O.glisa_nonneg(*args)


def main(names=None):
    for name, case in NONNEG_CASES.items():
        if names and name not in names:
            continue
        t0 = time.time()
        mol, helper = build_nonneg_inputs(case)
        res = solve(mol, helper)
        G, c = res["G"], res["propars"]
        # one self-consistent step of the reference (glisa.py:850-879) from the optimum
        rho0 = c @ G
        sick = (mol.density < O.DENSITY_CUTOFF) | (rho0 < O.DENSITY_CUTOFF)
        f = np.where(sick, 0.0, mol.density / np.where(sick, 1.0, rho0))
        sc_step = float(np.abs(c * (G @ (mol.grid.weights * f)) - c).max())
        kkt = res["kkt"]
        np.savez(os.path.join(HERE, f"{name}.npz"), charges=res["charges"], propars=c,
                 populations=res["populations"], niter=res["niter"],
                 kkt_stationarity=kkt["stationarity"],
                 kkt_dual_infeasibility=kkt["dual_infeasibility"],
                 population_error=kkt["population_error"], sc_step=sc_step,
                 nshell=len(c), fingerprint=fingerprint(mol))
        print(f"{name}: {mol.natom} atoms, {mol.npoint} points, {len(c)} shells, "
              f"{res['niter']} iterations, KKT {kkt['stationarity']:.1e} / "
              f"{kkt['dual_infeasibility']:.1e}, sc step {sc_step:.1e}, zero populations "
              f"{int((c == 0).sum())}, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main(sys.argv[1:])
