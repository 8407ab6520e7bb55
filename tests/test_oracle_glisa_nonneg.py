"""The oracle's non-negative gLISA optimum (the reference's cvxopt problem) and
its fixtures, checked on the CPU.

cvxopt is absent, so the optimum is certified, not copied: its KKT residuals
must vanish, and they are computed from a restatement of the reference's
``_working_matrix`` (``glisa.py:411-479``) that is itself pinned here to the
reference's own unconstrained Newton result (the golden
``glisa_newton_h2o_50x110``, written by running the reference), where the
same residuals vanish for every population.
"""

import os
import sys

import numpy as np
import pytest

from cases import CASES, build_inputs
from oracle import hp_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)
from make_glisa_nonneg import NONNEG_CASES, build_nonneg_inputs, fingerprint  # noqa: E402


def _golden(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as f:
        return {k: f[k] for k in f.files}


def _basis(mol, helper):
    rs = O.radial_distances(mol.grid.points, mol.coordinates)
    return np.concatenate([O.basis_functions(helper.get_order(z), helper.get_exponent(z), rs[a])
                           for a, z in enumerate(mol.numbers)])


def test_working_matrix_restatement_is_pinned_by_the_reference_newton_optimum():
    """At the reference's converged unconstrained Newton populations (threshold
    1e-8) the gradient of the restated objective is -1 for every shell."""
    from horton_part_gb300.basis import ExpBasisFuncHelper

    mol, _ = build_inputs(CASES["glisa_newton_h2o_50x110"])
    g = _golden("glisa_newton_h2o_50x110")
    G = _basis(mol, ExpBasisFuncHelper.from_function_type("gauss"))
    f, grad, hess = O.glisa_objective(G, mol.grid.weights, mol.density, g["propars"])
    assert np.abs(1.0 + grad).max() < 1e-7
    assert f == pytest.approx(float(g["history_entropies"][-1]), abs=1e-8)
    np.testing.assert_allclose(hess, hess.T, rtol=0, atol=1e-12 * np.abs(hess).max())


@pytest.mark.parametrize("name", sorted(NONNEG_CASES))
def test_fixture_is_a_certified_optimum(name):
    g = _golden(name)
    assert float(g["kkt_stationarity"]) < 1e-12
    assert float(g["kkt_dual_infeasibility"]) < 1e-12
    assert float(g["population_error"]) < 1e-10
    assert float(g["sc_step"]) < 1e-12  # a fixed point of the reference's sc update
    assert (g["propars"] >= 0).all() and (g["propars"] == 0).any()
    assert int(g["nshell"]) == len(g["propars"])


def test_oracle_reproduces_the_fixture():
    """Regenerated inputs match the fingerprints, and the projected Newton of
    the oracle returns the stored optimum (the 222-shell case)."""
    name = "glisa_nonneg_chain30_40x50"
    g = _golden(name)
    mol, helper = build_nonneg_inputs(NONNEG_CASES[name])
    np.testing.assert_allclose(fingerprint(mol), g["fingerprint"], rtol=1e-12)
    args = (mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points, mol.grid.weights,
            mol.density, [helper.get_order(z) for z in mol.numbers],
            [helper.get_exponent(z) for z in mol.numbers],
            [helper.get_initial(z) for z in mol.numbers])
    res = O.glisa_nonneg(*args)
    np.testing.assert_allclose(res["charges"], g["charges"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(res["propars"], g["propars"], rtol=0, atol=1e-10)


def test_kkt_detects_a_planted_error():
    """A perturbed optimum (a mistake planted in the oracle's output) fails
    the certificate."""
    name = "glisa_nonneg_chain38_40x50"
    g = _golden(name)
    mol, helper = build_nonneg_inputs(NONNEG_CASES[name])
    G = _basis(mol, helper)
    c = g["propars"].copy()
    ok = O.glisa_kkt(G, mol.grid.weights, mol.density, c)
    assert ok["stationarity"] < 1e-12 and ok["dual_infeasibility"] < 1e-12
    k = int(np.argmax(c))
    c[k] *= 1.0 + 1e-6
    bad = O.glisa_kkt(G, mol.grid.weights, mol.density, c)
    assert bad["stationarity"] > 1e-9
