"""The oracle against the reference's own outputs (golden fixtures).

The fixtures in tests/golden were written by running the unmodified
reference on the same seeded inputs (tests/golden/make_golden.py). Here the
inputs are regenerated, checked against the stored fingerprints, and the
oracle's results are compared with the reference's: the restatement must
agree to rounding (1e-10 e on charges, same iteration counts).
"""

import os
import warnings

import numpy as np
import pytest

from cases import CASES, build_inputs
from oracle import hp_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as f:
        return {k: f[k] for k in f.files}


def check_fingerprint(mol, g):
    assert mol.grid.weights.sum() == pytest.approx(float(g["fp_weights"]), rel=1e-12)
    assert np.dot(mol.grid.weights, mol.density) == pytest.approx(float(g["fp_density"]), rel=1e-12)
    assert np.abs(mol.grid.points).sum() == pytest.approx(float(g["fp_points"]), rel=1e-12)


def basis_tables(mol):
    from horton_part_gb300.basis import ExpBasisFuncHelper

    bs = ExpBasisFuncHelper.from_function_type("gauss")
    return ([bs.get_order(z) for z in mol.numbers], [bs.get_exponent(z) for z in mol.numbers],
            [bs.get_initial(z) for z in mol.numbers])


def run_oracle(case, mol, kwargs):
    args = (mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points, mol.grid.weights,
            mol.density)
    scheme = case["scheme"]
    if scheme == "mbis":
        return O.mbis(*args, **kwargs)
    if scheme in ("nlis", "gmbis"):
        kw = dict(kwargs)
        expn = kw.pop("exp_n_dict")
        nsd = kw.pop("nshell_dict", None) or {}
        init = [O.nlis_initial_propars(int(z), expn, nsd) if scheme == "nlis"
                else O.gmbis_initial_propars(int(z), expn) for z in mol.numbers]
        ranges = np.concatenate([[0], np.cumsum([len(x) for x in init])])
        return O.nlis(*args, np.concatenate(init), ranges, **kw)
    orders, exps, inits = basis_tables(mol)
    if scheme in ("gisa", "lisa"):
        kw = dict(kwargs)
        solver = kw.pop("solver")
        return O.basis_scheme(scheme, *args, orders, exps, inits, solver=solver, **kw)
    kw = dict(kwargs)
    kw.setdefault("maxiter", 100 if kw.get("solver") != "sc" else 500)
    return O.glisa(*args, orders, exps, inits, **kw)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(name):
    case = CASES[name]
    g = load_golden(name)
    mol, kwargs = build_inputs(case)
    check_fingerprint(mol, g)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        res = run_oracle(case, mol, kwargs)
    tol = case.get("tol", {})
    assert int(res["niter"]) == int(g["niter"])
    np.testing.assert_allclose(res["charges"], g["charges"], rtol=0, atol=tol.get("charges", 1e-10))
    np.testing.assert_allclose(res["propars"], g["propars"], rtol=tol.get("propars", 1e-9),
                               atol=1e-12)
    np.testing.assert_allclose(res["history_changes"], g["history_changes"], rtol=1e-6,
                               atol=tol.get("changes", 1e-14))
    np.testing.assert_allclose(res["history_entropies"], g["history_entropies"],
                               rtol=tol.get("entropies", 1e-9),
                               atol=1e-12)
    if "core_charges" in g:
        np.testing.assert_allclose(res["core_charges"], g["core_charges"], atol=1e-10)
        np.testing.assert_allclose(res["valence_widths"], g["valence_widths"], rtol=1e-10)
