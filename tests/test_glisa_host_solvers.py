"""The host side of the gLISA solvers that iterate on the host (DIIS, CDIIS,
quasi-Newton, trust-region), checked on the CPU against the unmodified
reference's own runs (fixtures written by tests/golden/make_glisa_host.py).

The solver logic of :mod:`horton_part_gb300.glisa_solvers` is driven here by
an FP64 NumPy evaluator built from the oracle's restatement of
``_working_matrix`` (pinned to the reference through the golden Newton
cases); on the GPU the same logic drives the device evaluation service
(tests/test_gpu_glisa_host_solvers.py). Bar: the reference's iteration count
and its charges to 1e-8 e. Trust-region is the exception: SciPy's
trust-constr stops on a step tolerance (xtol) well before the optimum, so
its end point depends on rounding-level differences of the function values
(the reference's own trust-region charges lie 1.1e-5 e from the optimum the
other solvers reach); its bar is 2e-5 e from the reference's trust-region
run and from the optimum.
"""

import os
import sys

import numpy as np
import pytest

from horton_part_gb300 import glisa_solvers as hs
from horton_part_gb300.basis import ExpBasisFuncHelper
from oracle import hp_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)
from make_glisa_host import HOST_CASES, build_host_inputs, fixture_name  # noqa: E402


class NumpyEvaluator:
    """The evaluation service in FP64 NumPy on the oracle's functions."""

    def __init__(self, mol, helper, tau=1.0, linspace_size=40):
        self.w, self.rho = mol.grid.weights, mol.density
        rs = O.radial_distances(mol.grid.points, mol.coordinates)
        self.G = np.concatenate([O.basis_functions(helper.get_order(z), helper.get_exponent(z), rs[a])
                                 for a, z in enumerate(mol.numbers)])
        self.ranges = np.concatenate([[0], np.cumsum([helper.get_nshell(z) for z in mol.numbers])])
        self.tau, self.L = tau, linspace_size

    def evaluate(self, x, nderiv=1):
        out = O.glisa_objective(self.G, self.w, self.rho, x, nderiv=max(nderiv, 1))
        f, grad = out[0], out[1]
        hess = out[2] if nderiv == 2 else None
        return f, grad, hess, float(self.w @ (x @ self.G))

    def change(self, x, y, kind=0):
        d = x - y
        if kind == 0:
            v = d @ self.G
            return float(np.sqrt(self.w @ (v * v)))
        msd = 0.0
        for a in range(len(self.ranges) - 1):
            sl = slice(self.ranges[a], self.ranges[a + 1])
            v = d[sl] @ self.G[sl]
            msd += self.w @ (v * v)
        return float(np.sqrt(msd))

    def line_search(self, x, delta, keep):
        for t in np.linspace(self.tau, 0.0, self.L, endpoint=False):
            new = x + keep * (t * delta)
            if all((new[self.ranges[a]:self.ranges[a + 1]] @ self.G[self.ranges[a]:self.ranges[a + 1]]
                    >= O.NEGATIVE_CUTOFF).all() for a in range(len(self.ranges) - 1)):
                return float(t), new
        return -1.0, x.copy()

    def charges(self, mol, x):
        pros = [x[self.ranges[a]:self.ranges[a + 1]] @ self.G[self.ranges[a]:self.ranges[a + 1]]
                for a in range(len(self.ranges) - 1)]
        _, atw = O.stockholder_weights(pros)
        return np.array([mol.pseudo_numbers[a] - self.w @ (atw[a] * self.rho)
                         for a in range(mol.natom)])


@pytest.fixture(scope="module")
def setup():
    mol = build_host_inputs()
    helper = ExpBasisFuncHelper.from_function_type("gauss")
    ev = NumpyEvaluator(mol, helper)
    x0 = O.init_basis_propars([helper.get_initial(z) for z in mol.numbers], mol.pseudo_numbers,
                              mol.grid.weights, mol.density)
    exps = [helper.get_exponent(z) for z in mol.numbers]
    return mol, ev, x0, exps


@pytest.mark.parametrize("solver", HOST_CASES)
def test_host_solver_logic_matches_the_reference(setup, solver):
    mol, ev, x0, exps = setup
    with np.load(os.path.join(GOLDEN, fixture_name(solver) + ".npz")) as f:
        g = {k: f[k] for k in f.files}
    assert mol.grid.weights.sum() == pytest.approx(float(g["fp_weights"]), rel=1e-12)
    thr = 1e-8
    if solver == "diis":
        x, niter, _ = hs.solve_diis(ev, x0, thr)
    elif solver == "cdiis":
        conv, niter, _, x, _ = hs.solve_cdiis(ev, x0, thr, maxiter=500)
        assert conv
    elif solver == "quasi-newton":
        x, niter, _, ents, _ = hs.solve_quasi_newton(ev, x0, thr, exps, ev.ranges)
        np.testing.assert_allclose(ents, g["history_entropies"], rtol=1e-9, atol=1e-12)
    else:
        x, niter = hs.solve_trust_region(ev, x0, thr, 500, float(mol.grid.weights @ mol.density))
    q = ev.charges(mol, x)
    dq = float(np.abs(q - g["charges"]).max())
    print(f"{solver}: niter {niter} (reference {int(g['niter'])}), max|dq| {dq:.2e} e")
    if solver == "trust-region":
        with np.load(os.path.join(GOLDEN, fixture_name("diis") + ".npz")) as f:
            optimum = f["charges"]
        assert dq < 2e-5 and float(np.abs(q - optimum).max()) < 2e-5
        return
    assert dq < 1e-8
    if int(g["niter"]) >= 0:
        assert niter == int(g["niter"])


class _FakeJob(NumpyEvaluator):
    """A device job stand-in for ``GlobalLinearISAWPart._run_job``: the NumPy
    evaluation service plus the ``finish`` call that ends a host-driven job."""

    def finish(self, x, niter):
        self.finished = (np.array(x), int(niter))


@pytest.mark.parametrize("solver", HOST_CASES)
def test_class_runs_the_host_solver_and_returns_histories(solver):
    """The class's host-solver driver on the NumPy service: the solver's end
    point reaches ``finish`` and the histories have the reference's shapes
    (trust-region keeps none)."""
    from horton_part_gb300.utils import wpart_schemes

    mol = build_host_inputs()
    part = wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver=solver, threshold=1e-8)
    job = _FakeJob(mol, ExpBasisFuncHelper.from_function_type("gauss"))
    hist = part._run_job(job)
    x, niter = job.finished
    nshell = job.G.shape[0]
    assert x.shape == (nshell,) and niter > 0
    assert hist["history_propars"].ndim == 2 and hist["history_propars"].shape[1] == nshell
    assert len(hist["history_entropies"]) == len(hist["history_propars"])
    if solver == "trust-region":
        assert hist["history_propars"].shape[0] == 0
    else:
        assert hist["history_propars"].shape[0] > 0
        np.testing.assert_allclose(hist["history_propars"][-1].sum(), x.sum(), rtol=1e-6)
