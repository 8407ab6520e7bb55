"""GPU parity: the public classes (through libhpgpu.so) against the
reference's results on the same inputs.

Golden values come from the unmodified reference (tests/golden). FP64 path
tolerances: charges within 1e-8 e (the accuracy target is 1e-6 e), pro-atom
parameters within 1e-7 relative, identical iteration counts unless the
reference's final change lies within 1e-6 (relative) of the threshold.
"""

import os
import warnings

import numpy as np
import pytest

from cases import CASES, build_inputs, tolerances
from horton_part_gb300 import synthetic
from horton_part_gb300.basis import ExpBasisFuncHelper
from horton_part_gb300.utils import wpart_schemes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
Q_TOL = 1e-8
P_RTOL = 1e-7


def load_golden(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as f:
        return {k: f[k] for k in f.files}


def run_case(name, precision="fp64", store_at_weights=True):
    case = CASES[name]
    mol, kwargs = build_inputs(case)
    grid_type = 1 if kwargs.pop("local", None) is not None else 3  # atom grids: mol.grid.atgrids
    cls = wpart_schemes(case["scheme"])
    part = cls(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid, mol.density,
               grid_type=grid_type, precision=precision, store_at_weights=store_at_weights,
               **kwargs)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        part.do_partitioning()
    return part, mol


def niter_must_match(g, threshold):
    ch = np.asarray(g["history_changes"])
    return abs(ch[-1] - threshold) > 1e-6 * threshold and (len(ch) < 2 or abs(ch[-2] - threshold) > 1e-6 * threshold)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_parity_with_reference(name, gpu_context):
    g = load_golden(name)
    part, mol = run_case(name)
    thr = CASES[name]["kwargs"]["threshold"]
    tol = tolerances(CASES[name])
    q_tol = max(Q_TOL, tol.get("charges", 0.0))
    if niter_must_match(g, thr):
        assert part["niter"] == int(g["niter"])
    np.testing.assert_allclose(part["charges"], g["charges"], rtol=0, atol=q_tol)
    np.testing.assert_allclose(part["propars"], g["propars"], rtol=P_RTOL, atol=1e-10)
    n = min(len(part["history_changes"]), len(g["history_changes"]))
    np.testing.assert_allclose(part["history_entropies"][:n], g["history_entropies"][:n],
                               rtol=max(1e-8, CASES[name].get("tol", {}).get("entropies", 0.0)),
                               atol=1e-10)
    np.testing.assert_allclose(part["history_propars"][:n], g["history_propars"][:n],
                               rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(part["populations"], g["populations"], atol=q_tol)
    if CASES[name]["scheme"] != "glisa":
        np.testing.assert_allclose(part["history_charges"][:n], g["history_charges"][:n],
                                   atol=q_tol)
        assert part["change"] == pytest.approx(float(g["change"]), rel=1e-4,
                                               abs=tol.get("changes", 0.0))
    else:
        assert part["history_charges"].size == 0
    if "core_charges" in g:
        np.testing.assert_allclose(part["core_charges"], g["core_charges"], atol=q_tol)
        np.testing.assert_allclose(part["valence_charges"], g["valence_charges"], atol=q_tol)
        np.testing.assert_allclose(part["valence_widths"], g["valence_widths"], rtol=P_RTOL)


def test_at_weights_and_promolecule(gpu_context):
    """at_weights are the clipped pro-atom / promolecule ratios and sum to one
    where the promolecule is well above 1e-100 (core/stockholder.py:352-377)."""
    part, mol = run_case("mbis_h2o_75x110")
    aw = np.array([part[f"at_weights_{i}"] for i in range(mol.natom)])
    promol = part["promoldens"]
    assert aw.min() >= 0.0 and aw.max() <= 1.0
    big = promol > 1e-30
    np.testing.assert_allclose(aw[:, big].sum(axis=0), 1.0, atol=1e-12)
    # charges from the at_weights on the grid agree with the loop's charges
    # up to one outer iteration's change
    q = mol.pseudo_numbers - np.array([mol.grid.integrate(aw[i], mol.density) for i in range(mol.natom)])
    np.testing.assert_allclose(q, part["charges"], atol=1e-6)


def test_do_charges_and_do_all(gpu_context):
    mol = synthetic.water(nrad=40, nang=50)
    cls = wpart_schemes("mbis")
    part = cls(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid, mol.density,
               grid_type=3, threshold=1e-6)
    part.do_charges()
    names = part.do_all()
    for key in ("charges", "propars", "niter", "change", "history_propars", "populations",
                "pseudo_populations", "core_charges", "valence_charges", "valence_widths"):
        assert key in part.cache and key in names
    assert abs(part["charges"].sum()) < 1e-3
    assert part["charges"] == pytest.approx(part["valence_charges"] + part["core_charges"])


def test_grid_type_1_needs_atom_grids_like_the_reference(gpu_context):
    """grid_type 1 without atom grids raises ValueError (core/base.py:461-465);
    aLISA's Newton solvers do not run on atom grids on this path."""
    from horton_part_gb300.molgrid import MolecularGrid

    mol = synthetic.water(nrad=20, nang=50)
    bare = MolecularGrid(mol.grid.points, mol.grid.weights)
    with pytest.raises(ValueError):
        wpart_schemes("mbis")(mol.coordinates, mol.numbers, mol.pseudo_numbers, bare, mol.density,
                              grid_type=1)
    part = wpart_schemes("lisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=1, solver="m-newton")
    with pytest.raises(NotImplementedError):
        part.do_partitioning()


def test_mbis_atom_grids_match_the_oracle(gpu_context):
    """grid_type 1 on a synthetic water grid (Becke transform radial grid,
    Lebedev-50): the GPU's atom-grid MBIS against the oracle's."""
    from horton_part_gb300.molgrid import atom_grid_arrays

    mol = synthetic.water(nrad=30, nang=50)
    arr = atom_grid_arrays(mol.grid)
    roff, spo = arr["radial_offsets"], arr["shell_point_offsets"]
    shell = np.repeat(np.arange(len(spo) - 1), np.diff(spo))
    local = dict(indices=np.asarray(mol.grid.indices),
                 rpoints=[arr["radial_points"][roff[a]:roff[a + 1]] for a in range(3)],
                 rweights=[arr["radial_weights"][roff[a]:roff[a + 1]] for a in range(3)],
                 shell=shell - np.repeat(roff[:-1], np.diff(roff))[shell],
                 wsph=arr["point_sphere_weights"])
    from oracle import hp_oracle as O

    ref = O.mbis(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points,
                 mol.grid.weights, mol.density, threshold=1e-8, local=local)
    part = wpart_schemes("mbis")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=1, threshold=1e-8)
    part.do_partitioning()
    assert part["niter"] == ref["niter"]
    np.testing.assert_allclose(part["charges"], ref["charges"], atol=1e-9)
    np.testing.assert_allclose(part["propars"], ref["propars"], rtol=1e-7)


def test_numbers_must_be_int64(gpu_context):
    mol = synthetic.water(nrad=20, nang=50)
    with pytest.raises(TypeError):
        wpart_schemes("mbis")(mol.coordinates, mol.numbers.astype(np.int32), mol.pseudo_numbers,
                              mol.grid, mol.density, grid_type=3)


def test_glisa_not_converged_raises(gpu_context):
    mol = synthetic.water(nrad=30, nang=50)
    part = wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver="newton",
                                  solver_options={"maxiter": 2}, threshold=1e-12)
    with pytest.raises(RuntimeError, match="Not converged"):
        part.do_partitioning()


def test_hbm_budget_rejects_oversized_job():
    from horton_part_gb300 import _lib

    ctx = _lib.Context(0, hbm_budget=1 << 16)
    mol = synthetic.water(nrad=40, nang=110)
    part = wpart_schemes("mbis")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=3, context=ctx)
    with pytest.raises(MemoryError):
        part.do_partitioning()
    ctx.close()


def test_custom_basis_helper(gpu_context):
    """A user-supplied ExpBasisFuncHelper object runs and matches the oracle;
    an ill-posed basis (tight 300 bohr^-2 Gaussians on H, whose optimal
    populations are zero) makes the unconstrained Newton system singular on
    the GPU exactly as in the reference (glisa.py:763-769 raises)."""
    from oracle import hp_oracle as O

    mol = synthetic.chain_molecule({6: 1, 8: 1, 1: 3}, 30, 50, seed=11)
    bad = synthetic.geometric_gaussian_basis({1: 4, 6: 6, 8: 6}, 0.05, 300.0)
    part = wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver="newton", basis_func=bad,
                                  threshold=1e-8)
    with pytest.raises(RuntimeError):
        part.do_partitioning()
    gauss = ExpBasisFuncHelper.from_function_type("gauss")
    helper = ExpBasisFuncHelper({z: gauss.get_order(z) for z in (1, 6, 8)},
                                {z: gauss.get_exponent(z) for z in (1, 6, 8)},
                                {z: gauss.get_initial(z) for z in (1, 6, 8)})
    part = wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver="newton", basis_func=helper,
                                  threshold=1e-8)
    part.do_partitioning()
    ref = O.glisa(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points,
                  mol.grid.weights, mol.density, [helper.get_order(z) for z in mol.numbers],
                  [helper.get_exponent(z) for z in mol.numbers],
                  [helper.get_initial(z) for z in mol.numbers], threshold=1e-8, solver="newton")
    np.testing.assert_allclose(part["charges"], ref["charges"], atol=Q_TOL)
    assert part["niter"] == ref["niter"]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("ff", 1e-9), ("mixed", 1e-6)])
def test_mbis_water_hf_sto3g_reference_data(precision, tol, gpu_context):
    """MBIS on the reference's cached water HF/STO-3G density (the input of
    horton-part's tests/test_wpart.py:95-101) against the unmodified
    reference run on the same molecular grid, and within the reference
    test's 2e-3 of its published charges."""
    from horton_part_gb300.molgrid import MolecularGrid

    path = os.path.join(os.path.dirname(__file__), "golden", "water_sto3g_hf_molgrid.npz")
    with np.load(path) as f:
        d = {k: f[k] for k in f.files}
    grid = MolecularGrid(d["points"], d["weights"])
    part = wpart_schemes("mbis")(d["coordinates"], d["numbers"], d["pseudo_numbers"], grid,
                                 d["density"], grid_type=3, threshold=1e-8, precision=precision)
    part.do_partitioning()
    dq = float(np.abs(part["charges"] - d["ref_charges"]).max())
    print(f"water HF/STO-3G {precision}: niter {part['niter']} (reference {int(d['ref_niter'])}), "
          f"max|dq| {dq:.2e}")
    assert dq < tol
    if precision != "mixed":
        assert part["niter"] == int(d["ref_niter"])
    published = np.array([-0.61891067, 0.3095756, 0.30932584])
    assert np.abs(part["charges"] - published).max() < 2e-3


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("ff", 1e-9), ("mixed", 1e-6)])
def test_mbis_atom_grids_water_hf_sto3g(precision, tol, gpu_context):
    """grid_type 1 (atom grids, the reference's default) on the reference's
    cached water HF/STO-3G data: against the unmodified reference run on the
    same atom grids, and within 5e-5 e of the published charges of
    horton-part's tests/test_wpart.py:95-101."""
    from horton_part_gb300.molgrid import AtomGrid, MolecularGrid

    path = os.path.join(os.path.dirname(__file__), "golden", "water_sto3g_hf_molgrid.npz")
    with np.load(path) as f:
        d = {k: f[k] for k in f.files}
    natom = len(d["numbers"])
    npa = len(d["radial_points"]) * 110
    atgrids = [AtomGrid(d["radial_points"], d["radial_weights"], 110) for _ in range(natom)]
    grid = MolecularGrid(d["points"], d["weights"], indices=np.arange(natom + 1) * npa,
                         atgrids=atgrids)
    part = wpart_schemes("mbis")(d["coordinates"], d["numbers"], d["pseudo_numbers"], grid,
                                 d["density"], grid_type=1, threshold=1e-8, precision=precision)
    part.do_partitioning()
    dq = float(np.abs(part["charges"] - d["ref1_charges"]).max())
    print(f"water HF/STO-3G atom grids {precision}: niter {part['niter']} "
          f"(reference {int(d['ref1_niter'])}), max|dq| {dq:.2e}")
    assert dq < tol
    if precision != "mixed":
        assert part["niter"] == int(d["ref1_niter"])
    published = np.array([-0.61891067, 0.3095756, 0.30932584])
    assert np.abs(part["charges"] - published).max() < 5e-5
    assert part["at_weights_0"].shape == (npa,)


@pytest.mark.parametrize("grid_type", [3, 1])
def test_nlis_general_orders_match_the_oracle(grid_type, gpu_context):
    """NLIS with more shells than MBIS (nshell_dict) and non-integer orders
    (r^1.5) on the molecular grid and on atom grids, against the oracle
    (nlis.py:99-195; the reference's own runs pin the oracle in
    tests/test_oracle_golden.py)."""
    from cases import local_description
    from oracle import hp_oracle as O

    mol = synthetic.water(nrad=30, nang=50)
    nsd = {1: 2, 8: 3}
    expn = {(1, 0): 1.0, (1, 1): 1.5, (8, 0): 1.0, (8, 1): 2.0, (8, 2): 1.5}
    init = [O.nlis_initial_propars(int(z), expn, nsd) for z in mol.numbers]
    ranges = np.concatenate([[0], np.cumsum([len(x) for x in init])])
    local = local_description(mol, 50) if grid_type == 1 else None
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = O.nlis(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points,
                     mol.grid.weights, mol.density, np.concatenate(init), ranges, threshold=1e-8,
                     inner_threshold=1e-8, local=local)
    part = wpart_schemes("nlis")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=grid_type, threshold=1e-8,
                                 exp_n_dict=expn, nshell_dict=nsd)
    part.do_partitioning()
    assert part["niter"] == ref["niter"]
    np.testing.assert_allclose(part["charges"], ref["charges"], atol=1e-7 if grid_type == 1 else 1e-9)
    np.testing.assert_allclose(part["propars"], ref["propars"], rtol=1e-7, atol=1e-10)
    np.testing.assert_allclose(part["valence_widths"], ref["valence_widths"], rtol=1e-7)
