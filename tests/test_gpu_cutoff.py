"""Per-atom cutoff of the MBIS inner solve and outer change.

The reference evaluates every atom at every grid point. The GPU path skips an
(atom, point tile) pair of the inner solve when the atom's AIM density is
below density_cutoff on the whole tile (the reference's sick mask makes those
moments exact zeros) and the pair's share of the inner change is bounded
below 1e-16 of the squared threshold; the outer change skips a pair on the
same bound. On a molecule whose atoms lie far apart (a row of six waters,
15 bohr between neighbours, 75 bohr long) a share of the work is skipped
(measured: a quarter in FP64, a tenth in the FP32 and float-float forms,
whose inner solves take fewer iterations where the cutoff applies), and the
result must still be the oracle's: the same iteration count and charges
within 1e-10 e (FP64), 1e-6 e (mixed precision).
"""

import numpy as np
import pytest

from horton_part_gb300 import synthetic
from horton_part_gb300.molgrid import becke_molecular_grid
from horton_part_gb300.utils import wpart_schemes
from oracle import hp_oracle as O

pytestmark = pytest.mark.gpu


def water_row(n=6, spacing=15.0, nrad=30, nang=50, seed=21):
    unit = np.array([[0.0, 0.0, 0.0], [0.757, 0.586, 0.0], [-0.757, 0.586, 0.0]]) * synthetic.ANGSTROM
    coords = np.concatenate([unit + [i * spacing, 0.0, 0.0] for i in range(n)])
    numbers = np.tile(np.array([8, 1, 1], dtype=np.int64), n)
    grid = becke_molecular_grid(coords, nrad, nang)
    rho = synthetic.slater_density(grid.points, coords, numbers, seed)
    rho *= 10.0 * n / grid.integrate(rho)
    return synthetic.Molecule(coords, numbers, grid, rho, name=f"{n} H2O row")


@pytest.fixture(scope="module")
def row_and_oracle():
    mol = water_row()
    ref = O.mbis(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points,
                 mol.grid.weights, mol.density, threshold=1e-8, maxiter=500, inner_threshold=1e-8)
    return mol, ref


@pytest.mark.parametrize("precision,q_tol", [("fp64", 1e-10), ("mixed", 1e-6), ("ff", 1e-9)])
def test_cutoff_keeps_the_oracle_result(row_and_oracle, precision, q_tol, gpu_context):
    mol, ref = row_and_oracle
    part = wpart_schemes("mbis")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=3, threshold=1e-8, inner_threshold=1e-8,
                                 precision=precision)
    part.do_partitioning()
    info = part.job_info
    frac = info.point_atom_evals_skipped / info.point_atom_evals
    dq = float(np.abs(part["charges"] - ref["charges"]).max())
    print(f"{precision}: niter {part['niter']} (oracle {ref['niter']}), max|dq| {dq:.2e} e, "
          f"skipped {frac:.1%} of {info.point_atom_evals:.3e} point-atom evaluations")
    assert frac > 0.05
    assert dq < q_tol
    if precision != "mixed":
        assert part["niter"] == ref["niter"]
        np.testing.assert_allclose(part["propars"], ref["propars"], rtol=1e-7)
