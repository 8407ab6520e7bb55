"""Write the fixture of aLISA (sc solver) on a small peptide-like molecule with
the basis of the large-molecule workload, from the oracle.

    python tests/golden/make_lisa_peptide.py

The workload is 200 atoms (H:C:N:O:S = 100:64:18:16:2) on 150 radial x
Lebedev-590 points per atom with 6-10 s-Gaussians per element (exponents
geometric 0.05..500); the oracle cannot run at that size, so the fixture is
the same construction at 11 atoms (H5 C3 N O S) on 20 x Lebedev-50 points per
atom. The oracle's aLISA sc restates the reference's solver_sc
(alisa.py:193-291) and is pinned to the reference's own run through the
golden ``lisa_sc_h2o_50x110``. The fixture holds charges, parameters,
iteration counts and input fingerprints (a few KB).
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from horton_part_gb300 import synthetic  # noqa: E402
from oracle import hp_oracle as O  # noqa: E402

COUNTS = {1: 5, 6: 3, 7: 1, 8: 1, 16: 1}
SHELLS = {1: 6, 6: 9, 7: 9, 8: 9, 16: 10}


def build_peptide_inputs():
    mol = synthetic.peptide_molecule(counts=COUNTS, nrad=20, nang=50, seed=4, device="cpu")
    helper = synthetic.geometric_gaussian_basis(SHELLS, 0.05, 500.0)
    return mol, helper


def fingerprint(mol):
    return np.array([mol.grid.weights.sum(), mol.density.sum(), np.abs(mol.grid.points).sum(),
                     float(mol.npoint)])


def main():
    t0 = time.time()
    mol, h = build_peptide_inputs()
    res = O.basis_scheme("lisa", mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points,
                         mol.grid.weights, mol.density, [h.get_order(z) for z in mol.numbers],
                         [h.get_exponent(z) for z in mol.numbers],
                         [h.get_initial(z) for z in mol.numbers], solver="sc", threshold=1e-6,
                         inner_threshold=1e-8)
    np.savez(os.path.join(HERE, "lisa_sc_peptide11_20x50.npz"), charges=res["charges"],
             propars=res["propars"], niter=res["niter"], fingerprint=fingerprint(mol))
    print(f"{mol.natom} atoms, {mol.npoint} points, niter {res['niter']}, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
