"""aLISA (sc) on the construction of the large-molecule workload (peptide-like
chain with S, 6-10 s-Gaussians per element up to exponent 500), at a size the
oracle finishes: 11 atoms on 20 x Lebedev-50 points per atom.

FP64 must match the oracle's iteration count and charges to 1e-8 e; the
mixed form (FP32 bulk, FP64 finish) to 1e-6 e. The per-atom cutoff of the
inner solve is active on both (the molecule is 18 bohr long).
"""

import os
import sys

import numpy as np
import pytest

from horton_part_gb300.utils import wpart_schemes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)
from make_lisa_peptide import build_peptide_inputs, fingerprint  # noqa: E402


@pytest.mark.parametrize("precision,q_tol", [("fp64", 1e-8), ("mixed", 1e-6)])
def test_lisa_sc_peptide_matches_the_oracle(precision, q_tol, gpu_context):
    with np.load(os.path.join(GOLDEN, "lisa_sc_peptide11_20x50.npz")) as f:
        g = {k: f[k] for k in f.files}
    mol, helper = build_peptide_inputs()
    np.testing.assert_allclose(fingerprint(mol), g["fingerprint"], rtol=1e-10)
    part = wpart_schemes("lisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=3, solver="sc", basis_func=helper,
                                 threshold=1e-6, inner_threshold=1e-8, precision=precision)
    part.do_partitioning()
    info = part.job_info
    dq = float(np.abs(part["charges"] - g["charges"]).max())
    print(f"aLISA sc peptide {precision}: niter {part['niter']} (oracle {int(g['niter'])}), "
          f"max|dq| {dq:.2e} e, skipped {info.point_atom_evals_skipped / info.point_atom_evals:.1%}")
    assert dq < q_tol
    if precision == "fp64":
        assert part["niter"] == int(g["niter"])
