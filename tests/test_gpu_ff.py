"""MBIS in float-float arithmetic (precision "ff") and the mixed-precision
path that finishes in float-float (precision "mixed", polish on).

"ff" evaluates distances, shell exponentials, pro-atoms, at_weights and the
moments in float pairs (~48 significant bits) on the FP32 pipes; the
parameter updates and tests are FP64. It must reproduce the reference's FP64
results like the FP64 path does: same iteration counts, charges to 1e-9 e.
"""

import os
import warnings

import numpy as np
import pytest

from cases import CASES, build_inputs
from horton_part_gb300 import synthetic
from horton_part_gb300.utils import wpart_schemes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MBIS_CASES = [n for n, c in sorted(CASES.items()) if c["scheme"] == "mbis"]


def _run(mol, precision, **kwargs):
    part = wpart_schemes("mbis")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=3, precision=precision, **kwargs)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        part.do_partitioning()
    return part


def _scaled_dp(p, ref):
    n = p[0::2], ref[0::2]
    s = p[1::2], ref[1::2]
    return max(float(np.abs(n[0] - n[1]).max() / np.abs(n[1]).max()),
               float(np.abs(s[0] - s[1]).max() / np.abs(s[1]).max()))


@pytest.mark.parametrize("name", MBIS_CASES)
def test_ff_matches_reference(name, gpu_context):
    case = CASES[name]
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as f:
        g = {k: f[k] for k in f.files}
    mol, kwargs = build_inputs(case)
    part = _run(mol, "ff", **kwargs)
    dq = float(np.abs(part["charges"] - g["charges"]).max())
    dp = _scaled_dp(part["propars"], g["propars"])
    print(f"{name} ff: niter {part['niter']} (reference {int(g['niter'])}), max|dq| {dq:.2e}, "
          f"max scaled dp {dp:.2e}")
    assert part["niter"] == int(g["niter"])
    assert dq < 1e-9
    assert dp < 1e-9


@pytest.mark.parametrize("name", MBIS_CASES)
def test_mixed_with_ff_finish_matches_reference(name, gpu_context):
    case = CASES[name]
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as f:
        g = {k: f[k] for k in f.files}
    mol, kwargs = build_inputs(case)
    part = _run(mol, "mixed", **kwargs)
    dq = float(np.abs(part["charges"] - g["charges"]).max())
    print(f"{name} mixed+ff finish: niter {part['niter']} (reference {int(g['niter'])}), "
          f"finish iterations {part.job_info.polish_iterations}, max|dq| {dq:.2e}")
    assert dq < 1e-7


def test_ff_matches_fp64_on_a_larger_molecule(gpu_context):
    """A 16-atom chain (75 x Lebedev-110 per atom): ff and FP64 take the
    same iterations and agree to 1e-9 e."""
    mol = synthetic.batch_molecules(natoms=[16], nrad=75, nang=110, seed=5)[0]
    ff = _run(mol, "ff", threshold=1e-8, maxiter=300)
    fp = _run(mol, "fp64", threshold=1e-8, maxiter=300)
    dq = float(np.abs(ff["charges"] - fp["charges"]).max())
    print(f"chain16: niter ff {ff['niter']} fp64 {fp['niter']}, max|dq| {dq:.2e}")
    assert ff["niter"] == fp["niter"]
    assert dq < 1e-9
