"""gLISA solvers that iterate on the host (DIIS, CDIIS, quasi-Newton,
trust-region) through the public class: the iteration logic on the host,
every pass over the grid on the device (hp_glisa_evaluate, hp_glisa_change,
hp_glisa_line_search, hp_glisa_finish). Against the unmodified reference's
own runs (fixtures from tests/golden/make_glisa_host.py): its iteration count
and charges to 1e-8 e; trust-region (which stops on a step tolerance well
before the optimum) within 2e-5 e of the reference's run and of the optimum.
"""

import os
import sys

import numpy as np
import pytest

from horton_part_gb300.utils import wpart_schemes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)
from make_glisa_host import HOST_CASES, build_host_inputs, fixture_name  # noqa: E402


def _fixture(name):
    with np.load(os.path.join(GOLDEN, fixture_name(name) + ".npz")) as f:
        return {k: f[k] for k in f.files}


@pytest.mark.parametrize("solver", HOST_CASES)
def test_host_solver_on_the_device_matches_the_reference(solver, gpu_context):
    mol = build_host_inputs()
    g = _fixture(solver)
    part = wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver=solver, threshold=1e-8)
    part.do_partitioning()
    dq = float(np.abs(part["charges"] - g["charges"]).max())
    print(f"{solver}: niter {part['niter']} (reference {int(g['niter'])}), max|dq| {dq:.2e} e")
    if solver == "trust-region":
        optimum = _fixture("diis")["charges"]
        assert dq < 2e-5 and float(np.abs(part["charges"] - optimum).max()) < 2e-5
        return
    assert dq < 1e-8
    assert part["niter"] == int(g["niter"])
    if solver == "quasi-newton":
        np.testing.assert_allclose(part["history_entropies"], g["history_entropies"], rtol=1e-9,
                                   atol=1e-12)


def test_host_solvers_refuse_mixed_precision(gpu_context):
    mol = build_host_inputs()
    part = wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver="diis", precision="mixed")
    with pytest.raises(NotImplementedError):
        part.do_partitioning()
