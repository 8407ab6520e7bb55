"""The validators' error and warning paths (utils.py:305-398), provoked with
inputs on the GPU path.

check_pro_atom_parameters raises RuntimeError when the pro-atom density has
values below negative_cutoff and warns when the populations do not sum to
the molecule's within population_cutoff. A positive negative_cutoff makes
every point of the final promolecule "negative"; a population_cutoff far
below rounding makes the population check fail. The gLISA Newton solver
applies both checks at convergence (glisa.py:786-798); the host-driven DIIS
applies them at its end (glisa.py:902-909).
"""

import logging

import numpy as np
import pytest

from horton_part_gb300 import synthetic
from horton_part_gb300.utils import wpart_schemes

pytestmark = pytest.mark.gpu


def _glisa(solver, **kw):
    mol = synthetic.water(nrad=30, nang=50)
    return wpart_schemes("glisa")(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                  mol.density, grid_type=3, solver=solver, threshold=1e-8, **kw)


@pytest.mark.parametrize("solver", ["newton", "diis"])
def test_negative_pro_atom_density_raises(solver, gpu_context):
    part = _glisa(solver, negative_cutoff=1.0)
    with pytest.raises(RuntimeError, match="[Nn]egative"):
        part.do_partitioning()


@pytest.mark.parametrize("solver", ["newton", "diis"])
def test_population_mismatch_warns(solver, gpu_context, caplog):
    logger = logging.getLogger(f"hp-validators-{solver}")
    part = _glisa(solver, population_cutoff=1e-300, logger=logger)
    with caplog.at_level(logging.WARNING, logger=logger.name):
        part.do_partitioning()
    assert any("population" in r.getMessage() for r in caplog.records)
    # the result itself is unaffected
    ref = _glisa(solver)
    ref.do_partitioning()
    np.testing.assert_allclose(part["charges"], ref["charges"], rtol=0, atol=1e-12)
