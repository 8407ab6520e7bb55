"""NLIS / GMBIS host logic (no GPU): initial parameters against the values
in the reference's own tests, the shell counts, and the reference's
behaviour with its default ``exp_n_dict`` (tests/test_nlis.py of horton-part:
``test_get_nlis_nshell``, ``test_get_initial_nlis_propars``)."""

import numpy as np
import pytest

from horton_part_gb300 import synthetic
from horton_part_gb300.nlis import (get_initial_gmbis_propars, get_initial_nlis_propars,
                                    get_nlis_nshell)
from horton_part_gb300.utils import wpart_schemes
from oracle import hp_oracle as O


@pytest.mark.parametrize("nshell", [4, 5, 6])
def test_nlis_nshell_from_dict(nshell):
    nsd = {n: nshell for n in range(1, 119)}
    for z in (1, 2, 3, 17, 18, 21, 44, 72, 104):
        assert get_nlis_nshell(z, nsd) == nshell
    assert get_nlis_nshell(8, {}) == 2  # MBIS shell count without an entry


def test_initial_nlis_propars_known_answer():
    nsd = {n: 4 for n in range(1, 119)}
    expn = {(1, k): 2 for k in range(4)}
    values_h = get_initial_nlis_propars(1, expn, nsd)
    assert values_h == pytest.approx([0.25, 2.0, 2.0, 0.25, 1.25992105, 2.0,
                                      0.25, 0.79370053, 2.0, 0.25, 0.5, 2.0])
    np.testing.assert_allclose(values_h, O.nlis_initial_propars(1, expn, nsd), rtol=0, atol=0)


def test_initial_gmbis_propars_match_the_oracle():
    expn = {(8, 1): 2.0}
    for z in (1, 6, 8, 17):
        np.testing.assert_allclose(get_initial_gmbis_propars(z, expn),
                                   O.gmbis_initial_propars(z, expn), rtol=0, atol=0)
    p = get_initial_gmbis_propars(8, expn)
    assert p[0::3].sum() == pytest.approx(8.0) and p[5] == 2.0


@pytest.mark.parametrize("scheme", ["nlis", "gmbis"])
def test_default_exp_n_dict_fails_like_the_reference(scheme):
    """exp_n_dict defaults to 1.0 in the reference and is used as a mapping:
    TypeError at the first membership test (nlis.py:92, gmbis.py:48)."""
    mol = synthetic.water(nrad=10, nang=50)
    part = wpart_schemes(scheme)(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, grid_type=3)
    with pytest.raises(TypeError):
        part.do_partitioning()
