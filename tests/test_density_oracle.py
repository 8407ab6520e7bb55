"""The density generator's host side and oracle, on the CPU: the fchk parser
and the FP64 restatement of the density against the densities stored
beside horton-part's own fchk test files (tests/golden/density_*.npz,
written by tests/golden/make_density.py), the pure-function tables, and the
parser's error paths."""

import glob
import math
import os

import numpy as np
import pytest

from fchk_fixture import load_fixture, render_fchk
from horton_part_gb300 import gto
from horton_part_gb300.fchk import Shell, load_fchk
from oracle import hp_density as H

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "density_*.npz")))


def _ids(path):
    return os.path.basename(path)[8:-4]


@pytest.mark.parametrize("path", FIXTURES, ids=_ids)
def test_oracle_density_matches_the_reference_data(path, tmp_path):
    fx = load_fixture(path)
    render_fchk(fx, tmp_path / "w.fchk")
    data = load_fchk(str(tmp_path / "w.fchk"))
    assert data.nbasis == int(fx["f:Number of basis functions"])
    if "azirine" in path:
        assert data.one_rdm_kind == "post_scf"  # generate_density.py:146 prefers the post-SCF density
    rho = H.density(data.one_rdm, data.shells, fx["points"])
    ref = fx["dens"]
    assert np.abs(rho - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs((rho - ref) / ref).max() < 1e-12
    if "spin_dens" in fx:
        spin = H.density(data.spin_rdm, data.shells, fx["points"])
        assert np.abs(spin - fx["spin_dens"]).max() <= 1e-13 * np.abs(fx["spin_dens"]).max()


def test_sp_shells_split_and_atoms():
    fx = load_fixture(os.path.join(GOLDEN, "density_water_sto3g.npz"))
    fields = {k[2:]: v for k, v in fx.items() if k.startswith("f:")}
    nsp = int(np.sum(fields["Shell types"] == -1))
    assert nsp > 0
    from horton_part_gb300.fchk import FchkData
    data = FchkData(fields)
    assert len(data.shells) == len(fields["Shell types"]) + nsp
    assert [s.atom for s in data.shells][0] == 0 and data.natom == 3
    assert np.allclose(data.one_rdm, data.one_rdm.T)


@pytest.mark.parametrize("l", [2, 3])
def test_pure_tables_are_orthonormal_and_match_the_oracle_forms(l):
    T = gto.pure_matrix(l)
    G = gto._cart_overlap(l)
    np.testing.assert_allclose(T @ G @ T.T, np.eye(2 * l + 1), atol=1e-14)
    rng = np.random.default_rng(5)
    x, y, z = rng.normal(size=(3, 50))
    cart = np.array([x ** i * y ** j * z ** k for i, j, k in gto.cartesian_powers(l)])
    np.testing.assert_allclose(T @ cart, np.array(H._angular(l, True, x, y, z)), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(cart, np.array(H._angular(l, False, x, y, z)), rtol=1e-15)


def test_primitive_normalisation():
    """A primitive of each l is normalised as x^l (numerical quadrature)."""
    a = 0.7
    t = np.linspace(-8, 8, 4001)
    h = t[1] - t[0]
    for l in range(4):
        n = gto.primitive_norm(np.array([a]), l)[0]
        one_d = [np.sum(t ** (2 * k) * np.exp(-2 * a * t * t)) * h for k in (l, 0, 0)]
        assert n * n * math.prod(one_d) == pytest.approx(1.0, rel=1e-10)


def test_density_from_orbitals(tmp_path):
    """Without a stored density matrix the density comes from the occupied
    orbitals (generate_density.py:149-155)."""
    fx = load_fixture(os.path.join(GOLDEN, "density_water_sto3g.npz"))
    data = load_fchk(_render(fx, tmp_path))
    w, v = np.linalg.eigh(data.one_rdm)  # a rank-5 closed-shell density: 2 C C^T
    occ = v[:, -5:] * np.sqrt(w[-5:] / 2.0)
    fields = {k[2:]: fx[k] for k in fx if k.startswith("f:") and "Density" not in k}
    fields["Alpha MO coefficients"] = occ[:, ::-1].T.ravel()
    fields["Number of alpha electrons"] = 5
    fields["Number of beta electrons"] = 5
    from horton_part_gb300.fchk import FchkData
    d2 = FchkData(fields)
    assert d2.one_rdm_kind == "mo"
    np.testing.assert_allclose(d2.one_rdm, data.one_rdm, atol=1e-12)


def _render(fx, tmp_path):
    path = str(tmp_path / "x.fchk")
    render_fchk(fx, path)
    return path


def test_parser_errors(tmp_path):
    bad = tmp_path / "bad.fchk"
    bad.write_text("only one line\n")
    with pytest.raises(ValueError):
        load_fchk(str(bad))
    fx = load_fixture(os.path.join(GOLDEN, "density_water_sto3g.npz"))
    fx["f:Number of basis functions"] = np.array(8)
    with pytest.raises(ValueError):
        load_fchk(_render(fx, tmp_path))
    with pytest.raises(NotImplementedError):
        gto.shell_tables([Shell(np.zeros(3), 4, True, [1.0], [1.0], 0)])
