"""The part-gen program on the GPU path (scripts/generate_density.py:208-262):
wavefunction file -> grid and density -> result file, then part-dens
(MBIS) on that file, against the reference's own MBIS known answer for the
same water wavefunction (tests/test_wpart.py:95-101 of horton-part: charges
[-0.61891067, 0.3095756, 0.30932584] within 2e-3, on its own grid)."""

import os

import numpy as np
import pytest

from fchk_fixture import load_fixture, render_fchk
from horton_part_gb300 import part_dens, part_gen

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MBIS_WATER = np.array([-0.61891067, 0.3095756, 0.30932584])


def test_part_gen_then_part_dens_water(tmp_path, gpu_context):
    fx = load_fixture(os.path.join(GOLDEN, "density_water_sto3g.npz"))
    fchk = tmp_path / "water.fchk"
    render_fchk(fx, fchk)
    cfg = tmp_path / "gen.yaml"
    cfg.write_text(f"nrad: 100\nnang: 110\ninputs:\n  - {fchk}\noutputs:\n  - {tmp_path / 'dens.npz'}\n")
    assert part_gen.main([str(cfg)]) == 0
    with np.load(tmp_path / "dens.npz") as f:
        d = {k: f[k] for k in f.files}
    for key in ("density", "atcoords", "atnums", "atcorenums", "points", "weights", "aim_weights",
                "cellvecs", "nelec", "atom_idxs", "atom0/points", "atom2/rgrid/weights"):
        assert key in d
    assert d["points"].shape == (3 * 100 * 110, 3) and (d["density"] >= 0).all()
    assert abs(float(d["weights"] @ d["density"]) - 10.0) < 1e-3  # ten electrons
    lo, hi = int(d["atom_idxs"][0]), int(d["atom_idxs"][1])
    np.testing.assert_allclose(d["aim_weights"][lo:hi] * d["atom0/weights"], d["weights"][lo:hi],
                               rtol=1e-12)
    dcfg = tmp_path / "dens.yaml"
    dcfg.write_text(f"type: mbis\ngrid_type: 3\nthreshold: 1.0e-8\ninputs:\n  - {tmp_path / 'dens.npz'}\n"
                    f"outputs:\n  - {tmp_path / 'out.npz'}\n")
    assert part_dens.main([str(dcfg)]) == 0
    with np.load(tmp_path / "out.npz") as f:
        q = f["charges"]
    assert np.abs(q - MBIS_WATER).max() < 2e-3
    assert abs(q.sum()) < 1e-3
