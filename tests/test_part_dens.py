"""The part-dens program (scripts/partition_density.py:172-348): settings,
density files in the reference's layout and the rebuilt molecular grid (CPU),
and the whole program on the GPU path (marked gpu)."""

import os

import numpy as np
import pytest

from horton_part_gb300 import part_dens, synthetic
from horton_part_gb300.molgrid import atom_grid_arrays

OUTPUT_KEYS = {"natom", "atnums", "atcorenums", "type", "lmax", "maxiter", "threshold",
               "inner_threshold", "solver", "charges", "time", "time_update_at_weights",
               "time_update_propars", "niter", "history_charges", "history_propars",
               "history_entropies", "history_changes"}


def write_density_file(path, mol):
    """A density file in the layout of the reference's density generator
    (scripts/generate_density.py:232-257) for a synthetic molecule."""
    g = mol.grid
    data = {"atcoords": mol.coordinates, "atnums": mol.numbers, "atcorenums": mol.pseudo_numbers,
            "points": g.points, "weights": g.weights, "density": mol.density,
            "atom_idxs": np.asarray(g.indices), "cellvecs": np.zeros((0, 3)),
            "nelec": float(mol.numbers.sum())}
    aim = np.empty(g.size)
    for a, ag in enumerate(g.atgrids):
        lo, hi = g.indices[a], g.indices[a + 1]
        r, wr = ag.rgrid.points, ag.rgrid.weights
        shell = np.repeat(np.arange(r.size), np.diff(ag.shell_offsets))
        w_atom = wr[shell] * r[shell] ** 2 * 4.0 * np.pi * ag.sphere_weights
        aim[lo:hi] = g.weights[lo:hi] / w_atom
        data[f"atom{a}/points"] = g.points[lo:hi]
        data[f"atom{a}/weights"] = w_atom
        data[f"atom{a}/shell_idxs"] = ag.shell_offsets
        data[f"atom{a}/rgrid/points"] = r
        data[f"atom{a}/rgrid/weights"] = wr
    data["aim_weights"] = aim
    np.savez_compressed(path, **data)


def test_settings_reader(tmp_path):
    p = tmp_path / "cfg.yaml"
    p.write_text("# a part-dens configuration\n"
                 "type: mbis\nthreshold: 1.0e-8\nmaxiter: 200\ngrid_type: 3\n"
                 "solver: 'sc'\nfunc_file: null\nsave: [charges, niter]\n"
                 "inputs:\n  - a.npz\n  - b.npz\noutputs:\n  - out/a.npz\n  - out/b.npz\n")
    s = part_dens.read_settings(p)
    assert s["type"] == "mbis" and s["threshold"] == 1e-8 and s["maxiter"] == 200
    assert s["solver"] == "sc" and s["func_file"] is None and s["save"] == ["charges", "niter"]
    assert s["inputs"] == ["a.npz", "b.npz"] and s["outputs"][1] == "out/b.npz"
    (tmp_path / "c.json").write_text('{"type": "glisa", "inputs": ["x.npz"]}')
    assert part_dens.read_settings(tmp_path / "c.json")["type"] == "glisa"


def test_density_file_rebuilds_the_grid(tmp_path):
    mol = synthetic.water(nrad=20, nang=50)
    fn = tmp_path / "h2o.npz"
    write_density_file(fn, mol)
    with np.load(fn) as f:
        data = {k: f[k] for k in f.files}
    grid = part_dens.molgrid_from_density(data)
    np.testing.assert_array_equal(grid.points, mol.grid.points)
    np.testing.assert_array_equal(grid.weights, mol.grid.weights)
    a, b = atom_grid_arrays(grid), atom_grid_arrays(mol.grid)
    for k in a:
        np.testing.assert_allclose(a[k], b[k], rtol=1e-13, atol=0)
    assert grid.integrate(data["density"]) == pytest.approx(10.0, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,grid_type", [("mbis", 1), ("mbis", 3), ("lisa", 3), ("glisa", 3)])
def test_part_dens_program(tmp_path, kind, grid_type, gpu_context):
    """The program's result file carries the reference's keys and the charges
    of the same class run directly on the same grid."""
    from horton_part_gb300.utils import wpart_schemes

    mol = synthetic.water(nrad=30, nang=50)
    fn_in = tmp_path / "h2o.npz"
    write_density_file(fn_in, mol)
    cfg = tmp_path / "cfg.yaml"
    out = tmp_path / "res" / "h2o_out.npz"
    solver = "newton" if kind == "glisa" else "sc"
    cfg.write_text(f"type: {kind}\nthreshold: 1.0e-8\ngrid_type: {grid_type}\nsolver: {solver}\n"
                   f"inputs:\n  - {fn_in}\noutputs:\n  - {out}\nlog_files:\n  - {tmp_path / 'log.txt'}\n")
    assert part_dens.main([str(cfg)]) == 0
    with np.load(out) as f:
        res = {k: f[k] for k in f.files}
    assert OUTPUT_KEYS <= set(res)
    kw = dict(grid_type=grid_type, threshold=1e-8, maxiter=1000, lmax=3)
    if kind != "glisa":
        kw["inner_threshold"] = 1e-8
    if kind != "mbis":
        kw["solver"] = solver
    direct = wpart_schemes(kind)(mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid,
                                 mol.density, **kw)
    direct.do_partitioning()
    np.testing.assert_allclose(res["charges"], direct["charges"], rtol=0, atol=1e-12)
    assert int(res["niter"]) == int(direct["niter"])
    assert os.path.exists(tmp_path / "log.txt")
