"""``part-gen``: molecular grids and electron densities from wavefunction
files, as horton-part's ``part-gen`` program
(``scripts/generate_density.py:208-262``, settings ``data/part-gen.yaml``),
with the density on the GPU.

    python -m horton_part_gb300.part_gen config.yaml [--skip_exist_files]

Inputs are Gaussian formatted checkpoint files (``.fchk``; the reference
reads any iodata format). Per input the program builds an atom-centred
grid (Gauss-Chebyshev radial nodes mapped by Becke's transform with r_min
1e-4 and R 1.5, as ``_setup_grid``; Lebedev angular rules; Becke (k = 3)
fuzzy-cell weights), evaluates the density with
:class:`horton_part_gb300.density.DensityPlan` and writes the result file
with the keys the reference writes (``density``, ``atcoords``, ``atnums``,
``atcorenums``, ``points``, ``weights``, ``aim_weights``, ``cellvecs``,
``nelec``, ``atom_idxs`` and per atom ``atom<i>/points``, ``weights``,
``shell_idxs``, ``rgrid/points``, ``rgrid/weights``), which
:mod:`horton_part_gb300.part_dens` reads.

Differences from the reference, by construction: the Becke weights carry no
atomic-size adjustment (the reference's qc-grid ``BeckeWeights`` adjusts
cell boundaries by tabulated radii), and the angular rules are the
tabulated Lebedev rules of :func:`horton_part_gb300.molgrid.lebedev` (50,
110, 194, 302, 590 points). Density gradients and orbitals on the grid
(``gradient``, ``orbitals``) are not produced.
"""

from __future__ import annotations

import argparse
import logging
import os
import sys
import time

import numpy as np

from .density import DensityPlan
from .fchk import load_fchk
from .molgrid import becke_molecular_grid, lebedev
from .part_dens import read_settings

__all__ = ["DEFAULTS", "grid_and_density", "run_one", "main"]

# The reference's defaults of the part-gen program (data/part-gen.yaml).
DEFAULTS = {"log_level": "WARNING", "nrad": 150, "nang": 194, "chunk_size": 10000,
            "gradient": False, "orbitals": False}


def grid_and_density(data, nrad, nang, context=None):
    """(MolecularGrid, density) of a wavefunction read by ``load_fchk``."""
    grid = becke_molecular_grid(data.atcoords, int(nrad), int(nang))
    plan = DensityPlan(data.shells, data.one_rdm, context=context)
    try:
        rho = plan.evaluate(grid.points)[0]
    finally:
        plan.close()
    return grid, rho


def result_arrays(data, grid, rho):
    """The result file's arrays (generate_density.py:229-255)."""
    natom = data.natom
    idx = np.asarray(grid.indices, dtype=np.int64)
    out = {
        "density": rho, "atcoords": data.atcoords, "atnums": data.atnums,
        "atcorenums": data.atcorenums, "points": grid.points, "weights": grid.weights,
        "cellvecs": np.zeros((0, 3)),
        "nelec": float(data.fields.get("Number of electrons", np.sum(data.atcorenums))),
        "atom_idxs": idx,
    }
    aim = np.empty(grid.size)
    for a in range(natom):
        ag = grid.atgrids[a]
        sl = slice(int(idx[a]), int(idx[a + 1]))
        nang = int(ag.shell_offsets[1] - ag.shell_offsets[0])
        r, wr = ag.rgrid.points, ag.rgrid.weights
        _, wang = lebedev(nang)
        atw = ((wr * r * r)[:, None] * wang[None, :]).reshape(-1)  # radial x angular weights
        aim[sl] = grid.weights[sl] / atw  # the Becke weight of each point
        out[f"atom{a}/points"] = grid.points[sl]
        out[f"atom{a}/weights"] = atw
        out[f"atom{a}/shell_idxs"] = np.asarray(ag.shell_offsets, dtype=np.int64)
        out[f"atom{a}/rgrid/points"] = r
        out[f"atom{a}/rgrid/weights"] = wr
    out["aim_weights"] = aim
    return out


def run_one(settings, fn_in, fn_out, fn_log=None, context=None):
    lg = logging.getLogger("part-gen")
    lg.setLevel(getattr(logging, str(settings.get("log_level", "WARNING")).upper(), logging.WARNING))
    for h in list(lg.handlers):
        lg.removeHandler(h)
    h = logging.FileHandler(fn_log) if fn_log else logging.StreamHandler(sys.stdout)
    lg.addHandler(h)
    lg.propagate = False
    if settings.get("gradient") or settings.get("orbitals"):
        raise NotImplementedError("part-gen: density gradients and orbitals on the grid are not produced")
    data = load_fchk(fn_in)
    lg.info(f"part-gen: {fn_in}: {data.natom} atoms, {data.nbasis} basis functions, "
            f"density matrix: {data.one_rdm_kind}")
    grid, rho = grid_and_density(data, settings["nrad"], settings["nang"], context=context)
    if not (rho >= 0).all():  # generate_density.py:201
        raise RuntimeError("negative density on the grid")
    d = os.path.dirname(os.path.abspath(fn_out))
    os.makedirs(d, exist_ok=True)
    np.savez_compressed(fn_out, **result_arrays(data, grid, rho))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(prog="part-gen", description="Molecular grids and densities on the GPU path.")
    ap.add_argument("config_file")
    ap.add_argument("--skip_exist_files", action="store_true",
                    help="skip inputs whose output (and log) file exists")
    args = ap.parse_args(argv)
    settings = read_settings(args.config_file)
    for k, v in DEFAULTS.items():
        settings.setdefault(k, v)
    inputs = settings.get("inputs")
    if not isinstance(inputs, list):
        raise RuntimeError("the settings need a list of 'inputs'")
    outputs = settings.setdefault("outputs", [f"output_{i + 1}.npz" for i in range(len(inputs))])
    logs = settings.setdefault("log_files", [None] * len(inputs))
    if not len(inputs) == len(outputs) == len(logs):
        raise RuntimeError("The settings for part-gen is not fully correct.")
    rc = 0
    for fn_in, fn_out, fn_log in zip(inputs, outputs, logs):
        if args.skip_exist_files and os.path.exists(fn_out) and (fn_log is None or os.path.exists(fn_log)):
            print(f"Skip the calculations with input: {fn_in}")
            continue
        t0 = time.time()
        rc |= run_one(settings, fn_in, fn_out, fn_log)
        print(f"{fn_in} -> {fn_out} ({time.time() - t0:.2f} s)")
    return rc


if __name__ == "__main__":
    sys.exit(main())
