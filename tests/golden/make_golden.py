"""Write the golden fixtures in this folder by running the unmodified
reference (horton-part) on seeded synthetic inputs.

Run from the repository root, naming the reference's source tree:

    HP_REFERENCE_SRC=<horton-part checkout>/src python tests/golden/make_golden.py

Each ``<case>.npz`` holds the reference's results (charges, pro-atom
parameters, iteration counts and histories) plus fingerprints of the inputs
(sums of the grid weights and density), so that tests can regenerate the
inputs with :mod:`horton_part_gb300.synthetic` on any machine and confirm they
are the same arrays before comparing results.
"""

import os
import sys
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from cases import CASES, build_inputs  # noqa: E402
from oracle import refrun  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = ("charges", "propars", "niter", "change", "history_changes", "history_entropies",
        "history_propars", "history_charges", "populations", "pseudo_populations",
        "core_charges", "valence_charges", "valence_widths")


def main(names=None):
    if not refrun.available():
        raise SystemExit("reference source not found; set HP_REFERENCE_SRC")
    warnings.simplefilter("ignore")
    for name, case in CASES.items():
        if names and name not in names:
            continue
        mol, kwargs = build_inputs(case)
        ref = refrun.run(case["scheme"], mol.coordinates, mol.numbers, mol.pseudo_numbers,
                         mol.grid.points, mol.grid.weights, mol.density, **kwargs)
        out = {k: np.asarray(ref[k]) for k in KEYS if k in ref}
        out["fp_weights"] = np.array(mol.grid.weights.sum())
        out["fp_density"] = np.array(np.dot(mol.grid.weights, mol.density))
        out["fp_points"] = np.array(np.abs(mol.grid.points).sum())
        out["fp_rho_abs"] = np.array(mol.density.sum())
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, "niter", int(out["niter"]), "charges", out["charges"])


if __name__ == "__main__":
    main(sys.argv[1:])
