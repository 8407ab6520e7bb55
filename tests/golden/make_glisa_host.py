"""Write the fixtures of the reference's gLISA solvers that iterate on the
host (DIIS, CDIIS, quasi-Newton, trust-region; glisa.py:595-615, 883-1028),
by running the unmodified reference through ``oracle/refrun.py``.

    HP_REFERENCE_SRC=<horton-part checkout>/src python tests/golden/make_glisa_host.py

Input: the H2O case of the golden suite (50 radial x Lebedev-110 per atom,
the reference's default Gaussian basis), threshold 1e-8. Each
``glisa_<solver>_h2o_50x110.npz`` holds the reference's charges, parameters,
iteration count (where the reference stores one) and histories.
"""

import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from horton_part_gb300 import synthetic  # noqa: E402
from oracle import refrun  # noqa: E402

HOST_CASES = ("diis", "cdiis", "quasi-newton", "trust-region")


def build_host_inputs():
    return synthetic.water(nrad=50, nang=110)


def fixture_name(solver):
    return f"glisa_{solver.replace('-', '')}_h2o_50x110"


def main():
    if not refrun.available():
        raise SystemExit("reference source not found; set HP_REFERENCE_SRC")
    warnings.simplefilter("ignore")
    mol = build_host_inputs()
    for solver in HOST_CASES:
        ref = refrun.run("glisa", mol.coordinates, mol.numbers, mol.pseudo_numbers, mol.grid.points,
                         mol.grid.weights, mol.density, threshold=1e-8, solver=solver)
        out = {k: np.asarray(ref[k]) for k in ("charges", "propars", "history_entropies",
                                                "history_propars", "history_changes") if k in ref}
        out["niter"] = np.asarray(ref.get("niter", -1))
        out["fp_weights"] = mol.grid.weights.sum()
        out["fp_density"] = np.dot(mol.grid.weights, mol.density)
        np.savez(os.path.join(HERE, fixture_name(solver) + ".npz"), **out)
        print(solver, "niter", int(out["niter"]), "charges", out["charges"])


if __name__ == "__main__":
    main()
