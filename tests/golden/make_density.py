"""Write the density-generator fixtures from the reference's own test data.

    HP_REFERENCE_TESTS=<horton-part checkout>/tests python tests/golden/make_density.py

horton-part's ``tests/cached`` holds Gaussian formatted checkpoint files and,
beside several of them, the electron density (and spin density) evaluated
on grid points (``*.npz``: ``points``, ``dens``[, ``spin_dens``]). For each
pair this script stores in ``density_<name>.npz`` the fields of the file the
density needs (shells with their primitives, density matrices as stored,
atoms) and a seeded sample of 1500 points with their reference densities.
The tests render the fields back into fchk text, parse it with
``horton_part_gb300.fchk`` and compare the densities (CPU oracle and GPU).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from horton_part_gb300.fchk import load_fchk  # noqa: E402

CASES = {
    "water_sto3g": ("water_sto3g_hf_g03.fchk", "water_sto3g_hf_g03_fchk_exp:5e-4:2e1:120:110.npz"),
    "azirine_cc": ("2h-azirine-cc.fchk", "2h-azirine-cc-fchk-medium.npz"),
    "azirine_mp2": ("2h-azirine-mp2.fchk", "2h-azirine-mp2-fchk-medium.npz"),
    "ch3_sto3g": ("ch3_hf_sto3g.fchk", "ch3_hf_sto3g_fchk_medium.npz"),
    "lih_321g": ("li_h_3-21G_hf_g09.fchk", "li_h_3-21G_hf_g09_fchk_exp:1e-3:1e1:100:110.npz"),
    "sioh4_lanl2dz": ("monosilicic_acid_hf_lan.fchk",
                      "monosilicic_acid_hf_lan_fchk_exp:5e-4:2e1:120:110.npz"),
    "n2_sto3g": ("n2_hfs_sto3g.fchk", "n2_hfs_sto3g_fchk_exp:1e-3:1e1:100:110.npz"),
}

# fchk records a density fixture keeps (name -> kind)
FIELDS = {
    "Number of electrons": "I", "Number of alpha electrons": "I", "Number of beta electrons": "I",
    "Number of basis functions": "I", "Atomic numbers": "IA", "Nuclear charges": "RA",
    "Current cartesian coordinates": "RA", "Shell types": "IA",
    "Number of primitives per shell": "IA", "Shell to atom map": "IA", "Primitive exponents": "RA",
    "Contraction coefficients": "RA", "P(S=P) Contraction coefficients": "RA",
    "Coordinates of each shell": "RA",
}


def _key(name):
    return "f:" + name


def main():
    base = os.environ.get("HP_REFERENCE_TESTS")
    if not base:
        raise SystemExit("set HP_REFERENCE_TESTS to the reference's tests directory")
    rng = np.random.default_rng(20240611)
    for name, (fchk, npz) in CASES.items():
        data = load_fchk(os.path.join(base, "cached", fchk))
        out = {}
        for field in FIELDS:
            if field in data.fields:
                out[_key(field)] = np.asarray(data.fields[field])
        for field, value in data.fields.items():
            if field.endswith(" Density") and (field.startswith("Total") or field.startswith("Spin")):
                out[_key(field)] = np.asarray(value)
        with np.load(os.path.join(base, "cached", npz)) as g:
            idx = np.sort(rng.choice(len(g["points"]), size=min(1500, len(g["points"])), replace=False))
            out["points"] = g["points"][idx]
            out["dens"] = g["dens"][idx]
            if "spin_dens" in g.files:
                out["spin_dens"] = g["spin_dens"][idx]
        out["title"] = np.array(data.title)
        np.savez_compressed(os.path.join(HERE, f"density_{name}.npz"), **out)
        print(name, data.nbasis, len(out["points"]), sorted(k for k in out if k.startswith("f:")))


if __name__ == "__main__":
    main()
