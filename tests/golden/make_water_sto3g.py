"""Write ``water_sto3g_hf_molgrid.npz``: the reference's own cached water
HF/STO-3G density on its 120-radial x Lebedev-110 molecular grid, for the
known-answer test of horton-part's ``tests/test_wpart.py`` (MBIS charges
[-0.61891067, 0.3095756, 0.30932584], tolerance 2e-3).

The cached file (``tests/cached/water_sto3g_hf_g03_fchk_exp:5e-4:2e1:120:110.npz``
in the reference tree) stores the points and the density but not the grid
weights. As the reference's test does (test_wpart.py:46-55), the grid is
rebuilt - radial ExpRTransform(5e-4, 20, 119) over 120 integer nodes times
the Lebedev-110 rule on every atom - and the stored points are matched to it
row by row (to 1e-6 bohr); the weights are radial x angular x the Becke
fuzzy-cell weight (this package's unadjusted Becke partition). The fixture
holds the matched points, weights and density plus the molecule.

Run from the repository root where the reference tree is available:

    python tests/golden/make_water_sto3g.py [path/to/reference]
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from horton_part_gb300.molgrid import becke_partition_weights, lebedev  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
CACHED = "tests/cached/water_sto3g_hf_g03_fchk_exp:5e-4:2e1:120:110.npz"


def exp_radial(rmin=5e-4, rmax=20.0, n=120):
    """ExpRTransform over integer nodes 0..n-1: r_i = rmin (rmax/rmin)^(i/(n-1)),
    dr/di = r_i ln(rmax/rmin)/(n-1) (unit weights of the integer grid)."""
    i = np.arange(n, dtype=np.float64)
    c = np.log(rmax / rmin) / (n - 1)
    r = rmin * np.exp(c * i)
    return r, r * c


def main(reference=None):
    reference = reference or os.environ.get("HP_REFERENCE_ROOT")
    if not reference:
        raise SystemExit("set HP_REFERENCE_ROOT to the reference checkout (its tests/cached data)")
    with np.load(os.path.join(reference, CACHED)) as f:
        dens, stored = f["dens"], f["points"]
        numbers, coords, pseudo = f["numbers"], f["coordinates"], f["pseudo_numbers"]
    r, wr = exp_radial()
    ang, wang = lebedev(110)
    pts, wts, owner = [], [], []
    for a, c in enumerate(coords):
        pts.append((r[:, None, None] * ang[None]).reshape(-1, 3) + c)
        wts.append(((wr * r * r)[:, None] * wang[None]).reshape(-1))
        owner.append(np.full(len(r) * len(ang), a))
    pts, wts, owner = np.concatenate(pts), np.concatenate(wts), np.concatenate(owner)
    # match the stored points to the rebuilt grid (the reference's reorder_rows)
    key = {tuple(np.round(p, 8)): i for i, p in enumerate(stored)}
    order = np.array([key[tuple(np.round(p, 8))] for p in pts])
    assert np.abs(stored[order] - pts).max() < 1e-6
    weights = wts * becke_partition_weights(pts, coords, owner)
    density = dens[order]
    # the unmodified reference's MBIS on this molecular grid (grid_type 3),
    # threshold 1e-8: the exact target for the oracle and the GPU path
    from oracle import refrun

    ref = refrun.run("mbis", coords, numbers, pseudo, pts, weights, density, threshold=1e-8)
    # and on the atom grids (grid_type 1, the reference's default and the
    # setting of its published test): radial grid and Lebedev-110 per atom
    natom = len(numbers)
    local = atom_grid_description(natom, r, wr, wang)
    ref1 = refrun.run("mbis", coords, numbers, pseudo, pts, weights, density, local=local,
                      threshold=1e-8)
    out = os.path.join(HERE, "water_sto3g_hf_molgrid.npz")
    np.savez_compressed(out, points=pts, weights=weights, density=density, numbers=numbers,
                        coordinates=coords, pseudo_numbers=pseudo,
                        ref_charges=np.asarray(ref["charges"]), ref_propars=np.asarray(ref["propars"]),
                        ref_niter=np.asarray(ref["niter"]), radial_points=r, radial_weights=wr,
                        ref1_charges=np.asarray(ref1["charges"]),
                        ref1_propars=np.asarray(ref1["propars"]), ref1_niter=np.asarray(ref1["niter"]))
    print(out, "integrated density", float(weights @ density), "reference charges",
          ref["charges"], "niter", ref["niter"], "grid_type 1:", ref1["charges"], ref1["niter"])


def atom_grid_description(natom, r, wr, wang):
    """Atom-grid layout of this fixture (atom after atom, radial shell after
    radial shell, the Lebedev points of a shell together), in the form of the
    oracle's ``local`` argument."""
    nr, nq = len(r), len(wang)
    return dict(indices=np.arange(natom + 1) * nr * nq, rpoints=[r] * natom,
                rweights=[wr] * natom, shell=np.tile(np.repeat(np.arange(nr), nq), natom),
                wsph=np.tile(wang / (4.0 * np.pi), nr * natom), nang=nq)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
