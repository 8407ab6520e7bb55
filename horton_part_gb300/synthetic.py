"""Seeded synthetic molecules, densities and basis sets for the benchmark
workloads and the parity tests.

No public dataset is involved: every workload is generated here from a seed.

* :func:`water` - H2O, O at the origin, H at (+-0.757, 0.586, 0) Angstrom, a
  Slater-shell density times (1 + 0.05 tanh(smooth seeded Gaussian bumps)),
  renormalised to 10 electrons, on a Becke grid (75 radial x Lebedev-110 per
  atom = 24,750 points by default).
* :func:`chain_molecule` - a seeded self-avoiding chain (bonded distances
  U(1.0, 1.6) Angstrom, non-bonded separations >= 2.0 Angstrom) with a
  synthetic Slater-shell density (+-10 % exponent jitter).
* :func:`geometric_gaussian_basis` - s-type Gaussian shells with exponents in
  geometric progression, as a :class:`~horton_part_gb300.basis.ExpBasisFuncHelper`.
"""

from __future__ import annotations

import numpy as np

from .basis import ExpBasisFuncHelper
from .molgrid import MolecularGrid, becke_molecular_grid, lebedev, radial_becke_gauss_chebyshev

__all__ = [
    "ANGSTROM",
    "Molecule",
    "water",
    "chain_molecule",
    "geometric_gaussian_basis",
    "slater_density",
    "batch_molecules",
    "peptide_molecule",
    "contracted_basis",
    "density_matrix",
]

ANGSTROM = 1.889726133921252

# Slater shells (exponent in 1/bohr, population) of the synthetic densities.
_DENSITY_SHELLS = {
    1: [(2.0, 1.0)],
    6: [(11.0, 2.0), (2.6, 2.0), (1.5, 2.0)],
    7: [(13.0, 2.0), (2.2, 5.0)],
    8: [(15.0, 2.0), (2.2, 6.0)],
    16: [(31.0, 2.0), (9.0, 8.0), (1.8, 6.0)],
}


class Molecule:
    """A synthetic partitioning input: geometry, grid and density."""

    def __init__(self, coordinates, numbers, grid, density, name=""):
        self.coordinates = np.ascontiguousarray(coordinates, dtype=np.float64)
        self.numbers = np.ascontiguousarray(numbers, dtype=np.int64)
        self.pseudo_numbers = self.numbers.astype(np.float64)
        self.grid = grid
        self.density = np.ascontiguousarray(density, dtype=np.float64)
        self.name = name

    @property
    def natom(self):
        return self.numbers.size

    @property
    def npoint(self):
        return self.grid.size


def slater_density(points, coordinates, numbers, seed, jitter=0.0, noise=0.05):
    """rho = sum_a sum_k c_ak a_ak^3/(8 pi) exp(-a_ak r_a) * (1 + noise*tanh(bumps)).

    ``bumps`` is a sum of seeded Gaussians centred near the atoms. Exponents
    get a multiplicative U(1 - jitter, 1 + jitter) perturbation per shell.
    """
    rng = np.random.default_rng(seed)
    rho = np.zeros(points.shape[0])
    for a, z in enumerate(numbers):
        r = np.linalg.norm(points - coordinates[a], axis=1)
        for alpha, pop in _DENSITY_SHELLS[int(z)]:
            if jitter:
                alpha = alpha * rng.uniform(1.0 - jitter, 1.0 + jitter)
            rho += pop * alpha**3 / (8.0 * np.pi) * np.exp(-alpha * r)
    nbump = 2 * len(numbers) + 2
    centres = coordinates[rng.integers(0, len(numbers), nbump)] + rng.normal(0.0, 1.0, (nbump, 3))
    amps = rng.normal(0.0, 1.0, nbump)
    bumps = np.zeros(points.shape[0])
    for c, amp in zip(centres, amps):
        bumps += amp * np.exp(-0.5 * np.sum((points - c) ** 2, axis=1))
    return rho * (1.0 + noise * np.tanh(bumps))


def water(nrad=75, nang=110, seed=1234):
    """H2O with the Slater-shell density (O: (15.0, 2), (2.2, 6); H: (2.0, 1))."""
    coords = np.array([[0.0, 0.0, 0.0], [0.757, 0.586, 0.0], [-0.757, 0.586, 0.0]]) * ANGSTROM
    numbers = np.array([8, 1, 1], dtype=np.int64)
    grid = becke_molecular_grid(coords, nrad, nang)
    rho = slater_density(grid.points, coords, numbers, seed)
    rho *= 10.0 / grid.integrate(rho)
    return Molecule(coords, numbers, grid, rho, name=f"H2O {nrad}x{nang}")


def _chain_geometry(numbers, rng, dmin=1.0, dmax=1.6, nonbonded=2.0, max_tries=20000):
    coords = [np.zeros(3)]
    tries = 0
    while len(coords) < len(numbers):
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place a self-avoiding chain")
        d = rng.uniform(dmin, dmax)
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        cand = coords[-1] + d * v
        prev = np.array(coords[:-1])
        if prev.size and np.min(np.linalg.norm(prev - cand, axis=1)) < nonbonded:
            continue
        coords.append(cand)
    return np.array(coords) * ANGSTROM


def chain_molecule(counts, nrad, nang, seed=7):
    """Seeded self-avoiding chain for the element ``counts`` (e.g.
    ``{6: 6, 1: 10, 7: 2, 8: 2}``), atoms in a seeded random order."""
    rng = np.random.default_rng(seed)
    numbers = np.concatenate([np.full(n, z, dtype=np.int64) for z, n in sorted(counts.items())])
    rng.shuffle(numbers)
    coords = _chain_geometry(numbers, rng)
    grid = becke_molecular_grid(coords, nrad, nang)
    rho = slater_density(grid.points, coords, numbers, seed + 1, jitter=0.1)
    rho *= float(numbers.sum()) / grid.integrate(rho)
    return Molecule(coords, numbers, grid, rho, name=f"chain A={len(numbers)} {nrad}x{nang}")


def _becke_weights_torch(points, coords, owner, torch, chunk_bytes=1 << 29):
    """Becke (k = 3) partition weights on the GPU (FP64), chunked over points."""
    natom = coords.shape[0]
    out = torch.empty(points.shape[0], dtype=torch.float64, device=points.device)
    if natom == 1:
        out.fill_(1.0)
        return out
    rab = torch.cdist(coords, coords)
    rab.fill_diagonal_(1.0)
    inv = 1.0 / rab
    eye = torch.eye(natom, dtype=torch.bool, device=points.device)
    chunk = max(1024, chunk_bytes // (8 * natom * natom))
    for s in range(0, points.shape[0], chunk):
        d = torch.cdist(points[s:s + chunk], coords)  # (n, A)
        mu = (d[:, :, None] - d[:, None, :]) * inv[None]
        f = mu
        for _ in range(3):
            f = 1.5 * f - 0.5 * f * f * f
        sv = 0.5 * (1.0 - f)
        sv[:, eye] = 1.0
        cell = torch.prod(sv, dim=2)
        own = owner[s:s + chunk]
        out[s:s + chunk] = cell.gather(1, own[:, None])[:, 0] / cell.sum(dim=1)
    return out


def batch_molecules(nmol=512, amin=3, amax=60, nrad=75, nang=194, seed=3, ratio=None,
                    device="cuda", natoms=None):
    """Seeded batch of chain molecules for the batched-MBIS workload.

    Atom counts uniform in [amin, amax] (or the given ``natoms`` list, one
    molecule per entry); elements drawn H:C:N:O = 10:6:1:1; geometry, Becke
    grid (nrad radial x Lebedev-nang per atom) and Slater-shell density as
    :func:`chain_molecule`, computed on the GPU with torch (input preparation
    only). Returns a list of :class:`Molecule` with host arrays.
    """
    import torch

    ratio = ratio or {1: 10, 6: 6, 7: 1, 8: 1}
    rng = np.random.default_rng(seed)
    zs = np.array(sorted(ratio))
    pz = np.array([ratio[z] for z in zs], dtype=float)
    pz /= pz.sum()
    r, wr = radial_becke_gauss_chebyshev(nrad)
    ang, wang = lebedev(nang)
    shell_pts = torch.as_tensor((r[:, None, None] * ang[None]).reshape(-1, 3), device=device)
    shell_w = torch.as_tensor(((wr * r * r)[:, None] * wang[None]).reshape(-1), device=device)
    npa = shell_pts.shape[0]
    mols = []
    if natoms is not None:
        nmol = len(natoms)
    for m in range(nmol):
        natom = int(natoms[m]) if natoms is not None else int(rng.integers(amin, amax + 1))
        numbers = rng.choice(zs, size=natom, p=pz).astype(np.int64)
        coords = _chain_geometry(numbers, rng)
        c = torch.as_tensor(coords, device=device)
        pts = (shell_pts[None] + c[:, None, :]).reshape(-1, 3)
        owner = torch.arange(natom, device=device).repeat_interleave(npa)
        w = shell_w.repeat(natom) * _becke_weights_torch(pts, c, owner, torch)
        rho = torch.zeros(pts.shape[0], dtype=torch.float64, device=device)
        jit = rng.uniform(0.9, 1.1, size=(natom, 3))
        for a, z in enumerate(numbers):
            ra = torch.linalg.norm(pts - c[a], dim=1)
            for k, (alpha, pop) in enumerate(_DENSITY_SHELLS[int(z)]):
                al = alpha * jit[a, k]
                rho += pop * al**3 / (8.0 * np.pi) * torch.exp(-al * ra)
        nb = 2 * natom + 2
        centres = torch.as_tensor(coords[rng.integers(0, natom, nb)] + rng.normal(0, 1, (nb, 3)),
                                  device=device)
        amps = torch.as_tensor(rng.normal(0, 1, nb), device=device)
        bumps = torch.zeros_like(rho)
        for cc, am in zip(centres, amps):
            bumps += am * torch.exp(-0.5 * ((pts - cc) ** 2).sum(dim=1))
        rho = rho * (1.0 + 0.05 * torch.tanh(bumps))
        rho *= float(numbers.sum()) / float(torch.dot(w, rho))
        indices = np.arange(natom + 1, dtype=np.int64) * npa
        grid = MolecularGrid(pts.cpu().numpy(), w.cpu().numpy(), indices=indices)
        mols.append(Molecule(coords, numbers, grid, rho.cpu().numpy(), name=f"batch{m} A={natom}"))
    return mols


def _becke_weights_nearest(points, coords, owner, torch, k=16, chunk=1 << 17):
    """Becke (k = 3) weights over each point's ``k`` nearest atoms and its
    owner (GPU, FP64): P_b = prod_c s(mu_bc) over that set, weight =
    P_owner / sum_b P_b. It is a partition of unity over that set, so the
    molecular grid still integrates exactly what the atoms' radial x angular
    grids integrate; it departs from the full Becke partition mostly far from
    the molecule (a 30-atom chain on 75 x Lebedev-194 grids integrates the
    same Slater density to 1e-7 relative with both). The grid is an input of
    the partitioning: the oracle and the GPU path read the same weights."""
    natom = coords.shape[0]
    if natom <= k + 1:
        return _becke_weights_torch(points, coords, owner, torch)
    out = torch.empty(points.shape[0], dtype=torch.float64, device=points.device)
    rab_all = torch.cdist(coords, coords)
    for s in range(0, points.shape[0], chunk):
        p = points[s:s + chunk]
        own = owner[s:s + chunk]
        d = torch.cdist(p, coords)  # (n, A)
        near = torch.topk(d, k, dim=1, largest=False).indices  # (n, k)
        has_own = (near == own[:, None]).any(dim=1)
        near[:, -1] = torch.where(has_own, near[:, -1], own)
        dn = torch.gather(d, 1, near)  # (n, k)
        rab = rab_all[near[:, :, None], near[:, None, :]]  # (n, k, k)
        eye = torch.eye(k, dtype=torch.bool, device=p.device)
        rab = torch.where(eye[None], torch.ones_like(rab), rab)
        mu = (dn[:, :, None] - dn[:, None, :]) / rab
        f = mu
        for _ in range(3):
            f = 1.5 * f - 0.5 * f * f * f
        sv = 0.5 * (1.0 - f)
        sv = torch.where(eye[None], torch.ones_like(sv), sv)
        cell = torch.prod(sv, dim=2)  # (n, k)
        mine = (near == own[:, None]).to(torch.float64)
        out[s:s + chunk] = (cell * mine).sum(dim=1) / cell.sum(dim=1)
    return out


def peptide_molecule(counts=None, nrad=150, nang=590, seed=4, device="cuda"):
    """Large synthetic molecule: a seeded self-avoiding chain of
    ``counts`` (default H:C:N:O:S = 100:64:18:16:2, 200 atoms), the
    Slater-shell density of :func:`chain_molecule` (+-10 % exponent jitter,
    seeded bumps) on a Becke grid of ``nrad`` radial x Lebedev-``nang``
    points per atom (default 150 x 590: 17.7M points), built on the GPU with
    torch (input preparation only; Becke weights over each point's 16 nearest
    atoms). Returns a :class:`Molecule` with host arrays."""
    import torch

    counts = counts or {1: 100, 6: 64, 7: 18, 8: 16, 16: 2}
    rng = np.random.default_rng(seed)
    numbers = np.concatenate([np.full(n, z, dtype=np.int64) for z, n in sorted(counts.items())])
    rng.shuffle(numbers)
    coords = _chain_geometry(numbers, rng)
    natom = len(numbers)
    r, wr = radial_becke_gauss_chebyshev(nrad)
    ang, wang = lebedev(nang)
    shell_pts = torch.as_tensor((r[:, None, None] * ang[None]).reshape(-1, 3), device=device)
    shell_w = torch.as_tensor(((wr * r * r)[:, None] * wang[None]).reshape(-1), device=device)
    npa = shell_pts.shape[0]
    c = torch.as_tensor(coords, device=device)
    pts = (shell_pts[None] + c[:, None, :]).reshape(-1, 3)
    owner = torch.arange(natom, device=device).repeat_interleave(npa)
    w = shell_w.repeat(natom) * _becke_weights_nearest(pts, c, owner, torch)
    # density: per atom its jittered Slater shells, per point chunk
    shells = [(a, alpha * rng.uniform(0.9, 1.1), pop) for a, z in enumerate(numbers)
              for alpha, pop in _DENSITY_SHELLS[int(z)]]
    sa = torch.as_tensor([x[0] for x in shells], device=device)
    sal = torch.as_tensor([x[1] for x in shells], dtype=torch.float64, device=device)
    spre = torch.as_tensor([x[2] * x[1] ** 3 / (8.0 * np.pi) for x in shells], dtype=torch.float64,
                           device=device)
    nb = 2 * natom + 2
    centres = torch.as_tensor(coords[rng.integers(0, natom, nb)] + rng.normal(0, 1, (nb, 3)),
                              device=device)
    amps = torch.as_tensor(rng.normal(0, 1, nb), device=device)
    rho = torch.empty(pts.shape[0], dtype=torch.float64, device=device)
    chunk = 1 << 16
    for s in range(0, pts.shape[0], chunk):
        p = pts[s:s + chunk]
        d = torch.cdist(p, c)[:, sa]  # (n, shells)
        dens = (spre[None] * torch.exp(-sal[None] * d)).sum(dim=1)
        bumps = (amps[None] * torch.exp(-0.5 * torch.cdist(p, centres) ** 2)).sum(dim=1)
        rho[s:s + chunk] = dens * (1.0 + 0.05 * torch.tanh(bumps))
    rho *= float(numbers.sum()) / float(torch.dot(w, rho))
    indices = np.arange(natom + 1, dtype=np.int64) * npa
    grid = MolecularGrid(pts.cpu().numpy(), w.cpu().numpy(), indices=indices)
    return Molecule(coords, numbers, grid, rho.cpu().numpy(),
                    name=f"peptide A={natom} {nrad}x{nang}")


def geometric_gaussian_basis(nshell_per_element, amin=0.05, amax=300.0):
    """s-Gaussian (order 2) shells with exponents geometric in [amin, amax],
    uniform initial populations, for the given ``{Z: nshell}``."""
    orders, exps, inits = {}, {}, {}
    for z, k in nshell_per_element.items():
        orders[z] = np.full(k, 2.0)
        exps[z] = np.geomspace(amax, amin, k)
        inits[z] = np.full(k, 1.0 / k)
    return ExpBasisFuncHelper(orders, exps, inits)


def contracted_basis(numbers, coordinates, seed=5):
    """Contracted Gaussian shells of a split-valence-plus-polarisation shape on
    every atom (a stand-in for a published basis set, which this package does
    not carry): H s(3) s(1) p(1) (5 functions); heavier atoms s(6) s(3) s(1)
    p(3) p(1) and a pure d(1) (14 functions). Exponents follow an
    even-tempered ladder scaled by the nuclear charge, contraction
    coefficients are positive and seeded. Returns a list of
    :class:`horton_part_gb300.fchk.Shell`."""
    from .fchk import Shell

    rng = np.random.default_rng(seed)
    out = []
    for a, (z, c) in enumerate(zip(np.asarray(numbers), np.asarray(coordinates, dtype=np.float64))):
        scale = float(z) ** 1.5 if z > 1 else 1.0
        if z == 1:
            spec = [(0, False, 3, 20.0), (0, False, 1, 0.17), (1, False, 1, 0.8)]
        else:
            spec = [(0, False, 6, 700.0 * scale / 20.0), (0, False, 3, 5.0 * scale / 20.0),
                    (0, False, 1, 0.3), (1, False, 3, 4.0 * scale / 20.0), (1, False, 1, 0.25),
                    (2, True, 1, 0.8)]
        for l, pure, n, top in spec:
            exps = top / 3.2 ** np.arange(n)
            coefs = rng.uniform(0.2, 1.0, n)
            out.append(Shell(c, l, pure, exps, coefs, a))
    return out


def density_matrix(nbasis, nocc, seed=6):
    """Closed-shell one-particle density 2 C C^T of ``nocc`` seeded orthonormal
    orbitals (a stand-in for a converged SCF density)."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.normal(size=(nbasis, nocc)))
    return 2.0 * q @ q.T
