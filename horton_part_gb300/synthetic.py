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
from .molgrid import becke_molecular_grid

__all__ = [
    "ANGSTROM",
    "Molecule",
    "water",
    "chain_molecule",
    "geometric_gaussian_basis",
    "slater_density",
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


def geometric_gaussian_basis(nshell_per_element, amin=0.05, amax=300.0):
    """s-Gaussian (order 2) shells with exponents geometric in [amin, amax],
    uniform initial populations, for the given ``{Z: nshell}``."""
    orders, exps, inits = {}, {}, {}
    for z, k in nshell_per_element.items():
        orders[z] = np.full(k, 2.0)
        exps[z] = np.geomspace(amax, amin, k)
        inits[z] = np.full(k, 1.0 / k)
    return ExpBasisFuncHelper(orders, exps, inits)
