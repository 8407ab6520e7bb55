"""Gaussian formatted checkpoint (``.fchk``) files: the wavefunction data the
density generator needs (``scripts/generate_density.py:119-204`` of
horton-part, which reads them through iodata's ``load_one``).

Read: atomic numbers, nuclear (pseudo) charges, coordinates (bohr), the
contracted Gaussian shells (type, primitives, exponents, contraction
coefficients, the P coefficients of SP shells, centres) and the one-particle
density matrices: the post-SCF total density when the file has one (``Total
CC Density``, ``Total MP2 Density``, ...), else ``Total SCF Density`` (as
``_compute_stuff`` picks ``one_rdms["post_scf"]`` before ``"scf"``), the
matching spin density, and the MO coefficients with their occupations as a
fallback when no density matrix is stored.

Shell types follow the fchk convention: 0 s, 1 p, -1 sp, l >= 2 Cartesian,
-l pure (spherical) functions of angular momentum l.
"""

from __future__ import annotations

import numpy as np

__all__ = ["Shell", "FchkData", "load_fchk", "basis_size"]


class Shell:
    """One contracted shell: centre (3,), angular momentum ``l``, ``pure``
    (spherical) or Cartesian, exponents (nprim,) and the contraction
    coefficients of normalised primitives (nprim,). An SP shell of the file
    becomes two shells (s, then p) on the same primitives."""

    __slots__ = ("center", "l", "pure", "exponents", "coeffs", "atom")

    def __init__(self, center, l, pure, exponents, coeffs, atom):
        self.center = np.asarray(center, dtype=np.float64)
        self.l = int(l)
        self.pure = bool(pure) and self.l >= 2
        self.exponents = np.asarray(exponents, dtype=np.float64)
        self.coeffs = np.asarray(coeffs, dtype=np.float64)
        self.atom = int(atom)

    @property
    def nfunc(self):
        return 2 * self.l + 1 if self.pure else (self.l + 1) * (self.l + 2) // 2


def basis_size(shells):
    return int(sum(s.nfunc for s in shells))


class FchkData:
    """Fields of a formatted checkpoint file used by the density generator."""

    def __init__(self, fields, title=""):
        self.fields = fields
        self.title = title
        self.atnums = np.asarray(fields["Atomic numbers"], dtype=np.int64)
        self.atcorenums = np.asarray(fields.get("Nuclear charges", self.atnums), dtype=np.float64)
        self.atcoords = np.asarray(fields["Current cartesian coordinates"], dtype=np.float64).reshape(-1, 3)
        self.shells = _shells(fields)
        self.nbasis = int(fields["Number of basis functions"])
        if basis_size(self.shells) != self.nbasis:
            raise ValueError(f"the shells give {basis_size(self.shells)} basis functions, the file "
                             f"declares {self.nbasis}")
        self.one_rdm, self.one_rdm_kind = self._density("Total")
        self.spin_rdm, _ = self._density("Spin")

    @property
    def natom(self):
        return len(self.atnums)

    def _density(self, prefix):
        keys = [k for k in self.fields if k.startswith(prefix + " ") and k.endswith(" Density")
                and not k.startswith(prefix + " SCF")]
        kind = "post_scf"
        if not keys:
            keys = [k for k in self.fields if k == prefix + " SCF Density"]
            kind = "scf"
        if keys:
            return _triangle(self.fields[keys[0]], self.nbasis), kind
        if prefix == "Total":
            return self._density_from_orbitals(), "mo"
        return None, None

    def _density_from_orbitals(self):
        """sum_i n_i C_i C_i^T from the MO coefficients (aufbau occupations of
        the alpha and beta electrons; restricted files use the alpha orbitals
        for both spins)."""
        f = self.fields
        if "Alpha MO coefficients" not in f:
            raise ValueError("The input file lacks wavefunction data with which the density can be "
                             "computed.")
        nb = self.nbasis
        ca = np.asarray(f["Alpha MO coefficients"]).reshape(-1, nb).T
        cb = np.asarray(f["Beta MO coefficients"]).reshape(-1, nb).T if "Beta MO coefficients" in f else ca
        na = int(f["Number of alpha electrons"])
        nbeta = int(f["Number of beta electrons"])
        return ca[:, :na] @ ca[:, :na].T + cb[:, :nbeta] @ cb[:, :nbeta].T


def _triangle(values, n):
    """Symmetric matrix from its lower triangle stored row by row."""
    values = np.asarray(values, dtype=np.float64)
    if values.size != n * (n + 1) // 2:
        raise ValueError(f"a triangle of {n} x {n} needs {n * (n + 1) // 2} values, got {values.size}")
    out = np.zeros((n, n))
    out[np.tril_indices(n)] = values
    return out + np.tril(out, -1).T


def _shells(f):
    types = np.asarray(f["Shell types"], dtype=np.int64)
    nprim = np.asarray(f["Number of primitives per shell"], dtype=np.int64)
    owner = np.asarray(f["Shell to atom map"], dtype=np.int64) - 1
    exps = np.asarray(f["Primitive exponents"], dtype=np.float64)
    coeffs = np.asarray(f["Contraction coefficients"], dtype=np.float64)
    pcoeffs = f.get("P(S=P) Contraction coefficients")
    centers = np.asarray(f["Coordinates of each shell"], dtype=np.float64).reshape(-1, 3)
    out, k = [], 0
    for s, t in enumerate(types):
        sl = slice(k, k + int(nprim[s]))
        k += int(nprim[s])
        if t == -1:
            if pcoeffs is None:
                raise ValueError("SP shell without P(S=P) contraction coefficients")
            out.append(Shell(centers[s], 0, False, exps[sl], coeffs[sl], owner[s]))
            out.append(Shell(centers[s], 1, False, exps[sl], np.asarray(pcoeffs)[sl], owner[s]))
        else:
            out.append(Shell(centers[s], abs(int(t)), t < -1, exps[sl], coeffs[sl], owner[s]))
    return out


def load_fchk(path):
    """Parse a formatted checkpoint file into :class:`FchkData`."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    if len(lines) < 2:
        raise ValueError(f"{path}: not a formatted checkpoint file")
    fields = {}
    i = 2
    while i < len(lines):
        line = lines[i]
        name, kind, rest = line[:43].strip(), line[43:45].strip(), line[45:].strip()
        i += 1
        if not name:
            continue
        if rest.startswith("N="):
            n = int(rest[2:])
            if kind == "C":  # n 12-character chunks, five per line
                nlines = (n + 4) // 5
                fields[name] = "".join(lines[i:i + nlines])
                i += nlines
                continue
            vals = []
            while len(vals) < n and i < len(lines):
                vals.extend(lines[i].split())
                i += 1
            if kind == "I":
                fields[name] = np.array([int(v) for v in vals], dtype=np.int64)
            elif kind == "L":
                fields[name] = np.array([v == "T" for v in vals])
            else:
                fields[name] = np.array([float(v) for v in vals], dtype=np.float64)
        else:
            if kind == "I":
                fields[name] = int(rest)
            elif kind == "R":
                fields[name] = float(rest)
            else:
                fields[name] = rest
    return FchkData(fields, title=lines[0].strip())
