"""Electron density of a contracted-Gaussian wavefunction on grid points, on
the GPU: the density step of horton-part's ``part-gen`` program
(``scripts/generate_density.py:119-204``: ``evaluate_basis`` on the points,
then ``einsum("ab,bp,ap->p", one_rdm, basis, basis)`` at :186-188).

The one-particle density matrix is the file's post-SCF density when it has
one, else the SCF density, else ``C occ C^T`` from the orbitals (as
``_compute_stuff`` at :146-155); the spin density comes from the file's spin
density matrix. Kernel: ``k_density`` (``csrc/hp_density.cu``), FP64, with a
per-tile shell screening.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .gto import pure_matrix, shell_tables

__all__ = ["DensityPlan", "compute_density"]


class DensityPlan:
    """Basis and density matrices resident on the device (``hp_density_plan``)."""

    def __init__(self, shells, mats, context=None):
        self.ctx = context or _lib.default_context()
        mats = np.ascontiguousarray(np.asarray(mats, dtype=np.float64))
        if mats.ndim == 2:
            mats = mats[None]
        centers, info, exps, coefs, nbasis = shell_tables(shells)
        if mats.shape[1:] != (nbasis, nbasis):
            raise ValueError(f"density matrices of shape {mats.shape[1:]} for {nbasis} basis functions")
        self.nmat, self.nbasis = mats.shape[0], nbasis
        self._keep = [np.ascontiguousarray(centers), np.ascontiguousarray(info, dtype=np.int32),
                      np.ascontiguousarray(exps), np.ascontiguousarray(coefs), mats,
                      np.ascontiguousarray(pure_matrix(2)), np.ascontiguousarray(pure_matrix(3))]
        c, i, e, k, m, p2, p3 = self._keep
        desc = _lib.DensityDesc(
            nshell=len(shells), centers=_lib._ptr(c), shell_info=_lib._ptr(i, ctypes.c_int32),
            nprim=len(e), exponents=_lib._ptr(e), coeffs=_lib._ptr(k), nbasis=nbasis,
            nmat=self.nmat, mats=_lib._ptr(m), pure2=_lib._ptr(p2), pure3=_lib._ptr(p3))
        h = ctypes.c_void_p()
        _lib._check(_lib.lib().hp_density_plan_create(self.ctx.handle, ctypes.byref(desc),
                                                      ctypes.byref(h)))
        self._h = h

    def evaluate(self, points):
        """(nmat, N) densities at host points (N, 3); copies in and out."""
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        out = np.empty((self.nmat, len(pts)))
        _lib._check(_lib.lib().hp_density_plan_eval(self._h, len(pts), pts.ctypes.data,
                                                    out.ctypes.data, 0))
        return out

    def evaluate_device(self, points, out):
        """Densities at device points, written to a device array: ``points``
        (N, 3) and ``out`` (nmat, N) contiguous FP64 CUDA tensors of the
        plan's device (asynchronous on the context stream)."""
        n = int(points.shape[0])
        if out.numel() != self.nmat * n or not points.is_contiguous() or not out.is_contiguous():
            raise ValueError("contiguous (N, 3) points and (nmat, N) output expected")
        _lib._check(_lib.lib().hp_density_plan_eval(self._h, n, ctypes.c_void_p(points.data_ptr()),
                                                    ctypes.c_void_p(out.data_ptr()), 1))

    def stats(self):
        """Work since creation: shell-tile pairs kept by the screening, basis
        values evaluated, FMA per matrix in the contraction."""
        buf = (ctypes.c_uint64 * 3)()
        _lib._check(_lib.lib().hp_density_plan_stats(self._h, buf))
        return {"shell_tiles": int(buf[0]), "basis_values": int(buf[1]), "fma_per_matrix": int(buf[2])}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().hp_density_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def compute_density(data, points, spin=False, context=None):
    """{"density": (N,)[, "spin_density": (N,)]} of a wavefunction read by
    :func:`horton_part_gb300.fchk.load_fchk` at the points."""
    mats = [data.one_rdm]
    if spin:
        if data.spin_rdm is None:
            raise ValueError("the file has no spin density matrix")
        mats.append(data.spin_rdm)
    plan = DensityPlan(data.shells, np.array(mats), context=context)
    try:
        vals = plan.evaluate(points)
    finally:
        plan.close()
    out = {"density": vals[0]}
    if spin:
        out["spin_density"] = vals[1]
    return out
