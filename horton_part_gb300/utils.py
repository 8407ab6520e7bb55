"""Constants, geometry type checks and the scheme registry.

Same names and semantics as horton-part's ``utils.py`` (constants
``utils.py:50-59`` from ``data/constants.yaml``; ``typecheck_geo``
``utils.py:107-186``; ``wpart_schemes`` ``utils.py:62-104``) for the schemes
this package implements on the GPU: ``mbis``, ``gisa``, ``lisa``, ``glisa``,
``nlis``, ``gmbis``.
"""

from __future__ import annotations

import numpy as np

__all__ = ["DENSITY_CUTOFF", "NEGATIVE_CUTOFF", "POPULATION_CUTOFF", "ANGSTROM",
           "typecheck_geo", "wpart_schemes"]

DENSITY_CUTOFF = 1.0e-15
NEGATIVE_CUTOFF = -1.0e-12
POPULATION_CUTOFF = 1.0e-4
ANGSTROM = 1.889726133921252


def wpart_schemes(scheme):
    """Return the partitioning class registered under ``scheme``."""
    if scheme == "mbis":
        from .mbis import MBISWPart

        return MBISWPart
    if scheme == "gisa":
        from .gisa import GaussianISAWPart

        return GaussianISAWPart
    if scheme == "lisa":
        from .alisa import LinearISAWPart

        return LinearISAWPart
    if scheme == "glisa":
        from .glisa import GlobalLinearISAWPart

        return GlobalLinearISAWPart
    if scheme == "nlis":
        from .nlis import NLISWPart

        return NLISWPart
    if scheme == "gmbis":
        from .nlis import GMBISWPart

        return GMBISWPart
    if scheme in ("h", "hi", "is", "b"):
        raise NotImplementedError(f"scheme {scheme!r} is not part of the GPU partitioning path")
    raise UnboundLocalError(f"unknown scheme {scheme!r}")


def typecheck_geo(coordinates=None, numbers=None, pseudo_numbers=None, need_coordinates=True,
                  need_numbers=True, need_pseudo_numbers=True):
    """Type-check a geometry; returns ``[natom] + checked arguments``."""
    if coordinates is not None:
        natom = len(coordinates)
    elif numbers is not None:
        natom = len(numbers)
    elif pseudo_numbers is not None:
        natom = len(pseudo_numbers)
    else:
        raise TypeError("At least one argument is required and should not be None")
    if coordinates is None:
        if need_coordinates:
            raise TypeError("Coordinates can not be None.")
    elif coordinates.shape != (natom, 3) or not issubclass(coordinates.dtype.type, float):
        raise TypeError("The argument centers must be a float array with shape (natom,3).")
    if numbers is None:
        if need_numbers:
            raise TypeError("Numbers can not be None.")
    elif numbers.shape != (natom,) or not issubclass(numbers.dtype.type, np.int64):
        raise TypeError("The argument numbers must be a vector with length natom.")
    if pseudo_numbers is None:
        if need_pseudo_numbers:
            pseudo_numbers = numbers.astype(float)
    else:
        if pseudo_numbers.shape != (natom,):
            raise TypeError("The argument pseudo_numbers must be a vector with length natom.")
        if not issubclass(pseudo_numbers.dtype.type, float):
            pseudo_numbers = pseudo_numbers.astype(float)
    result = [natom]
    if need_coordinates:
        result.append(coordinates)
    if need_numbers:
        result.append(numbers)
    if need_pseudo_numbers:
        result.append(pseudo_numbers)
    return result
