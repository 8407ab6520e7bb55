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
    """Check a geometry and return ``[natom]`` followed by the needed arrays.

    Same contract as horton-part's ``utils.typecheck_geo``: the atom count
    comes from the first array given; ``coordinates`` must be float64 with
    shape (natom, 3), ``numbers`` int64 with shape (natom,); ``pseudo_numbers``
    (natom,) is converted to float64 and defaults to ``numbers``. An array
    whose ``need_*`` flag is False may be None and is left out of the result.
    Violations raise ``TypeError``.
    """
    given = [a for a in (coordinates, numbers, pseudo_numbers) if a is not None]
    if not given:
        raise TypeError("typecheck_geo needs coordinates, numbers or pseudo_numbers")
    natom = len(given[0])

    def check(label, array, needed, shape, dtype):
        if array is None:
            if needed:
                raise TypeError(f"{label} are required")
            return
        if array.shape != shape or array.dtype != dtype:
            raise TypeError(f"{label} must be a {np.dtype(dtype).name} array of shape {shape}, "
                            f"got {array.dtype} {array.shape}")

    check("coordinates", coordinates, need_coordinates, (natom, 3), np.float64)
    check("numbers", numbers, need_numbers, (natom,), np.int64)
    if pseudo_numbers is not None:
        if pseudo_numbers.shape != (natom,):
            raise TypeError(f"pseudo_numbers must have shape ({natom},), got {pseudo_numbers.shape}")
        pseudo_numbers = np.asarray(pseudo_numbers, dtype=np.float64)
    elif need_pseudo_numbers:
        if numbers is None:
            raise TypeError("pseudo_numbers default to numbers, and neither was given")
        pseudo_numbers = numbers.astype(np.float64)
    wanted = ((need_coordinates, coordinates), (need_numbers, numbers),
              (need_pseudo_numbers, pseudo_numbers))
    return [natom] + [array for needed, array in wanted if needed]
