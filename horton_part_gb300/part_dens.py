"""``part-dens``: partition molecular densities stored in files, as horton-part's
``part-dens`` program (``scripts/partition_density.py:172-348``,
``scripts/program.py:79-208``), on the GPU path.

    python -m horton_part_gb300.part_dens config.yaml [--skip_exist_files]

The configuration names the input density files (``inputs``), the result
files (``outputs``, default ``output_<i>.npz``), optional ``log_files`` and
the scheme settings (``type``, ``threshold``, ``maxiter``, ``solver``,
``grid_type`` ...); missing keys take the reference's defaults
(``data/part-dens.yaml``). An input file is the ``.npz`` written by the
reference's density generator: ``atcoords``, ``atnums``, ``atcorenums``,
``points``, ``weights``, ``aim_weights``, ``density``, ``atom_idxs`` and per
atom ``atom<i>/points``, ``atom<i>/weights``, ``atom<i>/shell_idxs``,
``atom<i>/rgrid/points``, ``atom<i>/rgrid/weights``. The molecular grid is
rebuilt from those arrays (no qc-grid). The result file holds the keys the
reference writes: the settings echo (``natom``, ``atnums``, ``atcorenums``,
``type``, ``lmax``, ``maxiter``, ``threshold``, ``inner_threshold``,
``solver``) and the results (``charges``, ``time``,
``time_update_at_weights``, ``time_update_propars``, ``niter``,
``history_charges``, ``history_propars``, ``history_entropies``,
``history_changes``).

pyyaml is not a dependency: :func:`read_settings` reads the flat YAML subset
such configurations use (``key: value`` lines, flow and block lists, quoted
strings, numbers, ``null``/``true``/``false``) and JSON.
"""

from __future__ import annotations

import argparse
import json
import logging
import os
import sys
import time

import numpy as np

from .molgrid import MolecularGrid, RadialGrid
from .utils import wpart_schemes

__all__ = ["DEFAULTS", "CLASS_ARGS", "read_settings", "molgrid_from_density", "run_one", "main"]

# The reference's defaults of the part-dens program (data/part-dens.yaml).
DEFAULTS = {
    "type": "lisa", "basis_func": "gauss", "func_file": None, "maxiter": 1000,
    "threshold": 1.0e-6, "inner_threshold": 1.0e-8, "lmax": 3, "log_level": "INFO",
    "solver": "sc", "exp_n_dict": None, "nshell_dict": None, "part_job_type": "do_partitioning",
    "grid_type": 1,
}

_COMMON = ["maxiter", "threshold", "inner_threshold", "lmax", "grid_type", "density_cutoff",
           "population_cutoff", "negative_cutoff"]
# Constructor arguments the program passes per scheme (data/keywords.yaml).
CLASS_ARGS = {
    "mbis": _COMMON,
    "gisa": _COMMON + ["solver", "solver_options"],
    "lisa": _COMMON + ["solver", "solver_options", "basis_func"],
    "glisa": [k for k in _COMMON if k != "inner_threshold"] + ["solver", "solver_options",
                                                               "basis_func"],
    "nlis": _COMMON + ["exp_n_dict", "nshell_dict"],
    "gmbis": _COMMON + ["exp_n_dict"],
}
IO_KEYS = ("inputs", "outputs", "log_files", "log_level", "part_job_type", "func_file")


# ---------------------------------------------------------------------------
# settings
# ---------------------------------------------------------------------------

def _scalar(text):
    t = text.strip()
    if not t:
        return None
    if t[0] in "\"'" and t[-1] == t[0]:
        return t[1:-1]
    low = t.lower()
    if low in ("null", "none", "~"):
        return None
    if low in ("true", "yes"):
        return True
    if low in ("false", "no"):
        return False
    if t[0] == "[" and t[-1] == "]":
        inner = t[1:-1].strip()
        return [_scalar(x) for x in inner.split(",")] if inner else []
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        return t


def read_settings(path):
    """Settings of a configuration file: JSON, or the flat YAML subset."""
    with open(path) as f:
        text = f.read()
    if text.lstrip().startswith("{"):
        return json.loads(text)
    out, key = {}, None
    for raw in text.splitlines():
        line = raw.split(" #")[0].rstrip() if not raw.lstrip().startswith("#") else ""
        if not line.strip():
            continue
        stripped = line.strip()
        if stripped.startswith("- ") or stripped == "-":
            if key is None:
                raise ValueError(f"{path}: list item without a key: {raw!r}")
            if not isinstance(out.get(key), list):
                out[key] = []
            out[key].append(_scalar(stripped[1:]))
            continue
        if ":" not in stripped or line[0] in " \t":
            raise ValueError(f"{path}: unsupported line (flat 'key: value' expected): {raw!r}")
        key, value = stripped.split(":", 1)
        key = key.strip()
        out[key] = _scalar(value)
    return out


def _exp_n_dict(table):
    """{Z: [n_0, n_1, ...]} -> {(Z, shell): n} (prepare_exp_n_dict)."""
    return {(int(z), i): float(v) for z, row in (table or {}).items() for i, v in enumerate(row)}


# ---------------------------------------------------------------------------
# molecular grid from a density file
# ---------------------------------------------------------------------------

class LoadedAtomGrid:
    """One atom's grid from a density file: radial nodes and weights, the
    point range of each radial shell (``indices``) and the point weights
    w_r r^2 w_angular, as qc-grid's ``AtomGrid``."""

    def __init__(self, rpoints, rweights, shell_idxs, weights):
        self.rgrid = RadialGrid(rpoints, rweights)
        self.indices = np.asarray(shell_idxs, dtype=np.int64)
        self.weights = np.asarray(weights, dtype=np.float64)
        r = self.rgrid.points
        shell = np.repeat(np.arange(r.size), np.diff(self.indices))
        self._shell = shell
        self._wsph = self.weights / (4.0 * np.pi * r[shell] ** 2 * self.rgrid.weights[shell])

    @property
    def size(self):
        return int(self.indices[-1])

    def spherical_average(self, values):
        from scipy.interpolate import CubicSpline

        avg = np.bincount(self._shell, weights=self._wsph * values, minlength=self.rgrid.size)
        return CubicSpline(self.rgrid.points, avg)


def molgrid_from_density(data):
    """The molecular grid of a density file (points and weights as stored,
    atom blocks from ``atom_idxs``, per-atom grids from ``atom<i>/...``)."""
    natom = len(data["atnums"])
    atgrids = [LoadedAtomGrid(data[f"atom{a}/rgrid/points"], data[f"atom{a}/rgrid/weights"],
                              data[f"atom{a}/shell_idxs"], data[f"atom{a}/weights"])
               for a in range(natom)]
    return MolecularGrid(data["points"], data["weights"], indices=data["atom_idxs"],
                         atgrids=atgrids)


# ---------------------------------------------------------------------------
# program
# ---------------------------------------------------------------------------

def _logger(settings, fn_log):
    lg = logging.getLogger("part-dens")
    lg.setLevel(getattr(logging, str(settings.get("log_level", "INFO")).upper(), logging.INFO))
    for h in list(lg.handlers):
        lg.removeHandler(h)
    h = logging.FileHandler(fn_log) if fn_log else logging.StreamHandler(sys.stdout)
    h.setFormatter(logging.Formatter("%(message)s"))
    lg.addHandler(h)
    lg.propagate = False
    return lg


def run_one(settings, fn_in, fn_out, fn_log=None, context=None):
    """Partition one density file and write its result file; returns 0 on
    success, 1 when the partitioning raised RuntimeError (logged)."""
    lg = _logger(settings, fn_log)
    kind = settings["type"]
    if kind not in CLASS_ARGS:
        raise NotImplementedError(f"part-dens type {kind!r} is not on the GPU path "
                                  f"(available: {sorted(CLASS_ARGS)})")
    with np.load(fn_in) as f:
        data = {k: f[k] for k in f.files}
    grid = molgrid_from_density(data)
    kwargs = dict(coordinates=data["atcoords"], numbers=np.asarray(data["atnums"], dtype=np.int64),
                  pseudo_numbers=np.asarray(data["atcorenums"], dtype=np.float64), grid=grid,
                  moldens=data["density"], logger=lg)
    for k in CLASS_ARGS[kind]:
        if k in settings and settings[k] is not None:
            kwargs[k] = settings[k]
    if "basis_func" in CLASS_ARGS[kind]:
        kwargs["basis_func"] = settings.get("func_file") or settings.get("basis_func")
    if "exp_n_dict" in CLASS_ARGS[kind]:
        kwargs["exp_n_dict"] = _exp_n_dict(settings.get("exp_n_dict"))
    if context is not None:
        kwargs["context"] = context
    part = wpart_schemes(kind)(**kwargs)
    lg.info(f"part-dens: {kind} on {fn_in} ({len(data['atnums'])} atoms, {grid.size} points)")
    try:
        getattr(part, settings.get("part_job_type", "do_partitioning"))()
    except RuntimeError as err:
        lg.info(str(err))
        return 1
    for z, q in zip(data["atnums"], part.cache["charges"]):
        lg.info(f"{int(z):>4} : {q:>15.8f}")
    out = {
        "natom": len(data["atnums"]), "atnums": data["atnums"], "atcorenums": data["atcorenums"],
        "type": kind, "lmax": settings["lmax"], "maxiter": settings["maxiter"],
        "threshold": settings["threshold"],
        "inner_threshold": settings["inner_threshold"] if kind != "glisa" else np.nan,
        "solver": settings["solver"],
        "charges": part.cache["charges"], "time": part.time_usage["do_partitioning"],
        "time_update_at_weights": part.cache["time_update_at_weights"],
        "time_update_propars": part.cache["time_update_propars"], "niter": part.cache["niter"],
        "history_charges": part.cache["history_charges"],
        "history_propars": part.cache["history_propars"],
        "history_entropies": part.cache["history_entropies"],
        "history_changes": part.cache["history_changes"],
    }
    d = os.path.dirname(os.path.abspath(fn_out))
    os.makedirs(d, exist_ok=True)
    np.savez_compressed(fn_out, **out)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(prog="part-dens",
                                 description="Molecular density partitioning on the GPU path.")
    ap.add_argument("config_file")
    ap.add_argument("--skip_exist_files", action="store_true",
                    help="skip inputs whose output (and log) file exists")
    args = ap.parse_args(argv)
    settings = read_settings(args.config_file)
    for k, v in DEFAULTS.items():
        settings.setdefault(k, v)
    inputs = settings.get("inputs")
    if not isinstance(inputs, list):
        raise RuntimeError("the settings need a list of 'inputs'")
    outputs = settings.setdefault("outputs", [f"output_{i + 1}.npz" for i in range(len(inputs))])
    logs = settings.setdefault("log_files", [None] * len(inputs))
    if not len(inputs) == len(outputs) == len(logs):
        raise RuntimeError("The settings for part-dens is not fully correct.")
    rc = 0
    for fn_in, fn_out, fn_log in zip(inputs, outputs, logs):
        if args.skip_exist_files and os.path.exists(fn_out) and (fn_log is None or os.path.exists(fn_log)):
            print(f"Skip the calculations with input: {fn_in}")
            continue
        t0 = time.time()
        rc |= run_one(settings, fn_in, fn_out, fn_log)
        print(f"{fn_in} -> {fn_out} ({time.time() - t0:.2f} s)")
    return rc


if __name__ == "__main__":
    sys.exit(main())
