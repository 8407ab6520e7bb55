"""Render the fields of a density fixture (tests/golden/density_*.npz) as a
formatted checkpoint file, so that the tests read it with the package's
fchk parser."""

import numpy as np


def render_fchk(fixture, path):
    """Write the fixture's fchk fields to ``path`` in the fchk layout (name in
    43 columns, type, value or N= count; integers six per line, reals four
    per line with 17 significant digits so that nothing is lost)."""
    lines = [str(fixture["title"]), "SP        RHF                                                         GEN"]
    for key in sorted(k for k in fixture if k.startswith("f:")):
        name = key[2:]
        value = np.asarray(fixture[key])
        kind = "I" if np.issubdtype(value.dtype, np.integer) else "R"
        head = f"{name:<43s}{kind}"
        if value.ndim == 0:
            lines.append(f"{head}   {int(value):>12d}" if kind == "I" else f"{head}   {float(value):25.17E}")
            continue
        vals = value.ravel()
        lines.append(f"{head}   N={len(vals):>12d}")
        per = 6 if kind == "I" else 4
        for s in range(0, len(vals), per):
            if kind == "I":
                lines.append("".join(f"{int(v):12d}" for v in vals[s:s + per]))
            else:
                lines.append("".join(f"{float(v):25.17E}" for v in vals[s:s + per]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def load_fixture(path):
    with np.load(path) as f:
        return {k: f[k] for k in f.files}
