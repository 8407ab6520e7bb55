"""Definitions of the golden parity cases (inputs and scheme options).

Each case regenerates its seeded synthetic input with
:mod:`horton_part_gb300.synthetic`; ``make_golden.py`` stores the reference's
results for it, and the parity tests compare the oracle and the GPU path
against those results.
"""

from horton_part_gb300 import synthetic

_CHAIN5 = {6: 1, 8: 1, 1: 3}

CASES = {
    # H2O, 75 radial x Lebedev-110 = 24,750 points, MBIS, threshold 1e-8, maxiter 500
    "mbis_h2o_75x110": dict(scheme="mbis", mol=("water", 75, 110),
                            kwargs=dict(threshold=1e-8, maxiter=500, inner_threshold=1e-8)),
    "mbis_chain5_40x50": dict(scheme="mbis", mol=("chain", _CHAIN5, 40, 50, 11),
                              kwargs=dict(threshold=1e-6, maxiter=500, inner_threshold=1e-8)),
    "gisa_h2o_50x110": dict(scheme="gisa", mol=("water", 50, 110),
                            kwargs=dict(threshold=1e-8, inner_threshold=1e-8, solver="quadprog")),
    "lisa_sc_h2o_50x110": dict(scheme="lisa", mol=("water", 50, 110),
                               kwargs=dict(threshold=1e-8, inner_threshold=1e-8, solver="sc")),
    "lisa_mnewton_h2o_50x110": dict(scheme="lisa", mol=("water", 50, 110),
                                    kwargs=dict(threshold=1e-8, inner_threshold=1e-8,
                                                solver="m-newton")),
    "glisa_newton_h2o_50x110": dict(scheme="glisa", mol=("water", 50, 110),
                                    kwargs=dict(threshold=1e-8, solver="newton")),
    "glisa_mnewton_chain5_40x50": dict(scheme="glisa", mol=("chain", _CHAIN5, 40, 50, 11),
                                       kwargs=dict(threshold=1e-8, solver="m-newton")),
    "glisa_sc_h2o_50x110": dict(scheme="glisa", mol=("water", 50, 110),
                                kwargs=dict(threshold=1e-8, solver="sc")),
}


def build_inputs(case):
    """Return (molecule, constructor kwargs) for a case."""
    kind = case["mol"][0]
    if kind == "water":
        mol = synthetic.water(nrad=case["mol"][1], nang=case["mol"][2])
    elif kind == "chain":
        _, counts, nrad, nang, seed = case["mol"]
        mol = synthetic.chain_molecule(counts, nrad, nang, seed=seed)
    else:
        raise ValueError(kind)
    return mol, dict(case["kwargs"])
