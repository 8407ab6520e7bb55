"""The GPU density kernel (k_density through hp_density_plan_*) against the
densities stored beside horton-part's fchk test files and against the FP64
oracle on d and f shells (Cartesian and pure), plus the device-pointer
path, the screening counters and the argument errors."""

import glob
import os

import numpy as np
import pytest

from fchk_fixture import load_fixture, render_fchk
from horton_part_gb300.density import DensityPlan, compute_density
from horton_part_gb300.fchk import Shell, load_fchk
from oracle import hp_density as H

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "density_*.npz")))


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[8:-4])
def test_gpu_density_matches_the_reference_data(path, tmp_path, gpu_context):
    fx = load_fixture(path)
    render_fchk(fx, tmp_path / "w.fchk")
    data = load_fchk(str(tmp_path / "w.fchk"))
    spin = "spin_dens" in fx
    out = compute_density(data, fx["points"], spin=spin, context=gpu_context)
    ref = fx["dens"]
    assert np.abs(out["density"] - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs((out["density"] - ref) / ref).max() < 1e-12
    if spin:
        assert np.abs(out["spin_density"] - fx["spin_dens"]).max() <= 1e-13 * np.abs(fx["spin_dens"]).max()


def _random_basis(pure, seed=3):
    """Two-centre basis with s, p, d and f shells and a random positive
    semi-definite density matrix."""
    rng = np.random.default_rng(seed)
    shells = []
    for atom, c in enumerate([np.zeros(3), np.array([0.3, -1.1, 1.7])]):
        for l in range(4):
            n = 1 + l % 3
            shells.append(Shell(c, l, pure, np.sort(rng.uniform(0.2, 8.0, n))[::-1],
                                rng.uniform(0.3, 1.0, n), atom))
    nb = sum(s.nfunc for s in shells)
    a = rng.normal(size=(nb, nb))
    return shells, a @ a.T / nb


@pytest.mark.parametrize("pure", [False, True], ids=["cartesian", "pure"])
def test_gpu_density_d_and_f_shells_match_the_oracle(pure, gpu_context):
    shells, D = _random_basis(pure)
    rng = np.random.default_rng(11)
    pts = rng.normal(scale=2.0, size=(3000, 3))
    plan = DensityPlan(shells, D, context=gpu_context)
    got = plan.evaluate(pts)[0]
    ref = H.density(D, shells, pts)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    plan.close()


def test_gpu_density_device_pointers_and_stats(gpu_context):
    import torch

    shells, D = _random_basis(True, seed=7)
    rng = np.random.default_rng(2)
    far = rng.normal(scale=1.0, size=(2000, 3)) + np.array([40.0, 0.0, 0.0])  # beyond every shell
    near = rng.normal(scale=1.5, size=(2048, 3))
    pts = np.concatenate([near, far])
    plan = DensityPlan(shells, np.array([D, 0.5 * D]), context=gpu_context)
    host = plan.evaluate(pts)
    dev_pts = torch.tensor(pts, device=f"cuda:{gpu_context.device}")
    dev_out = torch.empty((2, len(pts)), dtype=torch.float64, device=dev_pts.device)
    plan.evaluate_device(dev_pts, dev_out)
    gpu_context.synchronize()
    np.testing.assert_array_equal(dev_out.cpu().numpy(), host)
    np.testing.assert_allclose(host[1], 0.5 * host[0], rtol=1e-14, atol=0)
    assert np.all(host[0, len(near):] == 0.0)  # screened out entirely
    st = plan.stats()
    assert st["shell_tiles"] > 0 and st["basis_values"] > 0
    # the far tiles keep no shell: at most the near tiles' shells x 2 evaluations
    ntile_near = -(-len(near) // 64)
    assert st["shell_tiles"] <= 2 * len(shells) * (ntile_near + 1)
    assert plan.evaluate(np.zeros((0, 3))).shape == (2, 0)
    plan.close()


def test_gpu_density_argument_errors(gpu_context):
    shells, D = _random_basis(False)
    with pytest.raises(ValueError):
        DensityPlan(shells, D[:-1, :-1], context=gpu_context)
    with pytest.raises(NotImplementedError):
        DensityPlan([Shell(np.zeros(3), 4, False, [1.0], [1.0], 0)], np.eye(15), context=gpu_context)
