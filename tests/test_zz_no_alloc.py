"""hp_mbis_inner_noalloc: the MBIS inner solver for one atom that allocates
nothing, for callers that cannot call cudaMalloc (code inside a host
application's own device-memory pool, plug-in hosts that forbid allocation
after start-up, loops where an allocation would synchronise the device).

It is checked against the existing entry points: a job created and run
through hp_job_create / hp_job_run with maxiter=1 performs exactly one
inner solve per atom on rho_a = at_weights_a * rho (mbis.py:167-203). The
no-alloc call, fed the same rho_a, weights and distances in caller-owned
device memory, must return the same parameters (relative 1e-7, the FP64
parameter tolerance of the parity tests), on two calls in a row (the static
scratch keeps the previous call's contents).

This file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest

from horton_part_gb300 import _lib, synthetic
from horton_part_gb300.mbis import get_initial_mbis_propars, get_nshell

pytestmark = pytest.mark.gpu

P_RTOL = 1e-7


def _dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def test_noalloc_inner_solve_matches_job_entry_points():
    import torch

    from horton_part_gb300.build import build

    build()
    torch.cuda.set_device(0)
    mol = synthetic.water(nrad=40, nang=50)
    nsh = [int(get_nshell(z)) for z in mol.numbers]
    off = np.concatenate([[0], np.cumsum(nsh)]).astype(np.int32)
    init = np.concatenate([get_initial_mbis_propars(z) for z in mol.numbers])
    ranges = 2 * off

    # existing entry points: one outer iteration = one inner solve per atom
    ctx = _lib.Context(0)
    job = _lib.Job(ctx, "mbis", mol.coordinates, mol.pseudo_numbers, mol.grid.points,
                   mol.grid.weights, mol.density, off, init, threshold=1e-6, maxiter=1,
                   inner_threshold=1e-8, inner_maxiter=2000)
    job.run()
    res = job.results(at_weights=True)
    job.close()
    ctx.close()
    want = res["propars"]

    L = _lib.lib()
    w_dev = _dev(torch, mol.grid.weights)
    for call in range(2):
        got = np.zeros_like(want)
        for a in range(mol.natom):
            rho_a = _dev(torch, res["at_weights"][a] * mol.density)
            r = _dev(torch, np.linalg.norm(mol.grid.points - mol.coordinates[a], axis=1))
            par = _dev(torch, init[ranges[a]:ranges[a + 1]])
            niter, conv = ctypes.c_int32(), ctypes.c_int32()
            rc = L.hp_mbis_inner_noalloc(rho_a.data_ptr(), w_dev.data_ptr(), r.data_ptr(),
                                         mol.npoint, nsh[a], par.data_ptr(), 1e-8, 1e-15, 2000,
                                         ctypes.byref(niter), ctypes.byref(conv),
                                         torch.cuda.current_stream().cuda_stream)
            assert rc == _lib.HP_OK
            assert conv.value == 1 and 1 < niter.value < 2000
            torch.cuda.synchronize()
            got[ranges[a]:ranges[a + 1]] = par.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=P_RTOL, atol=0)


def _job_inner_solve(mol, init, off):
    """One outer iteration through the job entry points: one inner solve per atom."""
    ctx = _lib.Context(0)
    job = _lib.Job(ctx, "mbis", mol.coordinates, mol.pseudo_numbers, mol.grid.points,
                   mol.grid.weights, mol.density, off, init, threshold=1e-6, maxiter=1,
                   inner_threshold=1e-8, inner_maxiter=2000)
    job.run()
    res = job.results(at_weights=True)
    job.close()
    ctx.close()
    return res


def _noalloc(torch, L, rho_a, w, r, par0, nshell, maxiter):
    par = _dev(torch, par0)
    niter, conv = ctypes.c_int32(), ctypes.c_int32()
    rc = L.hp_mbis_inner_noalloc(rho_a.data_ptr(), w.data_ptr(), r.data_ptr(), rho_a.numel(),
                                 nshell, par.data_ptr(), 1e-8, 1e-15, maxiter, ctypes.byref(niter),
                                 ctypes.byref(conv), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.HP_OK, L.hp_last_error()
    torch.cuda.synchronize()
    return par.cpu().numpy(), niter.value, conv.value


def test_noalloc_maxiter_and_a_smaller_call_after_a_larger_one():
    """Stopping at maxiter returns converged=0, niter=maxiter and the
    parameters of the last update (three steps of the oracle's inner loop,
    mbis.py:122-160); a call with fewer shells and points right after a
    larger one (the scratch keeps the larger call's tiles) still matches the
    job entry point."""
    import torch

    from horton_part_gb300.build import build
    from oracle import hp_oracle as O

    build()
    torch.cuda.set_device(0)
    L = _lib.lib()
    big = synthetic.water(nrad=40, nang=50)
    small = synthetic.water(nrad=20, nang=50)
    for mol in (big, small):
        assert mol.numbers[0] == 8 and mol.numbers[1] == 1
    nsh = [int(get_nshell(z)) for z in big.numbers]
    off = np.concatenate([[0], np.cumsum(nsh)]).astype(np.int32)
    init = np.concatenate([get_initial_mbis_propars(z) for z in big.numbers])
    ranges = 2 * off
    res_big = _job_inner_solve(big, init, off)
    res_small = _job_inner_solve(small, init, off)

    # oxygen of the large grid, stopped after three inner iterations
    rho_o = res_big["at_weights"][0] * big.density
    r_o = np.linalg.norm(big.grid.points - big.coordinates[0], axis=1)
    want3, n3, c3 = O.opt_mbis_propars(rho_o.copy(), init[0:4].copy(), big.grid.weights, r_o, 1e-8,
                                       maxiter=3)
    assert (n3, c3) == (3, False)
    got3, nit, conv = _noalloc(torch, L, _dev(torch, rho_o), _dev(torch, big.grid.weights),
                               _dev(torch, r_o), init[0:4], 2, 3)
    assert (nit, conv) == (3, 0)
    np.testing.assert_allclose(got3, want3, rtol=P_RTOL, atol=0)

    # then hydrogen (one shell) of the small grid: fewer tiles than the call before
    a = 1
    rho_h = res_small["at_weights"][a] * small.density
    r_h = np.linalg.norm(small.grid.points - small.coordinates[a], axis=1)
    got, nit, conv = _noalloc(torch, L, _dev(torch, rho_h), _dev(torch, small.grid.weights),
                              _dev(torch, r_h), init[ranges[a]:ranges[a + 1]], nsh[a], 2000)
    assert conv == 1 and 1 < nit < 2000
    np.testing.assert_allclose(got, res_small["propars"][ranges[a]:ranges[a + 1]], rtol=P_RTOL,
                               atol=0)


def test_noalloc_rejects_sizes_beyond_its_limit():
    import torch

    from horton_part_gb300.build import build

    build()
    L = _lib.lib()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = torch.ones(2, dtype=torch.float64, device="cuda")
    args = (x.data_ptr(), x.data_ptr(), x.data_ptr())
    assert L.hp_mbis_inner_noalloc(*args, 2_097_153, 1, p.data_ptr(), 1e-8, 1e-15, 10, None,
                                   None, None) == _lib.HP_ERR_INVALID
    assert L.hp_mbis_inner_noalloc(*args, 8, 8, p.data_ptr(), 1e-8, 1e-15, 10, None, None,
                                   None) == _lib.HP_ERR_INVALID
