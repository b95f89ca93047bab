"""The two-level correction of the static solve (csrc/coarse.cu): the Galerkin coarse matrix
measured by coloured probes of the matrix-free operator against the scipy restatement
(oracle/coarse.py), its FP32 inverse, the correction itself, and the flexible CG with the
correction (with and without the network direction) against the direct solve."""

import ctypes as C

import numpy as np
import pytest
import torch

from _common import rel_err

pytestmark = pytest.mark.gpu


def _problem(nx, ny, seed=3):
    from goosefem_gb300 import learned as LR
    from goosefem_gb300 import mesh as M

    K, G, _ = LR.inclusion_material(nx, ny, seed, rmin=2.0, rmax=5.0)
    m = M.Quad4.Regular(nx, ny)
    iip, xp = LR.static_bc(m)
    lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=0)
    return m, K, G, iip, xp, lp


def _oracle_coarse(m, K, G, iip, nx, ny, hc):
    from oracle import coarse as OC
    from oracle import statics as S

    A = S.stiffness(m.coor(), m.conn(), K, G)
    free = np.ones(A.shape[0], dtype=bool)
    free[iip] = False
    P = OC.prolongation(nx, ny, hc, free)
    return A, free, P, OC.galerkin(A, P)


@pytest.mark.parametrize("nx,ny,hc", [(40, 28, 8), (37, 30, 8), (24, 24, 5)])
def test_coarse_matrix_and_inverse(nx, ny, hc):
    m, K, G, iip, xp, lp = _problem(nx, ny)
    ac = lp.coarse_setup(hc).cpu().numpy()
    _, _, P, ac_ref = _oracle_coarse(m, K, G, iip, nx, ny, hc)
    nc = ((nx + hc - 1) // hc + 1) * ((ny + hc - 1) // hc + 1) * 2
    assert ac.shape == ac_ref.shape == (nc, nc)
    assert rel_err(ac, ac_ref) <= 1e-12
    ainv = lp.ainv.cpu().numpy().astype(np.float64)
    assert ainv.shape[1] % 32 == 0 and np.all(ainv[:, nc:] == 0.0)
    ainv = ainv[:, :nc]
    assert np.abs(ainv @ ac_ref - np.eye(nc)).max() <= 1e-3
    # the correction z = P A_c^-1 P^T r on a random free-dof residual
    r = np.random.default_rng(4).standard_normal(P.shape[0])
    r[iip] = 0.0
    z = lp.coarse_apply(r).cpu().numpy()
    z_ref = P @ np.linalg.solve(ac_ref, P.T @ r)
    assert rel_err(z, z_ref) <= 1e-3
    assert np.all(z[iip] == 0.0)


@pytest.mark.parametrize("use_nn,post", [(False, False), (True, False), (True, True)])
def test_two_level_fcg_matches_direct_solve(use_nn, post):
    """Flexible CG with the two-level first direction (and the untrained network direction, on r
    or on the residual after the two-level step) to 1e-8: the same solution as the direct solve, in far fewer iterations than Jacobi-PCG."""
    from oracle import statics as S

    nx, ny = 64, 48
    m, K, G, iip, xp, lp = _problem(nx, ny)
    lp.coarse_setup(8)
    x = lp.initial_guess(xp)
    it2, rel2 = lp.fcg(x, tol=1e-8, use_nn=use_nn, nkeep=4, coarse=True, post=post)
    assert rel2 <= 1e-8
    A = S.stiffness(m.coor(), m.conn(), K, G)
    x_ref = S.solve_partitioned(A, iip, xp)
    assert np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref) <= 1e-6
    xj = lp.initial_guess(xp)
    itj, _ = lp.jacobi_pcg(xj)
    assert it2 * 3 < itj, (it2, itj)
    # run to run: identical bits
    x2 = lp.initial_guess(xp)
    lp.fcg(x2, tol=1e-8, use_nn=use_nn, nkeep=4, coarse=True, post=post)
    assert torch.equal(x, x2)


def test_coarse_errors():
    from goosefem_gb300 import _lib
    from goosefem_gb300.learned import CoarseDesc

    m, K, G, iip, xp, lp = _problem(16, 16)
    g = CoarseDesc()
    _lib.call("gfgpu_coarse_grid", 16, 16, 4, C.addressof(g))
    g.ncx += 1  # inconsistent with nx, hc
    with pytest.raises(_lib.GFGPUError):
        _lib.call("gfgpu_coarse_setup", lp._desc(), C.addressof(g), None, None, None, None)
    _lib.call("gfgpu_coarse_grid", 16, 15, 4, C.addressof(g))  # nodes do not match the mesh
    ws = torch.empty(1 << 20, dtype=torch.float64, device="cuda")
    out = torch.empty(64 * 64, dtype=torch.float32, device="cuda")
    with pytest.raises(_lib.GFGPUError):
        _lib.call("gfgpu_coarse_setup", lp._desc(), C.addressof(g), out.data_ptr(), None,
                  ws.data_ptr(), None)
