"""The explicit velocity-Verlet path at the full 2048 x 2048 Quad4 size (4.19 M elements, the
size of the throughput measurement, the same kernels): a few increments against the oracle's
per-operator loop (docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157 restated in
oracle/gfref.cpp), and over 1000 increments two size-independent properties of the linear,
damped dynamics: scaling the initial velocity by 2 scales every state array by exactly 2 (each
FP64 or FP32 operation commutes with a power-of-two scale), and the run is bit-identical run to
run. Both arithmetics of the square-element path run: the FP64 kernels and the float-float
("pair") fused kernel of the throughput measurement."""

import numpy as np
import pytest
import torch

from _common import RTOL, rel_err, seeded_field, seeded_material, to_np

pytestmark = pytest.mark.gpu

N = 2048


@pytest.fixture(scope="module")
def case(oracle):
    import goosefem_gb300 as gf

    mesh = gf.Mesh.Quad4.Regular(N, N)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 7)
    bottom = mesh.nodesBottomEdge()
    iip = dofs[bottom, :].ravel()
    v0 = seeded_field((mesh.nnode(), 2), 8)
    v0[bottom, :] = 0.0
    dt = 0.1 * gf.critical_dt(K, G)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, rho=1.0, dt=dt, eta=0.1, iip=iip)
    return dict(gf=gf, mesh=mesh, coor=coor, conn=conn, dofs=dofs, K=K, G=G, bottom=bottom,
                v0=v0, dt=dt, vv=vv)


def _run(case, v0, nsteps, arithmetic="fp64"):
    vv = case["vv"]
    vv.use_pair() if arithmetic == "pair" else vv.use_fp64()
    u = torch.zeros(v0.shape, dtype=torch.float64, device="cuda")
    v = torch.tensor(v0, device="cuda")
    a = torch.zeros_like(u)
    vv.step(u, v, a, nsteps)
    torch.cuda.synchronize()
    return u, v, a


@pytest.fixture(scope="module")
def oracle_4(case, oracle):
    """The oracle's loop over the first 4 increments (computed once for both arithmetics)."""
    R = oracle
    conn, dofs, coor = case["conn"], case["dofs"], case["coor"]
    nelem, nnode = conn.shape[0], coor.shape[0]
    xr = R.as_element(conn, coor)
    dNx, vol = R.compute_dN(xr, *R.quad4_gauss(), parallel=True)
    xin, win = R.quad4_nodal()
    _, voln = R.compute_dN(xr, xin, win, parallel=True)
    del xr
    Nn, _ = R.shape(xin)
    A = R.diag_assemble(conn, dofs, R.int_n_scalar_nt_dv(Nn, voln, np.ones((nelem, 4)), 2))
    del voln
    free = np.ones(nnode * 2, dtype=np.uint8)
    free.reshape(-1, 2)[case["bottom"], :] = 0
    nsteps = 4
    u = np.zeros_like(case["v0"])
    v = case["v0"].copy()
    a = np.zeros_like(u)
    R.verlet_run(conn, dofs, dNx, vol, case["K"], case["G"], A, free, None, case["dt"], 0.1,
                 nsteps, u, v, a, parallel=True)
    return nsteps, u, v, a


@pytest.mark.parametrize("arithmetic", ["fp64", "pair"])
def test_full_size_increments_match_oracle(case, oracle_4, arithmetic):
    nsteps, u, v, a = oracle_4
    ug, vg, ag = _run(case, case["v0"], nsteps, arithmetic)
    assert case["vv"].uniform  # the square-element kernels of the throughput measurement
    assert case["vv"].path == ("uniform-square-pair" if arithmetic == "pair" else "uniform-square")
    assert rel_err(to_np(ug), u) <= RTOL
    assert rel_err(to_np(vg), v) <= RTOL
    assert rel_err(to_np(ag), a) <= RTOL


@pytest.mark.parametrize("arithmetic", ["fp64", "pair"])
def test_full_size_linearity_and_determinism(case, arithmetic):
    nsteps = 1000
    u1, v1, a1 = _run(case, case["v0"], nsteps, arithmetic)
    u2, v2, a2 = _run(case, 2.0 * case["v0"], nsteps, arithmetic)
    assert torch.isfinite(u1).all() and u1.abs().max() > 0
    assert torch.equal(u2, 2.0 * u1) and torch.equal(v2, 2.0 * v1) and torch.equal(a2, 2.0 * a1)
    u3, v3, a3 = _run(case, case["v0"], nsteps, arithmetic)
    assert torch.equal(u3, u1) and torch.equal(v3, v1) and torch.equal(a3, a1)
    # the fixed bottom row never moves
    b = torch.as_tensor(case["bottom"], device="cuda").long()
    assert torch.count_nonzero(u1[b]) == 0
