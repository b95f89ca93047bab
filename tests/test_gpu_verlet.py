"""GPU parity of the fused explicit velocity-Verlet integrator against the oracle's loop
(docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157 restated in oracle/gfref.cpp)."""

import numpy as np
import pytest
import torch

from _common import RTOL, rel_err, seeded_field, seeded_material, to_np

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    yield gf
    gf.set_strict(False)


def _setup(gf, oracle, nx, ny, periodic, fixed_bottom, seed):
    mesh = gf.Mesh.Quad4.Regular(nx, ny)
    coor, conn = mesh.coor(), mesh.conn()
    dofs = mesh.dofsPeriodic() if periodic else mesh.dofs()
    K, G = seeded_material(mesh.nelem(), seed)
    iip = dofs[mesh.nodesBottomEdge(), :].ravel() if fixed_bottom else None
    v0 = seeded_field((mesh.nnode(), 2), seed + 1)
    if fixed_bottom:
        v0[mesh.nodesBottomEdge(), :] = 0.0
    if periodic:  # tied nodes share the velocity of their dof
        dv = np.zeros(int(dofs.max()) + 1)
        dv[dofs.ravel()] = v0.ravel()
        v0 = dv[dofs]
    dt = 0.1 * gf.critical_dt(K, G)
    R = oracle
    xr = R.as_element(conn, coor)
    dNx, vol = R.compute_dN(xr, *R.quad4_gauss())
    xin, win = R.quad4_nodal()
    _, voln = R.compute_dN(xr, xin, win)
    Nn, _ = R.shape(xin)
    A = R.diag_assemble(conn, dofs, R.int_n_scalar_nt_dv(Nn, voln, np.ones((mesh.nelem(), 4)), 2))
    free = np.ones(mesh.nnode() * 2, dtype=np.uint8)
    if fixed_bottom:
        free.reshape(-1, 2)[mesh.nodesBottomEdge(), :] = 0
    ref = dict(conn=conn, dofs=dofs, dNx=dNx, vol=vol, K=K, G=G, A=A, free=free)
    return mesh, coor, conn, dofs, K, G, iip, v0, dt, ref


def _run_oracle(oracle, ref, v0, dt, eta, nsteps, fext=None):
    u = np.zeros_like(v0)
    v = v0.copy()
    a = np.zeros_like(v0)
    oracle.verlet_run(ref["conn"], ref["dofs"], ref["dNx"], ref["vol"], ref["K"], ref["G"],
                      ref["A"], ref["free"], fext, dt, eta, nsteps, u, v, a)
    return u, v, a


@pytest.mark.parametrize("strict", [True, False])
def test_verlet_general_path_fixed_bottom(gf, oracle, strict):
    gf.set_strict(strict)
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 64, 64, False, True, 21)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, rho=1.0, dt=dt, eta=0.1, iip=iip,
                           uniform=False)
    assert not vv.uniform
    u = torch.zeros((mesh.nnode(), 2), dtype=torch.float64, device="cuda")
    v = torch.tensor(v0, device="cuda")
    a = torch.zeros_like(u)
    nsteps = 100
    vv.step(u, v, a, nsteps)
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, nsteps)
    for g, r in ((u, ur), (v, vr), (a, ar)):
        if strict:
            assert np.array_equal(to_np(g), r), rel_err(to_np(g), r)
        else:
            assert rel_err(to_np(g), r) <= RTOL


def test_verlet_split_calls_equal_one_call(gf, oracle):
    """step(n1) then step(n2) gives the same bits as step(n1 + n2)."""
    gf.set_strict(False)
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 33, 17, False, True, 23)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip)
    z = torch.zeros((mesh.nnode(), 2), dtype=torch.float64, device="cuda")
    s1 = [z.clone(), torch.tensor(v0, device="cuda"), z.clone()]
    s2 = [z.clone(), torch.tensor(v0, device="cuda"), z.clone()]
    vv.step(*s1, 30)
    vv.step(*s2, 10)
    vv.step(*s2, 20)
    for x, y in zip(s1, s2):
        assert torch.equal(x, y)


@pytest.mark.parametrize("variant", ["square", "onthefly"])
@pytest.mark.parametrize("periodic", [False, True])
def test_verlet_uniform_path(gf, oracle, periodic, variant):
    """The closed-form uniform Quad4 element kernels (precomputed square coefficients, or K, G
    read every increment) against the reference chain."""
    gf.set_strict(False)
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 64, 48, periodic,
                                                            not periodic, 25)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip)
    assert vv.path == "uniform-square"
    if variant == "onthefly":
        vv.use_uniform_onthefly()
        assert vv.path == "uniform"
    # internal force of a random displacement
    u_rand = seeded_field((mesh.nnode(), 2), 26)
    R = oracle
    fe_r = R.int_grad_n_dot_tensor2_dv(ref["dNx"], ref["vol"], R.elastic_stress(
        R.sym_grad_n_vector(ref["dNx"], R.as_element(conn, u_rand)), K, G))
    fint_r = R.assemble_node(conn, dofs, fe_r)
    assert rel_err(to_np(vv.internal_force(u_rand)), fint_r) <= RTOL
    # 100 increments
    u = torch.zeros((mesh.nnode(), 2), dtype=torch.float64, device="cuda")
    v = torch.tensor(v0, device="cuda")
    a = torch.zeros_like(u)
    vv.step(u, v, a, 100)
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, 100)
    for g, r in ((u, ur), (v, vr), (a, ar)):
        assert rel_err(to_np(g), r) <= RTOL


def test_verlet_rectangular_elements(gf, oracle):
    """Uniform path with hx != hy (a Regular mesh scaled anisotropically)."""
    gf.set_strict(False)
    mesh = gf.Mesh.Quad4.Regular(20, 13)
    coor = mesh.coor() * np.array([0.7, 1.3])
    conn, dofs = mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 27)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=0.01, eta=0.0)
    assert vv.uniform
    u = seeded_field((mesh.nnode(), 2), 28)
    R = oracle
    dNx, vol = R.compute_dN(R.as_element(conn, coor), *R.quad4_gauss())
    fe_r = R.int_grad_n_dot_tensor2_dv(dNx, vol, R.elastic_stress(
        R.sym_grad_n_vector(dNx, R.as_element(conn, u)), K, G))
    assert rel_err(to_np(vv.internal_force(u)), R.assemble_node(conn, dofs, fe_r)) <= RTOL


def test_verlet_distorted_mesh_uses_general_path(gf, oracle):
    gf.set_strict(False)
    mesh = gf.Mesh.Quad4.Regular(12, 9)
    coor = mesh.coor() + seeded_field((mesh.nnode(), 2), 29, amp=0.1)
    K, G = seeded_material(mesh.nelem(), 30)
    vv = gf.VelocityVerlet(coor, mesh.conn(), mesh.dofs(), K, G, dt=0.01)
    assert not vv.uniform


@pytest.mark.parametrize("periodic", [False, True])
def test_verlet_mass_class_node_update(gf, oracle, periodic):
    """The closed-form node update with lumped-mass classes (set up by default on Regular
    meshes) against the per-dof update and the oracle, with an external force as well."""
    gf.set_strict(False)
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 40, 30, periodic,
                                                            not periodic, 29)
    fext = seeded_field((mesh.nnode(), 2), 30, amp=1e-4)
    runs = []
    for per_dof in (False, True):
        vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, fext=fext)
        assert 1 <= vv.desc.ncls <= (4 if not periodic else 1)
        if per_dof:
            vv.use_per_dof_mass()
        u = torch.zeros((mesh.nnode(), 2), dtype=torch.float64, device="cuda")
        v = torch.tensor(v0, device="cuda")
        a = torch.zeros_like(u)
        vv.step(u, v, a, 100)
        runs.append((to_np(u), to_np(v), to_np(a)))
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, 100, fext)
    for k, r in enumerate((ur, vr, ar)):
        assert rel_err(runs[0][k], runs[1][k]) <= 1e-13
        assert rel_err(runs[0][k], r) <= RTOL



@pytest.mark.parametrize("periodic", [False, True])
def test_verlet_regular_node_kernel_same_bits(gf, oracle, periodic):
    """The Regular-mesh node kernel (element forces by index arithmetic) gives the same bits as
    the CSR gather; periodic dofs are not Regular-identity and keep the CSR."""
    gf.set_strict(False)
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 37, 23, periodic,
                                                            not periodic, 31)
    fext = seeded_field((mesh.nnode(), 2), 32, amp=1e-4)
    out = []
    for csr in (False, True):
        vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, fext=fext)
        assert (vv.desc.reg_nx == 37 and vv.desc.reg_ny == 23) == (not periodic)
        if csr:
            vv.use_csr_gather()
        u = torch.zeros((mesh.nnode(), 2), dtype=torch.float64, device="cuda")
        v = torch.tensor(v0, device="cuda")
        a = torch.zeros_like(u)
        vv.step(u, v, a, 50)
        out.append(torch.cat([u, v, a]))
    assert torch.equal(out[0], out[1])
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, 50, fext)
    assert rel_err(to_np(out[0][:mesh.nnode()]), ur) <= RTOL
