"""GPU parity of the element / vector / diagonal-matrix operators against the CPU oracle.

Every test runs the operator through the C ABI (libgfgpu.so via the goosefem_gb300 mirror of the
GooseFEM API) and compares with the oracle on the same seeded inputs:
 - strict mode: identical bits (the reference's operation order, no FMA contraction);
 - fast mode:   max|gpu - oracle| / max|oracle| <= 1e-12.
"""

import numpy as np
import pytest

from _common import RTOL, rel_err, seeded_field, seeded_material, to_np

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    yield gf
    gf.set_strict(False)


def _same(a, b, strict):
    if strict:
        assert np.array_equal(a, b), f"not bit-exact: rel err {rel_err(a, b):.3e}"
    else:
        assert rel_err(a, b) <= RTOL, f"rel err {rel_err(a, b):.3e}"


@pytest.mark.parametrize("strict", [True, False])
def test_quad4_force_chain_64x64(gf, oracle, strict):
    """The 64x64 Quad4 workload: AsElement -> SymGradN_vector -> stress -> Int_gradN_dot_tensor2_dV
    -> AssembleNode, and the lumped mass through MatrixDiagonal; every array vs the oracle."""
    gf.set_strict(strict)
    nx = 64
    mesh = gf.Mesh.Quad4.Regular(nx, nx)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 1)
    u = seeded_field((mesh.nnode(), 2), 2)

    vector = gf.Vector(conn, dofs)
    x = vector.AsElement(coor)
    quad = gf.Element.Quad4.Quadrature(x)
    ue = vector.AsElement(u)
    eps = quad.SymGradN_vector(ue)
    sig = gf.elastic_stress(eps, K, G)
    fe = quad.Int_gradN_dot_tensor2_dV(sig)
    fint = vector.AssembleNode(fe)

    R = oracle
    xr = R.as_element(conn, coor)
    dNx_r, vol_r = R.compute_dN(xr, *R.quad4_gauss())
    ue_r = R.as_element(conn, u)
    eps_r = R.sym_grad_n_vector(dNx_r, ue_r)
    sig_r = R.elastic_stress(eps_r, K, G)
    fe_r = R.int_grad_n_dot_tensor2_dv(dNx_r, vol_r, sig_r)
    fint_r = R.assemble_node(conn, dofs, fe_r)

    assert np.array_equal(to_np(x), xr)
    assert np.array_equal(to_np(quad.GradN()), dNx_r)  # set-up is always strict
    assert np.array_equal(to_np(quad.dV()), vol_r)
    assert np.array_equal(to_np(ue), ue_r)
    _same(to_np(eps), eps_r, strict)
    _same(to_np(sig), sig_r, strict)
    _same(to_np(fe), fe_r, strict)
    _same(to_np(fint), fint_r, strict)

    # lumped mass (nodal quadrature, density 1) through MatrixDiagonal
    nodal = gf.Element.Quad4.Quadrature(x, gf.Element.Quad4.Nodal.xi(), gf.Element.Quad4.Nodal.w())
    rho = np.ones((mesh.nelem(), 4))
    Me = nodal.Int_N_scalar_NT_dV(rho)
    M = gf.MatrixDiagonal(conn, dofs)
    M.assemble(Me)
    xin, win = R.quad4_nodal()
    _, voln = R.compute_dN(xr, xin, win)
    Nn, _ = R.shape(xin)
    Me_r = R.int_n_scalar_nt_dv(Nn, voln, rho, 2)
    _same(to_np(Me), Me_r, strict)
    A_r = R.diag_assemble(conn, dofs, Me_r)
    _same(to_np(M.data()), A_r, strict)
    b = seeded_field((mesh.nnode(), 2), 3)
    _same(to_np(M.Solve(b)), R.diag_solve(dofs, A_r, b), strict)
    _same(to_np(M.Dot(b)), R.diag_dot(dofs, A_r, b), strict)


@pytest.mark.parametrize("strict", [True, False])
def test_hex8_force_chain(gf, oracle, strict):
    gf.set_strict(strict)
    mesh = gf.Mesh.Hex8.Regular(6, 5, 4, 0.5)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 4)
    u = seeded_field((mesh.nnode(), 3), 5)
    vector = gf.Vector(conn, dofs)
    quad = gf.Element.Hex8.Quadrature(vector.AsElement(coor))
    ue = vector.AsElement(u)
    eps = quad.SymGradN_vector(ue)
    sig = gf.elastic_stress(eps, K, G)
    fe = quad.Int_gradN_dot_tensor2_dV(sig)
    fint = vector.AssembleNode(fe)

    R = oracle
    dNx_r, vol_r = R.compute_dN(R.as_element(conn, coor), *R.hex8_gauss())
    assert np.array_equal(to_np(quad.GradN()), dNx_r)
    assert np.array_equal(to_np(quad.dV()), vol_r)
    eps_r = R.sym_grad_n_vector(dNx_r, R.as_element(conn, u))
    sig_r = R.elastic_stress(eps_r, K, G)
    fe_r = R.int_grad_n_dot_tensor2_dv(dNx_r, vol_r, sig_r)
    _same(to_np(eps), eps_r, strict)
    _same(to_np(sig), sig_r, strict)
    _same(to_np(fe), fe_r, strict)
    _same(to_np(fint), R.assemble_node(conn, dofs, fe_r), strict)
    _same(to_np(quad.GradN_vector(ue)), R.grad_n_vector(dNx_r, R.as_element(conn, u)), strict)
    _same(to_np(quad.GradN_vector_T(ue)), R.grad_n_vector_T(dNx_r, R.as_element(conn, u)), strict)


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("elem", ["quad4", "hex8"])
def test_quadrature_operators(gf, oracle, strict, elem):
    """GradN_vector(_T), InterpQuad_vector, Int_N_vector_dV, Int_N_scalar_NT_dV and
    Int_gradN_dot_tensor4_dot_gradNT_dV on a distorted mesh (random node perturbation)."""
    gf.set_strict(strict)
    R = oracle
    if elem == "quad4":
        mesh = gf.Mesh.Quad4.Regular(7, 5)
        E, rule, nd = gf.Element.Quad4, R.quad4_gauss(), 2
    else:
        mesh = gf.Mesh.Hex8.Regular(3, 4, 2)
        E, rule, nd = gf.Element.Hex8, R.hex8_gauss(), 3
    coor = mesh.coor() + seeded_field((mesh.nnode(), nd), 6, amp=0.15)
    conn, dofs = mesh.conn(), mesh.dofs()
    vector = gf.Vector(conn, dofs)
    quad = E.Quadrature(vector.AsElement(coor))
    xr = R.as_element(conn, coor)
    dNx_r, vol_r = R.compute_dN(xr, *rule)
    assert np.array_equal(to_np(quad.GradN()), dNx_r)
    assert np.array_equal(to_np(quad.dV()), vol_r)
    N_r, _ = R.shape(rule[0])
    assert np.array_equal(to_np(quad.N()), N_r)

    u = seeded_field((mesh.nnode(), nd), 7)
    ue_r = R.as_element(conn, u)
    ue = vector.AsElement(u)
    _same(to_np(quad.GradN_vector(ue)), R.grad_n_vector(dNx_r, ue_r), strict)
    _same(to_np(quad.GradN_vector_T(ue)), R.grad_n_vector_T(dNx_r, ue_r), strict)
    _same(to_np(quad.SymGradN_vector(ue)), R.sym_grad_n_vector(dNx_r, ue_r), strict)
    _same(to_np(quad.InterpQuad_vector(ue)), R.interp_quad_vector(N_r, ue_r), strict)
    nip = quad.nip()
    qv = seeded_field((mesh.nelem(), nip, nd), 8)
    _same(to_np(quad.Int_N_vector_dV(qv)), R.int_n_vector_dv(N_r, vol_r, qv), strict)
    qs = seeded_field((mesh.nelem(), nip), 9)
    _same(to_np(quad.Int_N_scalar_NT_dV(qs)), R.int_n_scalar_nt_dv(N_r, vol_r, qs, nd), strict)
    C4 = seeded_field((mesh.nelem(), nip) + (nd,) * 4, 10)
    _same(to_np(quad.Int_gradN_dot_tensor4_dot_gradNT_dV(C4)),
          R.int_grad_n_dot_tensor4_dot_grad_nt_dv(dNx_r, vol_r, C4), strict)


@pytest.mark.parametrize("strict", [True, False])
def test_quad4_planar_operators(gf, oracle, strict):
    """Element::Quad4::QuadraturePlanar on a distorted mesh with thickness 1.7: dV, the 3x3
    gradients, the plane-strain force chain (3-d stress incl. sigma_zz), Int_N_scalar_NT_dV and
    the in-plane stiffness integral of a [3,3,3,3] tensor, against the oracle."""
    gf.set_strict(strict)
    R = oracle
    mesh = gf.Mesh.Quad4.Regular(7, 5)
    coor = mesh.coor() + seeded_field((mesh.nnode(), 2), 16, amp=0.15)
    conn, dofs = mesh.conn(), mesh.dofs()
    vector = gf.Vector(conn, dofs)
    quad = gf.Element.Quad4.QuadraturePlanar(vector.AsElement(coor), thick=1.7)
    assert quad.tdim() == 3 and quad.shape_qtensor(2) == (mesh.nelem(), 4, 3, 3)
    xr = R.as_element(conn, coor)
    dNx_r, vol_r = R.quad4_planar_compute_dN(xr, *R.quad4_gauss(), thick=1.7)
    assert np.array_equal(to_np(quad.GradN()), dNx_r)
    assert np.array_equal(to_np(quad.dV()), vol_r)
    u = seeded_field((mesh.nnode(), 2), 17)
    ue_r = R.as_element(conn, u)
    ue = vector.AsElement(u)
    for mode, fn in enumerate((quad.GradN_vector, quad.GradN_vector_T, quad.SymGradN_vector)):
        _same(to_np(fn(ue)), R.grad_n_vector_planar(dNx_r, ue_r, mode), strict)
    K, G = seeded_material(mesh.nelem(), 18)
    eps_r = R.grad_n_vector_planar(dNx_r, ue_r, 2)
    sig = gf.elastic_stress(quad.SymGradN_vector(ue), K, G)
    sig_r = R.elastic_stress(eps_r, K, G)
    _same(to_np(sig), sig_r, strict)
    assert np.abs(sig_r[..., 2, 2]).max() > 0.0  # plane strain: sigma_zz != 0
    _same(to_np(quad.Int_gradN_dot_tensor2_dV(sig)),
          R.int_grad_n_dot_tensor2_dv_planar(dNx_r, vol_r, sig_r), strict)
    N_r, _ = R.shape(R.quad4_gauss()[0])
    qs = seeded_field((mesh.nelem(), 4), 19)
    _same(to_np(quad.Int_N_scalar_NT_dV(qs)), R.int_n_scalar_nt_dv(N_r, vol_r, qs, 2), strict)
    C4 = seeded_field((mesh.nelem(), 4) + (3,) * 4, 20)
    _same(to_np(quad.Int_gradN_dot_tensor4_dot_gradNT_dV(C4)),
          R.int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(dNx_r, vol_r, C4), strict)


def test_vector_periodic(gf, oracle):
    """Vector conversions with periodic dofs (ties): asDofs (last writer wins), asNode,
    assembleDofs (nodevec and elemvec) and assembleNode are bit-exact."""
    R = oracle
    mesh = gf.Mesh.Quad4.Regular(9, 6)
    conn, dofs = mesh.conn(), mesh.dofsPeriodic()
    vector = gf.Vector(conn, dofs)
    nv = seeded_field((mesh.nnode(), 2), 11)
    ev = seeded_field((mesh.nelem(), 4, 2), 12)
    dv = seeded_field((vector.ndof(),), 13)
    assert np.array_equal(to_np(vector.AsDofs(nv)), R.as_dofs(dofs, nv))
    assert np.array_equal(to_np(vector.AsDofs(ev)), R.as_dofs_elemvec(conn, dofs, ev))
    assert np.array_equal(to_np(vector.AsNode(dv)), R.as_node(dofs, dv))
    assert np.array_equal(to_np(vector.AsElement(dv)), R.as_element_dofval(conn, dofs, dv))
    assert np.array_equal(to_np(vector.AssembleDofs(nv)), R.assemble_dofs(dofs, nv))
    assert np.array_equal(to_np(vector.AssembleDofs(ev)), R.assemble_dofs_elemvec(conn, dofs, ev))
    assert np.array_equal(to_np(vector.AssembleNode(ev)), R.assemble_node(conn, dofs, ev))


def test_matrix_diagonal_partitioned(gf, oracle):
    """MatrixDiagonalPartitioned assemble / solve (unknown dofs only) / reaction / dot."""
    R = oracle
    mesh = gf.Mesh.Quad4.Regular(8, 5)
    conn, dofs, coor = mesh.conn(), mesh.dofs(), mesh.coor()
    iip = np.concatenate([dofs[mesh.nodesBottomEdge(), :].ravel(), dofs[mesh.nodesTopEdge(), 1]])
    M = gf.MatrixDiagonalPartitioned(conn, dofs, iip)
    vector = gf.Vector(conn, dofs)
    x = vector.AsElement(coor)
    nodal = gf.Element.Quad4.Quadrature(x, gf.Element.Quad4.Nodal.xi(), gf.Element.Quad4.Nodal.w())
    rho = seeded_field((mesh.nelem(), 4), 14) + 2.0
    Me = nodal.Int_N_scalar_NT_dV(rho)
    M.assemble(Me)
    iiu, part = R.partition(dofs, iip)
    assert np.array_equal(M.iiu(), iiu) and np.array_equal(M.part(), part)
    Auu, App = R.diagp_assemble(conn, part, iiu.size, iip.size, to_np(Me))
    assert np.array_equal(to_np(M.data_uu()), Auu)
    assert np.array_equal(to_np(M.data_pp()), App)
    b = seeded_field((mesh.nnode(), 2), 15)
    x0 = seeded_field((mesh.nnode(), 2), 16)
    assert np.array_equal(to_np(M.Solve(b, x0)), R.diagp_solve(part, iiu.size, Auu, b, x0))
    assert np.array_equal(to_np(M.Reaction(x0, b)), R.diagp_reaction(part, iiu.size, App, x0, b))


def test_errors_are_reported(gf):
    """Bad shapes and unsupported element types raise; the context stays usable."""
    import torch

    mesh = gf.Mesh.Quad4.Regular(3, 3)
    vector = gf.Vector(mesh.conn(), mesh.dofs())
    with pytest.raises(ValueError):
        vector.asElement(np.zeros((mesh.nnode(), 2)), torch.empty((3, 3), dtype=torch.float64,
                                                                  device="cuda"))
    from goosefem_gb300 import _lib
    with pytest.raises(gf.GFGPUError):
        _lib.call("gfgpu_grad_n_vector", 0, 0, 1, 3, 4, 2, 0, None)
    # still usable
    assert np.isfinite(to_np(vector.AsElement(np.ones((mesh.nnode(), 2))))).all()
