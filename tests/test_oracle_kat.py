"""Pin the CPU oracle against GooseFEM's own known-answer tests (no GPU).

The fixture ``tests/golden/reference_kat.json`` holds the literal arrays of the
reference's C++ test-suite (see ``tests/golden/make_golden.py``); each case below
names the reference test it ports.
"""

import json
import os

import numpy as np
import pytest

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))


def kat(name, dtype=None):
    return np.array(KAT[name]["value"], dtype=dtype)


def test_quad4_regular_golden(oracle):
    # tests/basic/MeshQuad4.cpp:8-101 (Regular 5x3)
    coor, conn = oracle.quad4_regular(5, 3)
    assert np.array_equal(coor, kat("quad4_5x3_coor", float))
    assert np.array_equal(conn, kat("quad4_5x3_conn", np.int64))
    assert np.array_equal(oracle.dofs(24, 2), kat("quad4_5x3_dofs", np.int64))
    npr = oracle.quad4_nodes_periodic(5, 3)
    assert np.array_equal(npr, kat("quad4_5x3_nodesPeriodic", np.int64))
    assert np.array_equal(oracle.dofs_periodic(24, 2, npr), kat("quad4_5x3_dofsPeriodic", np.int64))
    nx, ny = 5, 3
    assert np.array_equal(np.arange(nx + 1), kat("quad4_5x3_nodesBottomEdge"))
    assert np.array_equal(np.arange(nx + 1) + ny * (nx + 1), kat("quad4_5x3_nodesTopEdge"))


def test_hex8_regular_golden(oracle):
    # tests/basic/MeshHex8.cpp:6-190 (Regular 3x3x3)
    coor, conn = oracle.hex8_regular(3, 3, 3)
    assert np.array_equal(coor, kat("hex8_3x3x3_coor", float))
    assert np.array_equal(conn, kat("hex8_3x3x3_conn", np.int64))
    assert np.array_equal(oracle.dofs(64, 3), kat("hex8_3x3x3_dofs", np.int64))
    # dofsPeriodic from the reference's own nodesPeriodic list (Mesh.h:291-306)
    npr = kat("hex8_3x3x3_nodesPeriodic", np.int64)
    assert np.array_equal(oracle.dofs_periodic(64, 3, npr), kat("hex8_3x3x3_dofsPeriodic", np.int64))
    # the restated 3-d nodesPeriodic list itself (Mesh.h:1577-1692)
    assert np.array_equal(oracle.hex8_nodes_periodic(3, 3, 3), npr)
    front = np.arange(16)
    assert np.array_equal(front, kat("hex8_3x3x3_nodesFront"))
    assert np.array_equal(front + 3 * 16, kat("hex8_3x3x3_nodesBack"))


def test_coordination_elem2node_golden(oracle):
    # tests/basic/Mesh.cpp:199-236
    _, conn = oracle.quad4_regular(3, 3)
    assert np.array_equal(oracle.coordination(conn), kat("quad4_3x3_coordination"))
    ptr, idx = oracle.elem2node(conn)
    expect = KAT["quad4_3x3_elem2node"]["value"]
    for n, row in enumerate(expect):
        assert list(idx[ptr[n]:ptr[n + 1]]) == row


@pytest.mark.parametrize("partitioned", [False, True])
def test_lumped_mass_golden(oracle, partitioned):
    # tests/basic/MatrixDiagonal.cpp:12-53 and MatrixDiagonalPartitioned.cpp:12-54
    coor, conn = oracle.quad4_regular(2, 2)
    dofs = oracle.dofs(9, 2)
    xi, w = oracle.quad4_nodal()
    x = oracle.as_element(conn, coor)
    dNx, vol = oracle.compute_dN(x, xi, w)
    N, _ = oracle.shape(xi)
    M = oracle.int_n_scalar_nt_dv(N, vol, np.ones((4, 4)), 2)
    assert oracle.is_diagonal(M)
    if not partitioned:
        A = oracle.diag_assemble(conn, dofs, M)
        assert np.allclose(A, kat("quad4_2x2_lumped_mass"))
    else:
        iip = np.array([0, 2])
        iiu, part = oracle.partition(dofs, iip)
        Auu, App = oracle.diagp_assemble(conn, part, iiu.size, iip.size, M)
        A = np.zeros(18)
        A[iiu] = Auu
        A[iip] = App
        assert np.allclose(A, kat("quad4_2x2_lumped_mass_partitioned"))


def _affine(oracle, nx, ny, F):
    coor, conn = oracle.quad4_regular(nx, ny)
    disp = coor @ F.T
    return coor, conn, disp


def test_quad4_patch_tests(oracle):
    # tests/basic/ElementQuad4.cpp:17-153: dV, GradN_vector(_T), SymGradN_vector of an affine field
    F = np.zeros((2, 2))
    F[0, 1] = 0.1
    coor, conn, disp = _affine(oracle, 3, 3, F)
    xi, w = oracle.quad4_gauss()
    dNx, vol = oracle.compute_dN(oracle.as_element(conn, coor), xi, w)
    assert np.allclose(vol, 0.25)
    ue = oracle.as_element(conn, disp)
    assert np.allclose(oracle.grad_n_vector(dNx, ue), F.T)
    assert np.allclose(oracle.grad_n_vector_T(dNx, ue), F)
    eps = oracle.sym_grad_n_vector(dNx, ue)
    assert np.allclose(eps, 0.5 * (F + F.T))
    N, _ = oracle.shape(xi)
    uq = oracle.interp_quad_vector(N, oracle.as_element(conn, np.ones_like(coor)))
    assert np.allclose(uq, 1.0)


def test_quad4_periodic_integrals(oracle):
    # tests/basic/ElementQuad4.cpp:155-218: Int_N_vector_dV, lumped mass = 1 and equilibrium on
    # periodic dofs.
    coor, conn = oracle.quad4_regular(3, 3)
    dofs = oracle.dofs_periodic(16, 2, oracle.quad4_nodes_periodic(3, 3))
    xi, w = oracle.quad4_gauss()
    x = oracle.as_element(conn, coor)
    dNx, vol = oracle.compute_dN(x, xi, w)
    N, _ = oracle.shape(xi)
    qv = np.empty((9, 4, 2))
    qv[..., 0] = 2.0
    qv[..., 1] = 5.0
    nv = oracle.assemble_node(conn, dofs, oracle.int_n_vector_dv(N, vol, qv))
    assert np.allclose(nv[:, 0], 2.0) and np.allclose(nv[:, 1], 5.0)

    xin, wn = oracle.quad4_nodal()
    Nn, _ = oracle.shape(xin)
    _, voln = oracle.compute_dN(x, xin, wn)
    M = oracle.int_n_scalar_nt_dv(Nn, voln, np.ones((9, 4)), 2)
    assert np.allclose(oracle.diag_assemble(conn, dofs, M), 1.0)

    F = np.zeros((2, 2))
    F[0, 1] = 0.1
    eps = oracle.sym_grad_n_vector(dNx, oracle.as_element(conn, coor @ F.T))
    fi = oracle.assemble_dofs_elemvec(conn, dofs, oracle.int_grad_n_dot_tensor2_dv(dNx, vol, eps))
    assert np.allclose(fi, 0.0)


def test_hex8_patch_and_equilibrium(oracle):
    # tests/basic/ElementHex8.cpp:19-203 (dV = 0.125, affine patch, equilibrium)
    coor, conn = oracle.hex8_regular(3, 3, 3)
    xi, w = oracle.hex8_gauss()
    x = oracle.as_element(conn, coor)
    dNx, vol = oracle.compute_dN(x, xi, w)
    assert np.allclose(vol, 0.125)
    F = np.zeros((3, 3))
    F[0, 1] = 0.1
    F[2, 0] = -0.05
    ue = oracle.as_element(conn, coor @ F.T)
    assert np.allclose(oracle.grad_n_vector(dNx, ue), F.T)
    eps = oracle.sym_grad_n_vector(dNx, ue)
    assert np.allclose(eps, 0.5 * (F + F.T))
    dofs = oracle.dofs_periodic(64, 3, kat("hex8_3x3x3_nodesPeriodic", np.int64))
    fi = oracle.assemble_dofs_elemvec(conn, dofs, oracle.int_grad_n_dot_tensor2_dv(dNx, vol, eps))
    assert np.allclose(fi, 0.0)


def test_vector_periodic_kat(oracle):
    # tests/basic/Vector.cpp:10-166 (AsDofs / AssembleDofs with periodic dofs, abs 1e-12)
    coor, conn = oracle.quad4_regular(2, 2)
    dofs = oracle.dofs_periodic(9, 2, oracle.quad4_nodes_periodic(2, 2))
    v = np.array([[1, 0], [1, 0], [1, 0], [1.5, 0], [1.5, 0], [1.5, 0], [1, 0], [1, 0], [1, 0]],
                 dtype=float)
    V = oracle.as_dofs(dofs, v)
    assert V.size == 8
    expect = [v[0, 0], v[0, 1], v[1, 0], v[1, 1], v[3, 0], v[3, 1], v[4, 0], v[4, 1]]
    assert np.allclose(V, expect, atol=1e-12, rtol=0)
    V2 = oracle.as_dofs_elemvec(conn, dofs, oracle.as_element_dofval(conn, dofs, V))
    assert np.allclose(V2, expect, atol=1e-12, rtol=0)
    f = np.array([[-1, -1], [0, -1], [1, -1], [-1, 0], [0, 0], [1, 0], [-1, 1], [0, 1], [1, 1]],
                 dtype=float)
    assert np.allclose(oracle.assemble_dofs(dofs, f), 0.0, atol=1e-12, rtol=0)
    assert np.allclose(oracle.assemble_dofs_elemvec(conn, dofs, oracle.as_element(conn, f)), 0.0,
                       atol=1e-12, rtol=0)


def test_matrix_diagonal_dot_solve(oracle):
    # tests/basic/MatrixDiagonal.cpp:55-89 (dot and solve with random data)
    rng = np.random.default_rng(0)
    dofs = oracle.dofs(9, 2)
    a = rng.random(18) + 0.1
    x = rng.random((9, 2))
    b = oracle.diag_dot(dofs, a, x)
    assert np.allclose(b, a.reshape(9, 2) * x)
    assert np.allclose(oracle.diag_solve(dofs, a, b), x)


def test_hex8_compute_dn_index_anomaly_is_inert_on_boxes(oracle):
    # Element.h:1220 accumulates Jinv(i,j)*dNxi(m,i); on axis-aligned boxes this equals the
    # textbook Jinv . dNxi bit for bit.
    coor, conn = oracle.hex8_regular(2, 2, 2, 0.7)
    xi, w = oracle.hex8_gauss()
    x = oracle.as_element(conn, coor)
    dNx, vol = oracle.compute_dN(x, xi, w)
    _, dNxi = oracle.shape(xi)
    J = np.einsum("qmi,emj->eqij", dNxi, x)
    Jinv = np.linalg.inv(J)
    textbook = np.einsum("eqij,qmj->eqmi", Jinv, dNxi)
    assert np.allclose(dNx, textbook, rtol=1e-14, atol=0)


def test_quad4_planar_properties(oracle):
    # tests/basic/ElementQuad4Planar.cpp:8-207: shapes, dV = 0.25 (x thickness), 3x3 GradN_vector
    # (F^T), GradN_vector_T (F), SymGradN_vector and its volume average, lumped mass = 1 on
    # periodic dofs, equilibrium of a homogeneous strain.
    coor, conn = oracle.quad4_regular(3, 3)
    xi, w = oracle.quad4_gauss()
    x = oracle.as_element(conn, coor)
    dNx, vol = oracle.quad4_planar_compute_dN(x, xi, w)
    assert dNx.shape == (9, 4, 4, 2) and np.allclose(vol, 0.25)
    dNq, volq = oracle.compute_dN(x, xi, w)
    assert np.array_equal(dNx, dNq) and np.array_equal(vol, volq)
    _, vol2 = oracle.quad4_planar_compute_dN(x, xi, w, thick=2.5)
    assert np.array_equal(vol2, volq * 2.5)
    F = np.zeros((3, 3))
    F[0, 1] = 0.1
    ue = oracle.as_element(conn, coor @ F[:2, :2].T)
    g = oracle.grad_n_vector_planar(dNx, ue, 0)
    gT = oracle.grad_n_vector_planar(dNx, ue, 1)
    eps = oracle.grad_n_vector_planar(dNx, ue, 2)
    assert g.shape == (9, 4, 3, 3)
    assert np.allclose(g, F.T) and np.allclose(gT, F) and np.allclose(eps, 0.5 * (F + F.T))
    epsbar = np.average(eps, axis=(0, 1), weights=np.broadcast_to(vol[..., None, None], eps.shape))
    assert np.allclose(epsbar, 0.5 * (F + F.T))
    # the in-plane blocks are the Quad4 operators bit for bit; everything else is 0
    for mode in (0, 1, 2):
        q4 = oracle._grad(dNq, ue, mode)
        p = oracle.grad_n_vector_planar(dNx, ue, mode)
        assert np.array_equal(p[..., :2, :2], q4)
        assert not p[..., 2, :].any() and not p[..., :, 2].any()
    dofs = oracle.dofs_periodic(16, 2, oracle.quad4_nodes_periodic(3, 3))
    xin, wn = oracle.quad4_nodal()
    Nn, _ = oracle.shape(xin)
    _, voln = oracle.quad4_planar_compute_dN(x, xin, wn)
    M = oracle.int_n_scalar_nt_dv(Nn, voln, np.ones((9, 4)), 2)
    A = oracle.diag_assemble(conn, dofs, M)
    assert np.allclose(A, 1.0)
    fe = oracle.int_grad_n_dot_tensor2_dv_planar(dNx, vol, eps)
    fi = oracle.assemble_dofs_elemvec(conn, dofs, fe)
    assert np.allclose(fi, 0.0)
    # stiffness: the in-plane block of a 3x3x3x3 tensor, equal to the Quad4 integral
    rng = np.random.default_rng(3)
    C3 = rng.normal(size=(9, 4, 3, 3, 3, 3))
    Kp = oracle.int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(dNx, vol, C3)
    C2 = np.ascontiguousarray(C3[..., :2, :2, :2, :2])
    Kq = oracle.int_grad_n_dot_tensor4_dot_grad_nt_dv(dNq, volq, C2)
    assert np.array_equal(Kp, Kq)
