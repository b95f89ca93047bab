"""Assembled sparse matrices on the GPU (Matrix, MatrixPartitioned, MatrixPartitionedSolver)
against the oracle's restatement of Eigen's triplet assembly and products, and against the
matrix-free stiffness operator and the direct partitioned solve."""

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


def _same(a, b, strict):
    if strict:
        assert np.array_equal(a, b), f"not bit-exact: rel err {rel_err(a, b):.3e}"
    else:
        assert rel_err(a, b) <= RTOL, f"rel err {rel_err(a, b):.3e}"


def _stiffness_elemmat(R, coor, conn, K, G):
    from oracle import statics as S

    nd = coor.shape[1]
    xi, w = R.quad4_gauss() if nd == 2 else R.hex8_gauss()
    dNx, vol = R.compute_dN(R.as_element(conn, coor), xi, w)
    return R.int_grad_n_dot_tensor4_dot_grad_nt_dv(dNx, vol, S.elasticity_tensor(K, G, w.size, nd))


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("periodic", [False, True])
def test_matrix_assemble_and_dot(gf, oracle, strict, periodic):
    gf.set_strict(strict)
    R = oracle
    mesh = gf.Mesh.Quad4.Regular(9, 7)
    conn = mesh.conn()
    dofs = mesh.dofsPeriodic() if periodic else mesh.dofs()
    ndof = int(dofs.max()) + 1
    em = seeded_field((mesh.nelem(), 8, 8), 30)
    A = gf.Matrix(conn, dofs)
    A.assemble(em)
    rp_r, col_r, val_r = R.matrix_assemble(conn, dofs, em, ndof)
    rp, col, val = (to_np(t) for t in A.data())
    assert np.array_equal(rp, rp_r) and np.array_equal(col, col_r)
    assert np.array_equal(val, val_r)  # assembly: same summation order in both modes
    x = seeded_field((ndof,), 31)
    _same(to_np(A.Dot(x)), R.matrix_dot(rp_r, col_r, val_r, x), strict)
    # nodevec: AsDofs (last writer) -> dot -> AsNode
    xn = seeded_field((mesh.nnode(), 2), 32)
    xd = R.as_dofs(dofs, xn)
    _same(to_np(A.Dot(xn)), R.as_node(dofs, R.matrix_dot(rp_r, col_r, val_r, xd)), strict)
    dense = A.Todense()
    assert np.array_equal(dense[np.repeat(np.arange(ndof), np.diff(rp_r)), col_r], val_r)


@pytest.mark.parametrize("strict", [True, False])
def test_matrix_partitioned_dot_reaction(gf, oracle, strict):
    gf.set_strict(strict)
    R = oracle
    mesh = gf.Mesh.Hex8.Regular(3, 4, 2)
    conn, dofs = mesh.conn(), mesh.dofs()
    ndof = int(dofs.max()) + 1
    iip = np.unique(np.concatenate([dofs[mesh.nodesFront()].ravel(), dofs[mesh.nodesBack(), 2]]))
    em = seeded_field((mesh.nelem(), 24, 24), 33)
    A = gf.MatrixPartitioned(conn, dofs, iip)
    A.assemble(em)
    part_h = A._part
    nnu = A.nnu()
    rp_r, col_r, val_r = R.matrix_assemble(conn, part_h, em, ndof)
    rp, col, val = (to_np(t) for t in A.data())
    assert np.array_equal(rp, rp_r) and np.array_equal(col, col_r) and np.array_equal(val, val_r)
    part1d = np.empty(ndof, dtype=np.int64)
    part1d[A._iperm_h] = np.arange(ndof)
    x = seeded_field((ndof,), 34)
    b_r = R.matrixp_dot(rp_r, col_r, val_r, nnu, part1d, x)
    _same(to_np(A.Dot(x)), b_r, strict)
    b0 = seeded_field((ndof,), 35)
    reac = b0.copy()
    reac[A.iip()] = b_r[A.iip()]
    _same(to_np(A.Reaction(x, b0)), reac, strict)
    # the partitioned matrix is the plain matrix with rows and columns permuted
    P = gf.Matrix(conn, dofs)
    P.assemble(em)
    assert np.array_equal(A.Todense(), P.Todense())


def test_assembled_stiffness_equals_matrix_free_operator(gf, oracle):
    """K u from the assembled stiffness (GPU assembly of Int_gradN_dot_tensor4_dot_gradNT_dV)
    equals the matrix-free internal force of the same displacement."""
    from oracle import statics as S

    mesh = gf.Mesh.Quad4.Regular(12, 10)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 36)
    vector = gf.Vector(conn, dofs)
    quad = gf.Element.Quad4.Quadrature(vector.AsElement(coor))
    C4 = torch.as_tensor(S.elasticity_tensor(K, G, 4, 2), device="cuda")
    Ke = quad.Int_gradN_dot_tensor4_dot_gradNT_dV(C4)
    A = gf.Matrix(conn, dofs)
    A.assemble(Ke)
    u = seeded_field((mesh.nnode(), 2), 37)
    st = gf.ElasticStatic(coor, conn, dofs, K, G, np.array([0], dtype=np.int32))
    fint = to_np(st.force(torch.as_tensor(u, device="cuda")))
    assert rel_err(to_np(A.Dot(u)), fint) <= 1e-12


def test_matrix_partitioned_solver_vs_direct(gf, oracle):
    from oracle import statics as S

    R = oracle
    mesh = gf.Mesh.Quad4.Regular(20, 14)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 38)
    bot, top = mesh.nodesBottomEdge(), mesh.nodesTopEdge()
    iip = np.unique(np.concatenate([dofs[bot].ravel(), dofs[top, 1]]))
    xp = np.where(np.isin(iip, dofs[top, 1]), -1e-2, 0.0)
    Ke = _stiffness_elemmat(R, coor, conn, K, G)
    A = gf.MatrixPartitioned(conn, dofs, iip)
    A.assemble(Ke)
    ndof = int(dofs.max()) + 1
    x = np.zeros(ndof)
    x[iip] = xp
    solver = gf.MatrixPartitionedSolver(tol=1e-12, method="pcg")
    xg = to_np(solver.Solve(A, np.zeros(ndof), x))
    Ad = S.stiffness(coor, conn, K, G)
    x_ref = S.solve_partitioned(Ad, iip, xp)
    assert solver.relres <= 1e-12 and solver.iterations > 0
    assert np.array_equal(xg[iip], xp)
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) <= 1e-9
    # the nodevec form and determinism
    xn = np.zeros((mesh.nnode(), 2))
    xn.ravel()[iip] = xp
    x2 = to_np(solver.Solve(A, np.zeros_like(xn), xn))
    assert np.array_equal(x2.ravel(), xg)


def test_reference_matrix_solve(gf):
    """tests/basic/Matrix.cpp "solve": random symmetric element matrices on a 2x2 mesh,
    C = A b, Solve(A, C) recovers b (MINRES: the assembled matrix is indefinite)."""
    rng = np.random.default_rng(50)
    mesh = gf.Mesh.Quad4.Regular(2, 2)
    nelem = mesh.nelem()
    a = rng.uniform(size=(nelem, 8, 8))
    a = 0.5 * (a + np.transpose(a, (0, 2, 1)))
    b = rng.uniform(size=mesh.nnode() * 2)
    A = gf.Matrix(mesh.conn(), mesh.dofs())
    A.assemble(a)
    C = A.Dot(b)
    solver = gf.MatrixSolver(tol=1e-13)
    B = to_np(solver.Solve(A, C))
    assert np.allclose(B, b, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("nodevec", [False, True])
def test_reference_matrix_set_add_dot_solve(gf, oracle, nodevec):
    """tests/basic/Matrix.cpp "set/add/dot/solve": K.set(a) then K.add(a^T) gives A = a + a^T;
    Todense, Dot and Solve (dofval and nodevec)."""
    rng = np.random.default_rng(51)
    a = rng.uniform(size=(10, 10))
    A = a + a.T
    conn = np.zeros((1, 5), dtype=np.int64)
    dofs = np.arange(10).reshape(5, 2)
    K = gf.Matrix(conn, dofs)
    K.set(np.arange(10), np.arange(10), a)
    K.add(np.arange(10), np.arange(10), a.T)
    assert np.allclose(K.Todense(), A, rtol=0, atol=1e-15)
    x = rng.uniform(size=(5, 2) if nodevec else 10)
    b = (A @ x.ravel()).reshape(x.shape)
    assert np.allclose(to_np(K.Dot(x)), b, rtol=1e-14, atol=1e-14)
    solver = gf.MatrixSolver(tol=1e-13)
    assert np.allclose(to_np(solver.Solve(K, b)), x, rtol=1e-8, atol=1e-10)
    # an element assembly afterwards restores the element pattern (here all five local nodes
    # are node 0, as in the reference test)
    em = rng.uniform(size=(1, 10, 10))
    K.assemble(em)
    rp, col, val = oracle.matrix_assemble(conn, dofs, em, 10)
    ref = np.zeros((10, 10))
    ref[np.repeat(np.arange(10), np.diff(rp)), col] = val
    assert np.array_equal(K.Todense(), ref)


def test_matrix_solver_spd_stiffness(gf, oracle):
    """MatrixSolver on an SPD system: the full stiffness plus a stiff spring at the fixed dofs
    (penalty) against a dense solve."""
    from oracle import statics as S

    mesh = gf.Mesh.Quad4.Regular(8, 6)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    Kmat, G = seeded_material(mesh.nelem(), 52)
    Ke = _stiffness_elemmat(oracle, coor, conn, Kmat, G)
    A = gf.Matrix(conn, dofs)
    A.assemble(Ke)
    fixed = dofs[mesh.nodesBottomEdge()].ravel()
    A.add(fixed, fixed, 1e3 * np.eye(fixed.size))
    rng = np.random.default_rng(53)
    b = rng.normal(size=A.ndof())
    solver = gf.MatrixSolver(tol=1e-12)
    x = to_np(solver.Solve(A, b))
    Ad = A.Todense()
    assert np.linalg.norm(Ad @ x - b) <= 1e-11 * np.linalg.norm(b)
    assert np.linalg.norm(x - np.linalg.solve(Ad, b)) <= 1e-8 * np.linalg.norm(x)



@pytest.mark.parametrize("method", ["minres", "pcg"])
def test_matrix_partitioned_solver_methods_agree(gf, oracle, method):
    from oracle import statics as S

    mesh = gf.Mesh.Quad4.Regular(12, 9)
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    K, G = seeded_material(mesh.nelem(), 54)
    bot, top = mesh.nodesBottomEdge(), mesh.nodesTopEdge()
    iip = np.unique(np.concatenate([dofs[bot].ravel(), dofs[top, 1]]))
    xp = np.where(np.isin(iip, dofs[top, 1]), -1e-2, 0.0)
    A = gf.MatrixPartitioned(conn, dofs, iip)
    A.assemble(_stiffness_elemmat(oracle, coor, conn, K, G))
    x = np.zeros(int(dofs.max()) + 1)
    x[iip] = xp
    solver = gf.MatrixPartitionedSolver(tol=1e-12, method=method)
    xg = to_np(solver.Solve(A, np.zeros_like(x), x))
    x_ref = S.solve_partitioned(S.stiffness(coor, conn, K, G), iip, xp)
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) <= 1e-9


@pytest.mark.parametrize("nodevec", [False, True])
def test_reference_matrix_partitioned(gf, nodevec):
    """tests/basic/MatrixParitioned.cpp: random symmetric (indefinite) matrices, "solve" on a
    2x2 mesh with iip = {0, 5, 7, 13} and "set/add/dot/solve" with iip = {0, 2, 4}."""
    rng = np.random.default_rng(55)
    mesh = gf.Mesh.Quad4.Regular(2, 2)
    a = rng.uniform(size=(mesh.nelem(), 8, 8))
    a = 0.5 * (a + np.transpose(a, (0, 2, 1)))
    x = rng.uniform(size=mesh.nnode() * 2)
    A = gf.MatrixPartitioned(mesh.conn(), mesh.dofs(), np.array([0, 5, 7, 13]))
    A.assemble(a)
    b = A.Dot(x)
    xc = to_np(gf.MatrixPartitionedSolver(tol=1e-13).Solve(A, b, x))
    assert np.allclose(xc, x, rtol=1e-8, atol=1e-10)
    # set / add / dot / solve
    a = rng.uniform(size=(10, 10))
    Ad = a + a.T
    conn = np.zeros((1, 5), dtype=np.int64)
    dofs = np.arange(10).reshape(5, 2)
    K = gf.MatrixPartitioned(conn, dofs, np.array([0, 2, 4]))
    K.set(np.arange(10), np.arange(10), a)
    K.add(np.arange(10), np.arange(10), a.T)
    assert np.allclose(K.Todense(), Ad, rtol=0, atol=1e-15)
    xv = rng.uniform(size=(5, 2) if nodevec else 10)
    bv = (Ad @ xv.ravel()).reshape(xv.shape)
    assert np.allclose(to_np(K.Dot(xv)), bv, rtol=1e-14, atol=1e-14)
    assert np.allclose(to_np(gf.MatrixPartitionedSolver(tol=1e-13).Solve(K, bv, xv)), xv,
                       rtol=1e-8, atol=1e-10)
