"""The reference's own unit tests for the element hot path, run through the GPU implementation:
tests/basic/Element.cpp, ElementQuad4.cpp, ElementHex8.cpp, ElementQuad4Planar.cpp,
MatrixDiagonal.cpp, MatrixDiagonalPartitioned.cpp and Vector.cpp, section by section, with the
reference's expectations (xt::allclose: rtol 1e-5, atol 1e-8; ISCLOSE: abs 1e-12). Exact
expected arrays (the lumped masses) come from the committed golden fixtures."""

import json
import os

import numpy as np
import pytest

from _common import to_np

pytestmark = pytest.mark.gpu

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    return gf


def allclose(a, b):
    return np.allclose(to_np(a), b, rtol=1e-5, atol=1e-8)


# ------------------------------------------------------------------------------- Element.cpp
def test_element_as_tensor_and_allocate(gf):
    """QuadratureBase AsTensor / allocate_q* (tests/basic/Element.cpp:11-35)."""
    mesh = gf.Mesh.Quad4.Regular(3, 1)
    vec = gf.Vector(mesh.conn(), mesh.dofs())
    quad = gf.Element.Quad4.Quadrature(vec.AsElement(mesh.coor()))
    qscalar = np.random.default_rng(0).random((3, 4))
    qtensor = quad.AsTensor(2, qscalar)
    assert tuple(quad.allocate_qscalar().shape) == qscalar.shape
    assert tuple(quad.allocate_qscalar(0.0).shape) == qscalar.shape
    assert tuple(quad.allocate_qtensor(2).shape) == tuple(qtensor.shape) == (3, 4, 2, 2)
    assert tuple(quad.allocate_qtensor(2, 0.0).shape) == tuple(qtensor.shape)
    assert np.array_equal(to_np(qtensor), np.broadcast_to(qscalar[:, :, None, None], (3, 4, 2, 2)))
    out = quad.allocate_qtensor(1, 7.0)
    quad.asTensor(qscalar, out)
    assert np.array_equal(to_np(out), np.broadcast_to(qscalar[:, :, None], (3, 4, 2)))


# ----------------------------------------------------------- ElementQuad4 / Hex8 / Planar.cpp
def _setup(gf, kind, periodic=False):
    if kind == "hex8":
        mesh = gf.Mesh.Hex8.Regular(3, 3, 3)
        elem = gf.Element.Hex8
    else:
        mesh = gf.Mesh.Quad4.Regular(3, 3)
        elem = gf.Element.Quad4
    dofs = mesh.dofsPeriodic() if periodic else mesh.dofs()
    vec = gf.Vector(mesh.conn(), dofs)
    x = vec.AsElement(mesh.coor())
    if kind == "planar":
        quad = elem.QuadraturePlanar(x)
    else:
        quad = elem.Quadrature(x)
    return mesh, vec, quad


KINDS = ["quad4", "hex8", "planar"]


def _affine_disp(mesh, F):
    """disp(n, i) = sum_j F(i, j) coor(n, j), over the mesh's ndim (the reference's loop)."""
    nd = mesh.ndim()
    return mesh.coor() @ F[:nd, :nd].T


@pytest.mark.parametrize("kind", KINDS)
def test_element_gradN_and_dV(gf, kind):
    """Sections "GradN" and "dV": shapes and dV = 0.5^ndim (ElementQuad4.cpp:8-26)."""
    mesh, vec, quad = _setup(gf, kind)
    assert tuple(quad.GradN().shape) == (mesh.nelem(), quad.nip(), mesh.nne(), mesh.ndim())
    assert tuple(quad.dV().shape) == quad.shape_qtensor(0) == quad.shape_qscalar()
    assert allclose(quad.dV(), 0.5 ** mesh.ndim())


@pytest.mark.parametrize("kind", KINDS)
def test_element_interp_quad_vector(gf, kind):
    """Section "InterpQuad_vector": a constant field interpolates to itself, periodic dofs."""
    mesh, vec, quad = _setup(gf, kind, periodic=True)
    uq = quad.InterpQuad_vector(vec.AsElement(vec.allocate_nodevec(1.0)))
    assert allclose(uq, 1.0)


@pytest.mark.parametrize("kind", KINDS)
def test_element_gradients_of_affine_field(gf, kind):
    """Sections "GradN_vector", "GradN_vector_T", "SymGradN_vector": for disp = F . x the
    gradient is F^T, its transpose F, the symmetric gradient EPS, and the dV-weighted average of
    EPS is EPS (ElementQuad4.cpp:41-153)."""
    mesh, vec, quad = _setup(gf, kind)
    td = quad.tdim()
    F = np.zeros((td, td))
    F[0, 1] = 0.1
    EPS = np.zeros((td, td))
    EPS[0, 1] = EPS[1, 0] = 0.05
    ue = vec.AsElement(_affine_disp(mesh, F))
    shape = (mesh.nelem(), quad.nip(), td, td)
    g = quad.GradN_vector(ue)
    gT = quad.GradN_vector_T(ue)
    eps = quad.SymGradN_vector(ue)
    for t in (g, gT, eps):
        assert tuple(t.shape) == shape == quad.shape_qtensor(2)
    assert allclose(g, np.broadcast_to(F.T, shape))
    assert allclose(gT, np.broadcast_to(F, shape))
    assert allclose(eps, np.broadcast_to(EPS, shape))
    dV = to_np(quad.AsTensor(2, quad.dV()))
    assert dV.shape == shape
    epsbar = (to_np(eps) * dV).sum(axis=(0, 1)) / dV.sum(axis=(0, 1))
    assert np.allclose(epsbar, EPS, rtol=1e-5, atol=1e-8)


def test_element_int_N_vector_dV(gf):
    """Section "Int_N_vector_dV" (ElementQuad4.cpp:155-170): a constant body load on the
    periodic unit cell assembles to the same nodal values."""
    mesh, vec, quad = _setup(gf, "quad4", periodic=True)
    qvector = np.empty((mesh.nelem(), quad.nip(), 2))
    qvector[..., 0], qvector[..., 1] = 2.0, 5.0
    nodevec = to_np(vec.AssembleNode(quad.Int_N_vector_dV(qvector)))
    assert np.allclose(nodevec[:, 0], 2.0) and np.allclose(nodevec[:, 1], 5.0)


@pytest.mark.parametrize("kind", KINDS)
def test_element_lumped_mass_periodic(gf, kind):
    """Section "Int_N_scalar_NT_dV": nodal quadrature, rho = 1, periodic dofs -> every diagonal
    entry of the assembled MatrixDiagonal is 1 (ElementQuad4.cpp:172-189)."""
    mesh = gf.Mesh.Hex8.Regular(3, 3, 3) if kind == "hex8" else gf.Mesh.Quad4.Regular(3, 3)
    elem = gf.Element.Hex8 if kind == "hex8" else gf.Element.Quad4
    dofs = mesh.dofsPeriodic()
    vec = gf.Vector(mesh.conn(), dofs)
    mat = gf.MatrixDiagonal(mesh.conn(), dofs)
    x = vec.AsElement(mesh.coor())
    Q = elem.QuadraturePlanar if kind == "planar" else elem.Quadrature
    quad = Q(x, elem.Nodal.xi(), elem.Nodal.w())
    mat.assemble(quad.Int_N_scalar_NT_dV(np.ones((mesh.nelem(), quad.nip()))))
    assert mat.data().numel() == vec.ndof()
    assert allclose(mat.data(), 1.0)


@pytest.mark.parametrize("kind", KINDS)
def test_element_internal_force_of_uniform_strain(gf, kind):
    """Section "Int_gradN_dot_tensor2_dV": a uniform strain gives zero assembled internal force
    on the periodic mesh (ElementQuad4.cpp:191-218)."""
    mesh, vec, quad = _setup(gf, kind, periodic=True)
    td = quad.tdim()
    F = np.zeros((td, td))
    F[0, 1] = 0.1
    eps = quad.SymGradN_vector(vec.AsElement(_affine_disp(mesh, F)))
    Fi = vec.AssembleDofs(quad.Int_gradN_dot_tensor2_dV(eps))
    assert Fi.numel() == vec.ndof()
    assert allclose(Fi, 0.0)


# ----------------------------------------------------- MatrixDiagonal(Partitioned).cpp
def _nodal_mass_elemmat(gf, mesh, vec):
    quad = gf.Element.Quad4.Quadrature(vec.AsElement(mesh.coor()), gf.Element.Quad4.Nodal.xi(),
                                       gf.Element.Quad4.Nodal.w())
    return quad.Int_N_scalar_NT_dV(np.ones((mesh.nelem(), quad.nip())))


@pytest.mark.parametrize("partitioned", [False, True])
def test_matrix_diagonal_assemble(gf, partitioned):
    """Section "assemble": the 2x2 lumped mass (MatrixDiagonal.cpp:12-53,
    MatrixDiagonalPartitioned.cpp:12-54), values from the golden fixture."""
    mesh = gf.Mesh.Quad4.Regular(2, 2)
    iip = np.array([0, 2])
    if partitioned:
        vec = gf.VectorPartitioned(mesh.conn(), mesh.dofs(), iip)
        A = gf.MatrixDiagonalPartitioned(mesh.conn(), mesh.dofs(), iip)
        key = "quad4_2x2_lumped_mass_partitioned"
    else:
        vec = gf.Vector(mesh.conn(), mesh.dofs())
        A = gf.MatrixDiagonal(mesh.conn(), mesh.dofs())
        key = "quad4_2x2_lumped_mass"
    A.assemble(_nodal_mass_elemmat(gf, mesh, vec))
    assert allclose(A.data(), np.array(KAT[key]["value"]))


@pytest.mark.parametrize("partitioned", [False, True])
def test_matrix_diagonal_dot_solve(gf, partitioned):
    """Sections "dot" and "solve" on dofvals (MatrixDiagonal.cpp:55-95,
    MatrixDiagonalPartitioned.cpp:56-97): B = A x, X = A^-1 B with the prescribed entries of X
    taken from x."""
    mesh = gf.Mesh.Quad4.Regular(2, 2)
    iip = np.array([0, 2])
    rng = np.random.default_rng(5)
    a = rng.random(mesh.nnode() * mesh.ndim())
    x = rng.random(mesh.nnode() * mesh.ndim())
    if partitioned:
        A = gf.MatrixDiagonalPartitioned(mesh.conn(), mesh.dofs(), iip)
    else:
        A = gf.MatrixDiagonal(mesh.conn(), mesh.dofs())
    A.set(a)
    B = A.Dot(x)
    assert B.numel() == x.size and allclose(B, a * x) and allclose(A.data(), a)
    X = to_np(A.Solve(B))
    if partitioned:
        X[iip] = x[iip]
    assert np.allclose(X, x, rtol=1e-5, atol=1e-8)


def test_matrix_diagonal_partitioned_variants(gf):
    """The u/p-split entry points (Dot_u, Dot_p, Solve_u, Reaction_p) and the dofval reaction
    against the diagonal restated in numpy (MatrixDiagonalPartitioned.h:234-421)."""
    mesh = gf.Mesh.Quad4.Regular(3, 2)
    dofs = mesh.dofs()
    iip = np.array([1, 4, 7, 8])
    A = gf.MatrixDiagonalPartitioned(mesh.conn(), dofs, iip)
    rng = np.random.default_rng(9)
    a = rng.random(dofs.size) + 0.5
    x = rng.random(dofs.size)
    A.set(a)
    iiu = A.iiu()
    x_u, x_p = x[iiu], x[iip]
    assert np.array_equal(to_np(A.Dot_u(x_u, x_p)), a[iiu] * x_u)
    assert np.array_equal(to_np(A.Dot_p(x_u, x_p)), a[iip] * x_p)
    assert np.array_equal(to_np(A.Reaction_p(x_u, x_p)), a[iip] * x_p)
    assert np.allclose(to_np(A.Solve_u(a[iiu] * x_u, x_p)), x_u, rtol=1e-14, atol=0)
    b = np.full(dofs.size, -3.0)
    r = to_np(A.Reaction(x, b))
    assert np.array_equal(r[iip], a[iip] * x[iip]) and np.all(r[iiu] == -3.0)
    xn = rng.random(dofs.shape)
    r = to_np(A.Reaction(xn, np.zeros_like(xn)))
    isp = np.isin(dofs, iip)
    assert np.array_equal(r[isp], (a[dofs] * xn)[isp]) and np.all(r[~isp] == 0.0)


# ------------------------------------------------------------------------------- Vector.cpp
V_NODE = np.array([[1, 0], [1, 0], [1, 0], [1.5, 0], [1.5, 0], [1.5, 0], [1, 0], [1, 0], [1, 0]])
F_NODE = np.array([[-1, -1], [0, -1], [1, -1], [-1, 0], [0, 0], [1, 0], [-1, 1], [0, 1], [1, 1]],
                  dtype=float)


def _vector_2x2_periodic(gf):
    mesh = gf.Mesh.Quad4.Regular(2, 2)
    return mesh, gf.Vector(mesh.conn(), mesh.dofsPeriodic())


def test_vector_as_dofs_nodevec_and_elemvec(gf):
    """Sections "asDofs - nodevec" and "asDofs - elemvec" (Vector.cpp:11-91)."""
    mesh, vec = _vector_2x2_periodic(gf)
    v = V_NODE.astype(float)
    V = vec.AsDofs(v)
    assert tuple(vec.allocate_dofval().shape) == tuple(V.shape)
    assert tuple(vec.allocate_elemvec().shape) == tuple(vec.AsElement(v).shape)
    assert tuple(vec.allocate_nodevec().shape) == tuple(vec.AsNode(V).shape)
    assert tuple(vec.allocate_elemvec().shape) == tuple(vec.AsElement(V).shape)
    n = (mesh.nnode() - mesh.nodesPeriodic().shape[0]) * mesh.ndim()
    expect = [v[0, 0], v[0, 1], v[1, 0], v[1, 1], v[3, 0], v[3, 1], v[4, 0], v[4, 1]]
    assert V.numel() == n and np.allclose(to_np(V), expect, rtol=0, atol=1e-12)
    V2 = vec.AsDofs(vec.AsElement(vec.AsDofs(v)))
    assert V2.numel() == n and np.allclose(to_np(V2), expect, rtol=0, atol=1e-12)


def test_vector_assemble_dofs_of_periodic_gradient(gf):
    """Sections "asDofs - assembleDofs" / "asDofs - assembleNode" (Vector.cpp:93-166): a nodal
    field antisymmetric across the periodic cell sums to zero on every independent dof."""
    mesh, vec = _vector_2x2_periodic(gf)
    n = (mesh.nnode() - mesh.nodesPeriodic().shape[0]) * mesh.ndim()
    F = vec.AssembleDofs(F_NODE)
    assert F.numel() == n and np.allclose(to_np(F), 0.0, rtol=0, atol=1e-12)
    F = vec.AssembleDofs(vec.AsElement(F_NODE))
    assert F.numel() == n and np.allclose(to_np(F), 0.0, rtol=0, atol=1e-12)


def test_mesh_center_of_gravity(gf):
    """tests/test_Mesh.py test_center_of_gravity: Quad4 Regular(3, 3) -> [1.5, 1.5] (the nodal
    masses through the device lumped-mass path); a Hex8 box likewise."""
    mesh = gf.Mesh.Quad4.Regular(3, 3)
    assert np.allclose(gf.Mesh.center_of_gravity(mesh.coor(), mesh.conn()),
                       KAT["quad4_3x3_center_of_gravity"]["value"])
    h = gf.Mesh.Hex8.Regular(2, 3, 4)
    assert np.allclose(gf.Mesh.center_of_gravity(h.coor(), h.conn()), [1.0, 1.5, 2.0])


def test_matrix_partitioned_reference_python_test(gf):
    """tests/test_MeshPartitioned.py of the reference: MatrixPartitioned and Matrix assembled from
    the same random symmetric element matrices have the same dense form, and
    MatrixPartitionedSolver recovers x from A.Dot(x) with x's prescribed values."""
    mesh = gf.Mesh.Quad4.Regular(2, 2)
    dofs, iip = mesh.dofs(), np.array([0, 5, 7, 13])
    rng = np.random.default_rng(17)
    a = rng.random((mesh.nelem(), 8, 8))
    a = 0.5 * (a + a.transpose(0, 2, 1))
    x = rng.random(mesh.nnode() * 2)
    A = gf.MatrixPartitioned(mesh.conn(), dofs, iip)
    B = gf.Matrix(mesh.conn(), dofs)
    A.assemble(a)
    B.assemble(a)
    assert np.allclose(to_np(A.Todense()), to_np(B.Todense()))
    xc = gf.MatrixPartitionedSolver(tol=1e-13).Solve(A, A.Dot(x), x)
    assert allclose(xc, x)
