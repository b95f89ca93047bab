"""The diagonal-only lumped mass (gfgpu_int_n_scalar_nt_dv_diag + assembly through the dof CSR)
against the full Int_N_scalar_NT_dV element matrices (ElementQuad4.h:437-464,
ElementHex8.h:324-352) and MatrixDiagonal(Partitioned)::assemble (MatrixDiagonal.h:151-167,
MatrixDiagonalPartitioned.h:73-98): identical bits in strict mode, the isDiagonal check
(Element.h:122-145) on the fly, and no element-matrix allocation in VelocityVerlet's set-up."""

import numpy as np
import pytest
import torch

from _common import seeded_field, to_np

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    yield gf
    gf.set_strict(False)


def _mesh(gf, elem, distorted):
    if elem == "quad4":
        mesh = gf.Mesh.Quad4.Regular(13, 9)
        E = gf.Element.Quad4
        fixed = mesh.nodesBottomEdge()
    else:
        mesh = gf.Mesh.Hex8.Regular(5, 4, 3)
        E = gf.Element.Hex8
        fixed = mesh.nodesFront()
    coor = mesh.coor()
    if distorted:
        coor = coor + seeded_field(coor.shape, 5, amp=0.1)
    return mesh, E, coor, fixed


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("distorted", [False, True])
@pytest.mark.parametrize("elem", ["quad4", "hex8"])
def test_diag_equals_full_matrix_diagonal(gf, oracle, elem, distorted, strict):
    gf.set_strict(strict)
    mesh, E, coor, fixed = _mesh(gf, elem, distorted)
    conn, dofs = mesh.conn(), mesh.dofs()
    vec = gf.Vector(conn, dofs)
    quad = E.Quadrature(vec.AsElement(coor), E.Nodal.xi(), E.Nodal.w())
    rho = np.random.default_rng(3).uniform(0.5, 2.0, (mesh.nelem(), quad.nip()))
    full = to_np(quad.Int_N_scalar_NT_dV(rho))
    diag = to_np(quad.Int_N_scalar_NT_dV_diag(rho))
    nne, nd = conn.shape[1], coor.shape[1]
    ref = np.einsum("ekk->ek", full).reshape(-1, nne, nd)
    assert np.array_equal(diag, ref)
    # the oracle's element matrices (ElementQuad4.h:437-464 restated)
    R = oracle
    xr = R.as_element(conn, coor)
    xi, w = (R.quad4_nodal() if elem == "quad4" else R.hex8_nodal())
    _, vol = R.compute_dN(xr, xi, w)
    Nr, _ = R.shape(xi)
    Mr = R.int_n_scalar_nt_dv(Nr, vol, rho, nd)
    Dr = np.einsum("ekk->ek", Mr).reshape(-1, nne, nd)
    if strict:
        assert np.array_equal(diag, Dr)
    else:
        assert np.max(np.abs(diag - Dr)) <= 1e-12 * np.max(np.abs(Dr))
    # assembly: MatrixDiagonal and MatrixDiagonalPartitioned
    for M in (gf.MatrixDiagonal(conn, dofs),
              gf.MatrixDiagonalPartitioned(conn, dofs, dofs[fixed, :].ravel())):
        M.assemble(full)
        A_full = to_np(M.data())
        M.assemble_diagonal(diag)
        assert np.array_equal(to_np(M.data()), A_full)
    A_r = R.diag_assemble(conn, dofs, Mr)
    if strict:
        assert np.array_equal(A_full, A_r)


def test_consistent_mass_is_not_diagonal(gf):
    """With the Gauss rule the element mass matrices are full: the on-the-fly isDiagonal check
    refuses them (as MatrixDiagonal::assemble does), and without the check the diagonal is still
    the full matrix's diagonal."""
    gf.set_strict(False)
    mesh, E, coor, _ = _mesh(gf, "quad4", False)
    vec = gf.Vector(mesh.conn(), mesh.dofs())
    quad = E.Quadrature(vec.AsElement(coor))
    rho = np.ones((mesh.nelem(), quad.nip()))
    with pytest.raises(RuntimeError):
        quad.Int_N_scalar_NT_dV_diag(rho)
    with pytest.raises(RuntimeError):
        gf.MatrixDiagonal(mesh.conn(), mesh.dofs()).assemble(quad.Int_N_scalar_NT_dV(rho))
    diag = to_np(quad.Int_N_scalar_NT_dV_diag(rho, check=False))
    full = to_np(quad.Int_N_scalar_NT_dV(rho))
    assert np.array_equal(diag, np.einsum("ekk->ek", full).reshape(diag.shape))


def test_velocity_verlet_setup_forms_no_element_matrices(gf, monkeypatch):
    """The explicit integrator's lumped-mass set-up goes through the diagonal-only integral: the
    full [nelem, nne*ndim, nne*ndim] element matrices (2.1 GB at 2048^2) are never formed."""
    Q = gf.Element.Quad4.Quadrature

    def refuse(self, *args, **kwargs):
        raise AssertionError("element mass matrices formed")

    monkeypatch.setattr(Q, "int_N_scalar_NT_dV", refuse)
    monkeypatch.setattr(Q, "Int_N_scalar_NT_dV", refuse)
    mesh = gf.Mesh.Quad4.Regular(40, 30)
    K = np.full(mesh.nelem(), 1.0)
    G = np.full(mesh.nelem(), 0.5)
    vv = gf.VelocityVerlet(mesh.coor(), mesh.conn(), mesh.dofs(), K, G, dt=0.01, eta=0.1,
                           iip=mesh.dofs()[mesh.nodesBottomEdge(), :].ravel())
    assert vv.desc.ncls >= 3
    # interior / edge / corner lumped masses of a unit-square mesh (0.25 per element corner)
    A = to_np(vv.mass.data())
    assert set(np.unique(A[A > 0]).tolist()) <= {0.25, 0.5, 1.0}
