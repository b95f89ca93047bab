"""Periodic tyings on the GPU (Tyings::Periodic + Control, VectorPartitionedTyings,
MatrixPartitionedTyings, MatrixPartitionedTyingsSolver) against the oracle: asDofs_i bit for
bit, the condensed solve against a direct solve of the condensed system, and the affine
solution of a homogeneous periodic cell under an applied mean shear."""

import numpy as np
import pytest
import torch

from _common import rel_err, seeded_field, seeded_material, to_np

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    yield gf
    gf.set_strict(False)


def _cell(gf, nx, ny):
    mesh = gf.Mesh.Quad4.Regular(nx, ny)
    control = gf.Tyings.Control(mesh.coor(), mesh.dofs())
    coor, dofs = control.coor(), control.dofs()
    cdofs = control.controlDofs()
    iip = np.concatenate([cdofs.ravel(), dofs[mesh.nodesOrigin()].ravel()])
    ty = gf.Tyings.Periodic(coor, dofs, cdofs, mesh.nodesPeriodic(), iip)
    return mesh, control, coor, ty


@pytest.mark.parametrize("strict", [True, False])
def test_as_dofs_i(gf, oracle, strict):
    gf.set_strict(strict)
    mesh, control, coor, ty = _cell(gf, 7, 5)
    vec = gf.VectorPartitionedTyings(mesh.conn(), ty.dofs(), ty.Cdu(), ty.Cdp(), ty.Cdi())
    assert (vec.nnu(), vec.nnp(), vec.nnd()) == (ty.nnu(), ty.nnp(), ty.nnd())
    nv = seeded_field(coor.shape, 40)
    for apply in (True, False):
        got = to_np(vec.asDofs_i(nv, torch.empty(ty.nni(), dtype=torch.float64, device="cuda"),
                                 apply))
        ref = oracle.tyings_as_dofs_i(ty.dofs(), ty.nni(), ty.Cdi().toarray(), nv, apply)
        if strict:
            assert np.array_equal(got, ref)
        else:
            assert rel_err(got, ref) <= 1e-12
    src = seeded_field((ty.nni(),), 41)
    dst = np.zeros(ty.nni())
    out = vec.copy_p(src, dst)
    assert np.array_equal(out[ty.nnu():], src[ty.nnu():]) and not out[:ty.nnu()].any()


def _stiffness(gf, mesh, coor, K, G):
    from oracle import statics as S

    vector = gf.Vector(mesh.conn(), mesh.dofs())
    quad = gf.Element.Quad4.Quadrature(vector.AsElement(coor[:mesh.nnode()]))
    C4 = torch.as_tensor(S.elasticity_tensor(K, G, 4, 2), device="cuda")
    return quad.Int_gradN_dot_tensor4_dot_gradNT_dV(C4)


def test_condensed_solve_vs_direct(gf, oracle):
    from oracle import statics as S

    mesh, control, coor, ty = _cell(gf, 10, 8)
    K, G = seeded_material(mesh.nelem(), 42)
    Ke = _stiffness(gf, mesh, coor, K, G)
    A = gf.MatrixPartitionedTyings(mesh.conn(), ty.dofs(), ty.Cdu(), ty.Cdp())
    A.assemble(Ke)
    # the blocks are index ranges of one CSR assembled in the tyings numbering
    rp, col, val = oracle.matrix_assemble(mesh.conn(), ty.dofs(), to_np(Ke), A.ndof())
    assert np.array_equal(to_np(A.data()[2]), val)
    b = seeded_field(coor.shape, 43, amp=1e-3)
    x = np.zeros(coor.shape)
    x[control.controlNodes()[0], 1] = 0.01  # mean shear F_01
    x[control.controlNodes()[1], 0] = -0.004
    solver = gf.MatrixPartitionedTyingsSolver(tol=1e-12)
    xg = to_np(solver.Solve(A, b, x))
    Ad = np.zeros((A.ndof(), A.ndof()))
    Ad[np.repeat(np.arange(A.ndof()), np.diff(rp)), col] = val
    xr = S.solve_tyings(Ad, ty.dofs(), ty.nnu(), ty.nnp(), ty.Cdi().toarray(), b, x)
    assert solver.relres <= 1e-12 and solver.iterations > 0
    assert np.linalg.norm(xg - xr) / np.linalg.norm(xr) <= 1e-9
    # prescribed entries are untouched
    iip_nodes = ty.dofs() >= ty.nnu()
    indep_p = iip_nodes & (ty.dofs() < ty.nni())
    assert np.array_equal(xg[indep_p], x[indep_p])


def test_homogeneous_cell_is_affine(gf):
    """A homogeneous periodic cell under the mean shear F_01 = 0.02 deforms affinely:
    u_x = 0.02 y, u_y = 0 at every mesh node (origin fixed)."""
    mesh, control, coor, ty = _cell(gf, 9, 7)
    K = np.full(mesh.nelem(), 0.8)
    G = np.full(mesh.nelem(), 0.3)
    Ke = _stiffness(gf, mesh, coor, K, G)
    A = gf.MatrixPartitionedTyings(mesh.conn(), ty.dofs(), ty.Cdu(), ty.Cdp())
    A.assemble(Ke)
    x = np.zeros(coor.shape)
    x[control.controlNodes()[0], 1] = 0.02
    solver = gf.MatrixPartitionedTyingsSolver(tol=1e-13)
    xg = to_np(solver.Solve(A, np.zeros(coor.shape), x))
    n = mesh.nnode()
    ref = np.stack([0.02 * coor[:n, 1], np.zeros(n)], axis=1)
    assert np.abs(xg[:n] - ref).max() <= 1e-11
