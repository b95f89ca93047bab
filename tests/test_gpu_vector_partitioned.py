"""VectorPartitioned on the GPU: the reference's own cases (tests/basic/VectorPartitioned.cpp,
sections "basic", "asDofs", "copy_u, copy_p") and every conversion from / to partitioned storage
against a numpy restatement of the reference's loops (VectorPartitioned.h:176-660) over the
oracle's partition (Mesh::Reorder)."""

import numpy as np
import pytest

from _common import to_np

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    return gf


def _periodic_lr(gf, n=9, seed=0):
    """The reference's 'asDofs' set-up: 9x9 Quad4, right open edge tied to the left one, top and
    bottom edges prescribed; u random with u[right] = u[left]."""
    mesh = gf.Mesh.Quad4.Regular(n, n)
    dofs = mesh.dofs()
    left, right = mesh.nodesLeftOpenEdge(), mesh.nodesRightOpenEdge()
    top, bottom = mesh.nodesTopEdge(), mesh.nodesBottomEdge()
    dofs[right] = dofs[left]
    iip = np.concatenate([dofs[top, 0], dofs[top, 1], dofs[bottom, 0], dofs[bottom, 1]])
    u = np.random.default_rng(seed).standard_normal((mesh.nnode(), mesh.ndim()))
    u[right] = u[left]
    return mesh, dofs, iip, u


def test_basic_dofs_is_p(gf):
    """Section "basic": iip = 0..7 on a 3x3 mesh -> the first four nodes are prescribed."""
    mesh = gf.Mesh.Quad4.Regular(3, 3)
    vec = gf.VectorPartitioned(mesh.conn(), mesh.dofs(), np.arange(8))
    is_p = np.zeros((16, 2), dtype=bool)
    is_p[:4] = True
    assert np.array_equal(vec.dofs_is_p(), is_p)
    assert np.array_equal(vec.dofs_is_u(), ~is_p)


def test_as_dofs_node_from_partitioned(gf):
    """Section "asDofs": NodeFromPartitioned(AsDofs_u(u), AsDofs_p(u)) == u."""
    mesh, dofs, iip, u = _periodic_lr(gf)
    vec = gf.VectorPartitioned(mesh.conn(), dofs, iip)
    u_u, u_p = vec.AsDofs_u(u), vec.AsDofs_p(u)
    assert np.array_equal(to_np(vec.NodeFromPartitioned(u_u, u_p)), u)


def test_copy_u_copy_p(gf):
    """Section "copy_u, copy_p": copying both parts into an empty nodevec reproduces u."""
    import torch

    mesh, dofs, iip, u = _periodic_lr(gf)
    vec = gf.VectorPartitioned(mesh.conn(), dofs, iip)
    v = torch.full(vec.shape_nodevec(), np.nan, dtype=torch.float64, device="cuda")
    vec.copy_u(u, v)
    assert np.array_equal(to_np(v)[vec.dofs_is_u()], u[vec.dofs_is_u()])
    assert np.all(np.isnan(to_np(v)[vec.dofs_is_p()]))
    vec.copy_p(u, v)
    assert np.array_equal(to_np(v), u)
    w = vec.Copy_p(np.zeros_like(u), u)  # returns a new array, u untouched
    assert np.array_equal(to_np(w)[vec.dofs_is_p()], 0 * u[vec.dofs_is_p()])
    assert np.array_equal(to_np(w)[vec.dofs_is_u()], u[vec.dofs_is_u()])


@pytest.mark.parametrize("periodic", [False, True])
def test_partitioned_conversions_match_restatement(gf, oracle, periodic):
    """dofsFromParitioned, nodeFromPartitioned, elementFromPartitioned and asDofs_u/_p of a
    dofval, nodevec and elemvec against the reference's loops restated in numpy (the partition
    itself is the oracle's)."""
    mesh = gf.Mesh.Quad4.Regular(7, 5)
    conn = mesh.conn()
    dofs = mesh.dofsPeriodic() if periodic else mesh.dofs()
    ndof = int(dofs.max()) + 1
    rng = np.random.default_rng(11)
    iip = rng.choice(ndof, 13, replace=False)
    iiu, part = oracle.partition(dofs, iip)
    nnu = iiu.size
    vec = gf.VectorPartitioned(conn, dofs, iip)
    assert np.array_equal(vec.iiu(), iiu)
    u_u, u_p = rng.standard_normal(nnu), rng.standard_normal(iip.size)

    # VectorPartitioned.h:293-314, 344-365, 395-418
    dofval = np.empty(ndof)
    dofval[iiu], dofval[iip] = u_u, u_p
    up = np.concatenate([u_u, u_p])
    assert np.array_equal(to_np(vec.DofsFromParitioned(u_u, u_p)), dofval)
    assert np.array_equal(to_np(vec.NodeFromPartitioned(u_u, u_p)), up[part])
    assert np.array_equal(to_np(vec.ElementFromPartitioned(u_u, u_p)), up[part[conn]])

    # VectorPartitioned.h:428-539 (_u) and 549-660 (_p); last writer wins in the serial loops
    nodevec = rng.standard_normal((mesh.nnode(), 2))
    elemvec = rng.standard_normal((mesh.nelem(), 4, 2))
    for arg, src, tab in ((dofval, dofval, None), (nodevec, nodevec, part),
                          (elemvec, elemvec, part[conn])):
        ref_u, ref_p = np.zeros(nnu), np.zeros(iip.size)
        if tab is None:
            ref_u, ref_p = src[iiu], src[iip]
        else:
            for k, d in zip(src.ravel(), tab.ravel()):
                if d < nnu:
                    ref_u[d] = k
                else:
                    ref_p[d - nnu] = k
        assert np.array_equal(to_np(vec.AsDofs_u(arg)), ref_u)
        assert np.array_equal(to_np(vec.AsDofs_p(arg)), ref_p)


def test_partitioned_shape_errors(gf):
    mesh = gf.Mesh.Quad4.Regular(3, 3)
    vec = gf.VectorPartitioned(mesh.conn(), mesh.dofs(), np.arange(8))
    with pytest.raises(ValueError):
        vec.NodeFromPartitioned(np.zeros(3), np.zeros(8))
    with pytest.raises(ValueError):
        vec.copy_u(np.zeros((16, 2)), np.zeros((15, 2)))
