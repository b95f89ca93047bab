"""CPU-only checks of libgfgpu.so: it loads, exports every entry point of include/gfgpu.h, and
its host-side set-up (GooseFEM Mesh / Vector bookkeeping) is bit-exact with the oracle."""

import json
import os

import numpy as np
import pytest

from _common import seeded_field

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from goosefem_gb300 import _lib

    return _lib


def test_exports_every_declared_symbol(lib):
    L = lib.lib()
    protos = lib.protos()
    assert len(protos) > 40
    for name in protos:
        assert hasattr(L, name), name
    assert lib.lib().gfgpu_version().startswith(b"gfgpu")


def test_binding_covers_every_declaration(lib):
    """Every gfgpu_* prototype of the header is bound with the right number of argument types:
    an unbound entry point would receive 64-bit pointers as 32-bit ints."""
    import re

    text = open(lib.HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = lib.protos()
    declared = re.findall(r"\b(gfgpu_\w+)\s*\(([^;{]*?)\)\s*;", text)
    assert declared
    for name, args in declared:
        assert name in protos, name
        nargs = 0 if args.strip() in ("", "void") else args.count(",") + 1
        assert len(protos[name][1]) == nargs, name
    with pytest.raises(KeyError):
        lib.call("gfgpu_not_declared")
    with pytest.raises(TypeError):
        lib.call("gfgpu_set_strict")


def test_mesh_against_reference_kat(lib):
    import goosefem_gb300 as gf

    m = gf.Mesh.Quad4.Regular(5, 3)
    assert np.array_equal(m.coor(), np.array(KAT["quad4_5x3_coor"]["value"]))
    assert np.array_equal(m.conn(), np.array(KAT["quad4_5x3_conn"]["value"]))
    assert np.array_equal(m.dofs(), np.array(KAT["quad4_5x3_dofs"]["value"]))
    assert np.array_equal(m.nodesPeriodic(), np.array(KAT["quad4_5x3_nodesPeriodic"]["value"]))
    assert np.array_equal(m.dofsPeriodic(), np.array(KAT["quad4_5x3_dofsPeriodic"]["value"]))
    h = gf.Mesh.Hex8.Regular(3, 3, 3)
    assert np.array_equal(h.coor(), np.array(KAT["hex8_3x3x3_coor"]["value"]))
    assert np.array_equal(h.conn(), np.array(KAT["hex8_3x3x3_conn"]["value"]))
    assert np.array_equal(h.nodesFront(), np.array(KAT["hex8_3x3x3_nodesFront"]["value"]))
    assert np.array_equal(h.nodesBack(), np.array(KAT["hex8_3x3x3_nodesBack"]["value"]))
    npr = np.array(KAT["hex8_3x3x3_nodesPeriodic"]["value"])
    assert np.array_equal(h.nodesPeriodic(), npr)
    assert np.array_equal(h.dofsPeriodic(npr), np.array(KAT["hex8_3x3x3_dofsPeriodic"]["value"]))
    assert np.array_equal(h.dofsPeriodic(), np.array(KAT["hex8_3x3x3_dofsPeriodic"]["value"]))
    q = gf.Mesh.Quad4.Regular(3, 3)
    assert np.array_equal(gf.Mesh.coordination(q.conn()),
                          np.array(KAT["quad4_3x3_coordination"]["value"]))
    assert gf.Mesh.elem2node(q.conn()) == KAT["quad4_3x3_elem2node"]["value"]


@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 1), (7, 4), (64, 33)])
def test_mesh_setup_matches_oracle(lib, oracle, nx, ny):
    import goosefem_gb300 as gf

    m = gf.Mesh.Quad4.Regular(nx, ny, 0.37)
    coor, conn = oracle.quad4_regular(nx, ny, 0.37)
    assert np.array_equal(m.coor(), coor) and np.array_equal(m.conn(), conn)
    npr = oracle.quad4_nodes_periodic(nx, ny)
    assert np.array_equal(m.nodesPeriodic(), npr)
    assert np.array_equal(m.dofsPeriodic(), oracle.dofs_periodic(m.nnode(), 2, npr))
    h = gf.Mesh.Hex8.Regular(nx, ny, 3, 0.37)
    hc, hn = oracle.hex8_regular(nx, ny, 3, 0.37)
    assert np.array_equal(h.coor(), hc) and np.array_equal(h.conn(), hn)
    assert np.array_equal(h.nodesPeriodic(), oracle.hex8_nodes_periodic(nx, ny, 3))
    assert np.array_equal(h.dofsPeriodic(),
                          oracle.dofs_periodic(h.nnode(), 3, oracle.hex8_nodes_periodic(nx, ny, 3)))


def test_partition_and_renumber_match_oracle(lib, oracle):
    import goosefem_gb300 as gf

    m = gf.Mesh.Quad4.Regular(11, 7)
    dofs = m.dofsPeriodic()
    rng = np.random.default_rng(3)
    iip = rng.choice(int(dofs.max()) + 1, 17, replace=False)
    iiu, part = gf.Mesh.partition(dofs, iip)
    iiu_r, part_r = oracle.partition(dofs, iip)
    assert np.array_equal(iiu, iiu_r) and np.array_equal(part, part_r)
    a = rng.integers(0, 1000, 500)
    assert np.array_equal(gf.Mesh.renumber(a), oracle.renumber(a))
    with pytest.raises(lib.GFGPUError):
        gf.Mesh.partition(dofs, np.array([1, 1]))  # not unique (GOOSEFEM_ASSERT(is_unique(iip)))


def test_dof_csr_is_the_serial_order(lib, oracle):
    """Summing an elemvec through the dof CSR in segment order reproduces the reference's serial
    assembleDofs bit for bit (checked here on the host with numpy)."""
    from goosefem_gb300 import _dev

    m = oracle.quad4_regular(13, 9)
    conn = m[1]
    dofs = oracle.dofs_periodic(14 * 10, 2, oracle.quad4_nodes_periodic(13, 9))
    ndof = int(dofs.max()) + 1
    ptr, idx = _dev.dof_csr(conn, dofs, ndof)
    ev = seeded_field((conn.shape[0], 4, 2), 31).ravel()
    out = np.zeros(ndof)
    for d in range(ndof):
        acc = 0.0
        for k in range(ptr[d], ptr[d + 1]):
            acc += ev[idx[k]]
        out[d] = acc
    assert np.array_equal(out, oracle.assemble_dofs_elemvec(conn, dofs, ev.reshape(-1, 4, 2)))
    assert all(np.all(np.diff(idx[ptr[d]:ptr[d + 1]]) > 0) for d in range(ndof))


def test_host_errors(lib):
    import goosefem_gb300 as gf

    with pytest.raises(ValueError):
        gf.Mesh.Quad4.Regular(0, 3)
    conn = np.array([[0, 1, 2, 99]], dtype=np.int32)
    dofs = np.arange(8, dtype=np.int32).reshape(4, 2)
    from goosefem_gb300 import _dev

    with pytest.raises(lib.GFGPUError) as ei:
        _dev.dof_csr(conn, dofs, 8)
    assert ei.value.code == -2


def test_unit_element_stiffness_matches_oracle(lib, oracle):
    """The element stiffness behind the energy-norm training loss (host computation in the
    library) against the oracle's element integrals, per unit bulk and per unit shear modulus."""
    from oracle import nn as O

    out = np.zeros(128)
    lib.call("gfgpu_nn_unit_element_stiffness", out.ctypes.data)
    for m, (K, G) in enumerate(((1.0, 0.0), (0.0, 1.0))):
        A = O.crop_stiffness(np.array([[[K, G]]])).toarray()
        # crop nodes (y, x) = (0,0), (0,1), (1,0), (1,1) -> element local nodes 0, 1, 3, 2
        loc = [0, 1, 3, 2]
        perm = [loc.index(a) * 2 + i for a in range(4) for i in range(2)]
        ref = A[np.ix_(perm, perm)]
        got = out[m * 64:(m + 1) * 64].reshape(8, 8)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("periodic", [False, True])
def test_matrix_pattern_matches_oracle(lib, oracle, periodic):
    """gfgpu_host_matrix_pattern (host set-up of the assembled sparse matrix): CSR pattern equal
    to the oracle's, and the per-nonzero triplet lists summed in order give the oracle's values
    bit for bit (Eigen setFromTriplets order), with periodic dofs (repeated dofs in an element)."""
    import ctypes as C

    R = oracle
    nx, ny = 5, 4
    coor, conn = R.quad4_regular(nx, ny)
    nnode = coor.shape[0]
    if periodic:
        dofs = R.dofs_periodic(nnode, 2, R.quad4_nodes_periodic(nx, ny))
    else:
        dofs = R.dofs(nnode, 2)
    ndof = int(dofs.max()) + 1
    rng = np.random.default_rng(4)
    elemmat = rng.normal(size=(conn.shape[0], 8, 8))
    rp_r, col_r, val_r = R.matrix_assemble(conn, dofs, elemmat, ndof)
    total = conn.shape[0] * 64
    rp = np.empty(ndof + 1, dtype=np.int32)
    col = np.empty(total, dtype=np.int32)
    cptr = np.empty(total + 1, dtype=np.int32)
    cidx = np.empty(total, dtype=np.int32)
    nnz = C.c_int64(0)
    c32, d32 = conn.astype(np.int32), dofs.astype(np.int32)
    lib.call("gfgpu_host_matrix_pattern", c32.ctypes.data, d32.ctypes.data, conn.shape[0], 4,
             nnode, 2, ndof, rp.ctypes.data, col.ctypes.data, cptr.ctypes.data, cidx.ctypes.data,
             C.addressof(nnz))
    k = nnz.value
    assert np.array_equal(rp, rp_r) and np.array_equal(col[:k], col_r)
    flat = elemmat.ravel()
    val = np.empty(k)
    for j in range(k):
        idx = cidx[cptr[j]:cptr[j + 1]]
        acc = flat[idx[0]]
        for q in idx[1:]:
            acc = acc + flat[q]
        val[j] = acc
        assert np.all(np.diff(idx) > 0)  # triplet order
    assert np.array_equal(val, val_r)


def test_tyings_setup_matches_oracle(lib, oracle):
    """Tyings::Control + Tyings::Periodic set-up (host, in the library): the renumbering into
    independent-unknown / -prescribed / dependent dofs and the tying matrix C_di, bit for bit
    against the oracle's restatement."""
    import goosefem_gb300 as gf

    mesh = gf.Mesh.Quad4.Regular(5, 4)
    control = gf.Tyings.Control(mesh.coor(), mesh.dofs())
    coor, dofs = control.coor(), control.dofs()
    cdofs = control.controlDofs()
    iip = np.concatenate([cdofs.ravel(), dofs[mesh.nodesOrigin()].ravel()])
    ty = gf.Tyings.Periodic(coor, dofs, cdofs, mesh.nodesPeriodic(), iip)
    d_r, c_r, counts_r, Cdi_r = oracle.tyings_periodic(coor, dofs, cdofs, mesh.nodesPeriodic(), iip)
    assert np.array_equal(ty.dofs(), d_r) and np.array_equal(ty.control(), c_r)
    assert (ty.nnu(), ty.nnp(), ty.nni(), ty.nnd()) == counts_r
    assert np.array_equal(ty.Cdi().toarray(), Cdi_r)
    assert np.array_equal(ty.Cdu().toarray(), Cdi_r[:, :ty.nnu()])
    assert np.array_equal(ty.Cdp().toarray(), Cdi_r[:, ty.nnu():])
    assert ty.nnd() == mesh.nodesPeriodic().shape[0] * 2


@pytest.mark.parametrize("nx,ny,hc", [(512, 512, 16), (37, 30, 8), (5, 3, 7), (1, 1, 1)])
def test_coarse_grid_matches_oracle(lib, nx, ny, hc):
    """gfgpu_coarse_grid (host): coarse node counts, the padded row stride of the dense inverse and
    the reciprocal interval lengths from the coarse coordinates of the oracle's restatement."""
    from goosefem_gb300.learned import CoarseDesc
    from oracle import coarse as OC
    import ctypes as C

    g = CoarseDesc()
    lib.call("gfgpu_coarse_grid", nx, ny, hc, C.addressof(g))
    X, Y = OC.coarse_coords(nx, hc), OC.coarse_coords(ny, hc)
    assert (g.ncx, g.ncy) == (X.size, Y.size)
    nc = 2 * X.size * Y.size
    assert g.ld % 32 == 0 and nc <= g.ld < nc + 32
    assert g.rhx == 1.0 / hc and g.rhy == 1.0 / hc
    assert g.rlx == 1.0 / (X[-1] - X[-2]) and g.rly == 1.0 / (Y[-1] - Y[-2])
    with pytest.raises(lib.GFGPUError):
        lib.call("gfgpu_coarse_grid", nx, ny, 0, C.addressof(g))


def test_mesh_tyings_utilities_against_reference_kat(lib):
    """tests/test_Mesh.py of the reference (Quad4 Regular(4, 4), periodic dofs): coordination of
    the dofs, node2dof, nodaltyings and the periodic elem2node (host set-up)."""
    import goosefem_gb300 as gf

    mesh = gf.Mesh.Quad4.Regular(4, 4)
    dofs = mesh.dofsPeriodic()
    real = np.array(KAT["quad4_4x4_coordination_dofsPeriodic"]["value"]).ravel()
    assert np.array_equal(gf.Mesh.coordination(dofs), real)
    assert gf.Mesh.node2dof(dofs) == KAT["quad4_4x4_node2dof"]["value"]
    assert gf.Mesh.nodaltyings(dofs) == KAT["quad4_4x4_nodaltyings"]["value"]
    real = np.sort(np.array(KAT["quad4_4x4_elem2node_periodic"]["value"]), axis=1)
    assert np.array_equal(np.array(gf.Mesh.elem2node(mesh.conn(), dofs)), real)


def test_quad4_regular_node_sets_reference_python_test(lib):
    """tests/test_MeshQuad4.py test_Regular of the reference: Regular(3, 3) connectivity from the
    node grid, the edges, open edges, corners and their aliases."""
    import goosefem_gb300 as gf

    mesh = gf.Mesh.Quad4.Regular(3, 3)
    nodes = np.arange(16).reshape(4, 4)
    conn = np.hstack([nodes[:-1, :-1].reshape(-1, 1), nodes[:-1, 1:].reshape(-1, 1),
                      nodes[1:, 1:].reshape(-1, 1), nodes[1:, :-1].reshape(-1, 1)])
    x, y = np.meshgrid(np.arange(4.0), np.arange(4.0))
    assert np.allclose(mesh.coor(), np.stack([x.ravel(), y.ravel()], axis=1))
    assert np.array_equal(mesh.conn(), conn)
    assert np.array_equal(mesh.nodesLeftEdge(), nodes[:, 0])
    assert np.array_equal(mesh.nodesRightEdge(), nodes[:, -1])
    assert np.array_equal(mesh.nodesBottomEdge(), nodes[0, :])
    assert np.array_equal(mesh.nodesTopEdge(), nodes[-1, :])
    assert np.array_equal(mesh.nodesLeftOpenEdge(), mesh.nodesLeftEdge()[1:-1])
    assert np.array_equal(mesh.nodesRightOpenEdge(), mesh.nodesRightEdge()[1:-1])
    assert np.array_equal(mesh.nodesBottomOpenEdge(), mesh.nodesBottomEdge()[1:-1])
    assert np.array_equal(mesh.nodesTopOpenEdge(), mesh.nodesTopEdge()[1:-1])
    assert mesh.nodesBottomLeftCorner() == mesh.nodesBottomEdge()[0]
    assert mesh.nodesBottomRightCorner() == mesh.nodesBottomEdge()[-1]
    assert mesh.nodesTopLeftCorner() == mesh.nodesTopEdge()[0]
    assert mesh.nodesTopRightCorner() == mesh.nodesTopEdge()[-1]
    assert mesh.nodesLeftBottomCorner() == mesh.nodesBottomLeftCorner()
    assert mesh.nodesRightBottomCorner() == mesh.nodesBottomRightCorner()
    assert mesh.nodesLeftTopCorner() == mesh.nodesTopLeftCorner()
    assert mesh.nodesRightTopCorner() == mesh.nodesTopRightCorner()
