"""GooseFEM.Mesh subset on the element hot path: Regular Quad4/Hex8 meshes and DOF bookkeeping.

Mirrors include/GooseFEM/Mesh.h, MeshQuad4.h and MeshHex8.h of the reference. Mesh tables
are host (numpy) arrays, as in the reference; the integer work runs in libgfgpu.so
(gfgpu_host_*), bit-exact with the reference.
"""

import numpy as np

from . import _lib


def dofs(nnode, ndim):
    """Mesh::dofs (Mesh.h:93-96)."""
    out = np.empty((nnode, ndim), dtype=np.int32)
    _lib.call("gfgpu_host_dofs", nnode, ndim, out.ctypes.data)
    return out


def renumber(a):
    """Mesh::renumber (Mesh.h:114-175)."""
    a = np.ascontiguousarray(a, dtype=np.int32)
    out = np.empty_like(a)
    _lib.call("gfgpu_host_renumber", a.ctypes.data, a.size, out.ctypes.data)
    return out


def coordination(conn, nnode=None):
    """Mesh::coordination (Mesh.h:2462-2477)."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nnode = int(conn.max()) + 1 if nnode is None else nnode
    out = np.empty(nnode, dtype=np.int32)
    _lib.call("gfgpu_host_coordination", conn.ctypes.data, conn.shape[0], conn.shape[1], nnode,
              out.ctypes.data)
    return out


def elem2node(conn, dofs=None, nnode=None):
    """Mesh::elem2node, sorted (Mesh.h:2485-2513): list of element lists per node. With `dofs`
    (Mesh.h:2517-2548) the lists of nodes tied by periodicity (nodes sharing their dofs) are
    merged, sorted, and given to every node of the tie."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    if dofs is not None and nnode is None:
        nnode = np.asarray(dofs).shape[0]
    nnode = int(conn.max()) + 1 if nnode is None else nnode
    ptr = np.empty(nnode + 1, dtype=np.int32)
    idx = np.empty(conn.size, dtype=np.int32)
    _lib.call("gfgpu_host_elem2node", conn.ctypes.data, conn.shape[0], conn.shape[1], nnode,
              ptr.ctypes.data, idx.ctypes.data)
    ret = [list(idx[ptr[i]:ptr[i + 1]]) for i in range(nnode)]
    if dofs is None:
        return ret
    ties = nodaltyings(dofs)
    for m in range(nnode):
        t = ties[m]
        if len(t) <= 1 or m > t[0]:
            continue
        merged = sorted(ret[m] + [e for j in t[1:] for e in ret[j]])
        ret[m] = merged
        for j in t[1:]:
            ret[j] = list(merged)
    return ret


def node2dof(dofs):
    """Mesh::node2dof (Mesh.h:2557-2560): the nodes of every dof, sorted."""
    return elem2node(dofs)


def nodaltyings(dofs):
    """Mesh::nodaltyings (Mesh.h:2840-2862): for every node the sorted list of nodes that share
    its dofs (itself included)."""
    d = np.asarray(dofs)
    nodemap = node2dof(d)
    return [sorted(nodemap[int(d[m, 0])]) for m in range(d.shape[0])]


def nodal_mass(coor, conn):
    """Mesh::nodal_mass (Mesh.h:2708-2752): lumped mass of unit density per node and component,
    through the device path (nodal quadrature, Int_N_scalar_NT_dV, MatrixDiagonal)."""
    from .element import Hex8 as _H, Quad4 as _Q
    from .matrix import MatrixDiagonal
    from .vector import Vector

    coor = np.asarray(coor, dtype=np.float64)
    conn = np.asarray(conn)
    d = dofs(coor.shape[0], coor.shape[1])
    E = {(4, 2): _Q, (8, 3): _H}.get((conn.shape[1], coor.shape[1]))
    if E is None:
        raise RuntimeError("Element-type not implemented")
    vec = Vector(conn, d)
    quad = E.Quadrature(vec.AsElement(coor), E.Nodal.xi(), E.Nodal.w())
    M = MatrixDiagonal(conn, d)
    M.assemble_diagonal(quad.Int_N_scalar_NT_dV_diag(np.ones(conn.shape)))
    return vec.AsNode(M.data())


def center_of_gravity(coor, conn):
    """Mesh::center_of_gravity (Mesh.h:2826-2831): the mass-weighted average of the nodal
    coordinates (unit density)."""
    coor = np.asarray(coor, dtype=np.float64)
    w = nodal_mass(coor, conn).cpu().numpy()
    return (coor * w).sum(axis=0) / w.sum(axis=0)


def partition(dofs_, iip):
    """iiu = setdiff1d(dofs, iip), part = Reorder({iiu, iip}).apply(dofs)
    (VectorPartitioned.h:72-88, Mesh.h:2384-2450). Returns (iiu, part)."""
    d = np.ascontiguousarray(dofs_, dtype=np.int32)
    iip = np.ascontiguousarray(iip, dtype=np.int32)
    iiu = np.empty(d.size, dtype=np.int32)
    part = np.empty_like(d)
    nnu = np.zeros(1, dtype=np.int64)
    _lib.call("gfgpu_host_partition", d.ctypes.data, d.size, iip.ctypes.data, iip.size,
              iiu.ctypes.data, part.ctypes.data, nnu.ctypes.data)
    return iiu[: int(nnu[0])].copy(), part


class _RegularBase:
    def nelem(self):
        return self._nelem

    def nnode(self):
        return self._nnode

    def nne(self):
        return self._nne

    def ndim(self):
        return self._ndim

    def nelx(self):
        return self._nx

    def nely(self):
        return self._ny

    def h(self):
        return self._h

    def dofs(self):
        return dofs(self._nnode, self._ndim)


class Quad4:
    class Regular(_RegularBase):
        """Mesh::Quad4::Regular (MeshQuad4.h:32-195)."""

        def __init__(self, nelx, nely, h=1.0):
            if nelx < 1 or nely < 1:
                raise ValueError("nelx, nely must be >= 1")
            self._nx, self._ny, self._h = int(nelx), int(nely), float(h)
            self._nne, self._ndim = 4, 2
            self._nnode = (self._nx + 1) * (self._ny + 1)
            self._nelem = self._nx * self._ny
            self._coor = None

        def _build(self):
            if self._coor is None:
                self._coor = np.empty((self._nnode, 2))
                self._conn = np.empty((self._nelem, 4), dtype=np.int32)
                _lib.call("gfgpu_host_quad4_regular", self._nx, self._ny, self._h,
                          self._coor.ctypes.data, self._conn.ctypes.data)

        def coor(self):
            self._build()
            return self._coor.copy()

        def conn(self):
            self._build()
            return self._conn.copy()

        def nodesBottomEdge(self):
            return np.arange(self._nx + 1, dtype=np.int32)

        def nodesTopEdge(self):
            return (np.arange(self._nx + 1) + self._ny * (self._nx + 1)).astype(np.int32)

        def nodesLeftEdge(self):
            return (np.arange(self._ny + 1) * (self._nx + 1)).astype(np.int32)

        def nodesRightEdge(self):
            return (np.arange(self._ny + 1) * (self._nx + 1) + self._nx).astype(np.int32)

        def nodesBottomOpenEdge(self):
            """Bottom edge without corners (MeshQuad4.h:148-151)."""
            return np.arange(1, self._nx, dtype=np.int32)

        def nodesTopOpenEdge(self):
            return (np.arange(1, self._nx) + self._ny * (self._nx + 1)).astype(np.int32)

        def nodesLeftOpenEdge(self):
            return (np.arange(1, self._ny) * (self._nx + 1)).astype(np.int32)

        def nodesRightOpenEdge(self):
            return (np.arange(1, self._ny) * (self._nx + 1) + self._nx).astype(np.int32)

        def nodesBottomLeftCorner(self):
            return 0

        def nodesBottomRightCorner(self):
            return self._nx

        def nodesTopLeftCorner(self):
            return self._ny * (self._nx + 1)

        def nodesTopRightCorner(self):
            return self._ny * (self._nx + 1) + self._nx

        # the reference's aliases (Mesh.h:466-500)
        nodesLeftBottomCorner = nodesBottomLeftCorner
        nodesLeftTopCorner = nodesTopLeftCorner
        nodesRightBottomCorner = nodesBottomRightCorner
        nodesRightTopCorner = nodesTopRightCorner

        def nodesOrigin(self):
            return 0

        def nodesPeriodic(self):
            """RegularBase2d::nodesPeriodic (Mesh.h:511-540)."""
            out = np.empty(((self._nx - 1) + (self._ny - 1) + 3, 2), dtype=np.int32)
            n = np.zeros(1, dtype=np.int64)
            _lib.call("gfgpu_host_quad4_nodes_periodic", self._nx, self._ny, out.ctypes.data,
                      n.ctypes.data)
            return out[: int(n[0])].copy()

        def dofsPeriodic(self):
            """RegularBase::dofsPeriodic (Mesh.h:291-306)."""
            npr = self.nodesPeriodic()
            out = np.empty((self._nnode, 2), dtype=np.int32)
            _lib.call("gfgpu_host_dofs_periodic", self._nnode, 2, npr.ctypes.data, npr.shape[0],
                      out.ctypes.data)
            return out


class Hex8:
    class Regular(_RegularBase):
        """Mesh::Hex8::Regular (MeshHex8.h:26-608)."""

        def __init__(self, nelx, nely, nelz, h=1.0):
            if nelx < 1 or nely < 1 or nelz < 1:
                raise ValueError("nelx, nely, nelz must be >= 1")
            self._nx, self._ny, self._nz, self._h = int(nelx), int(nely), int(nelz), float(h)
            self._nne, self._ndim = 8, 3
            self._nnode = (self._nx + 1) * (self._ny + 1) * (self._nz + 1)
            self._nelem = self._nx * self._ny * self._nz
            self._coor = None

        def nelz(self):
            return self._nz

        def _build(self):
            if self._coor is None:
                self._coor = np.empty((self._nnode, 3))
                self._conn = np.empty((self._nelem, 8), dtype=np.int32)
                _lib.call("gfgpu_host_hex8_regular", self._nx, self._ny, self._nz, self._h,
                          self._coor.ctypes.data, self._conn.ctypes.data)

        def coor(self):
            self._build()
            return self._coor.copy()

        def conn(self):
            self._build()
            return self._conn.copy()

        def nodesFront(self):
            """z = 0 face (MeshHex8.h:133-144)."""
            return np.arange((self._nx + 1) * (self._ny + 1), dtype=np.int32)

        def nodesBack(self):
            """z = top face (MeshHex8.h:146-158)."""
            n = (self._nx + 1) * (self._ny + 1)
            return (np.arange(n) + self._nz * n).astype(np.int32)

        def _grid(self):
            nx, ny, nz = self._nx + 1, self._ny + 1, self._nz + 1
            return np.arange(nx * ny * nz, dtype=np.int32).reshape(nz, ny, nx)

        def nodesLeft(self):
            """x = 0 face, iz outer, iy inner (MeshHex8.h:160-171)."""
            return self._grid()[:, :, 0].ravel().copy()

        def nodesRight(self):
            """x = top face (MeshHex8.h:173-185)."""
            return self._grid()[:, :, -1].ravel().copy()

        def nodesBottom(self):
            """y = 0 face, iz outer, ix inner (MeshHex8.h:187-198)."""
            return self._grid()[:, 0, :].ravel().copy()

        def nodesTop(self):
            """y = top face (MeshHex8.h:200-212)."""
            return self._grid()[:, -1, :].ravel().copy()

        def nodesOrigin(self):
            return 0

        def nodesPeriodic(self):
            """RegularBase3d::nodesPeriodic (Mesh.h:1577-1692)."""
            nx, ny, nz = self._nx, self._ny, self._nz
            n = 7 + 3 * (nx - 1 + ny - 1 + nz - 1) + (nx - 1) * (ny - 1) + (ny - 1) * (nz - 1) \
                + (nx - 1) * (nz - 1)
            out = np.empty((n, 2), dtype=np.int32)
            k = np.zeros(1, dtype=np.int64)
            _lib.call("gfgpu_host_hex8_nodes_periodic", nx, ny, nz, out.ctypes.data, k.ctypes.data)
            return out[: int(k[0])].copy()

        def dofsPeriodic(self, nodes_periodic=None):
            """RegularBase::dofsPeriodic (Mesh.h:291-306); `nodes_periodic` defaults to
            nodesPeriodic()."""
            if nodes_periodic is None:
                nodes_periodic = self.nodesPeriodic()
            npr = np.ascontiguousarray(nodes_periodic, dtype=np.int32)
            out = np.empty((self._nnode, 3), dtype=np.int32)
            _lib.call("gfgpu_host_dofs_periodic", self._nnode, 3, npr.ctypes.data, npr.shape[0],
                      out.ctypes.data)
            return out
