"""GooseFEM.Tyings (Periodic, Control), VectorPartitionedTyings, MatrixPartitionedTyings and
MatrixPartitionedTyingsSolver on the GPU (mirror of TyingsPeriodic.h, VectorPartitionedTyings.h,
MatrixPartitionedTyings.h).

The tying set-up (renumbering into independent-unknown, independent-prescribed and dependent
dofs, and the tying matrix C_di) is host integer / small sparse work done by the library
(gfgpu_host_tyings_*); the tying matrices are returned as scipy.sparse CSR matrices where the
reference returns Eigen sparse matrices. The solver applies the condensed operator of
MatrixPartitionedTyingsSolver matrix-free on the device (gfgpu_tyings_solve).
"""

import ctypes as C

import numpy as np
import torch

from . import _dev, _lib
from .matrix import Matrix
from .vector import Vector


def _csr(rowptr, col, val, shape):
    import scipy.sparse as sp

    return sp.csr_matrix((val, col, rowptr), shape=shape)


def _transpose(rowptr, col, val, nrow, ncol):
    trow = np.empty(ncol + 1, dtype=np.int32)
    tcol = np.empty(max(col.size, 1), dtype=np.int32)
    tval = np.empty(max(col.size, 1))
    _lib.call("gfgpu_host_csr_transpose", rowptr.ctypes.data, col.ctypes.data, val.ctypes.data,
              nrow, ncol, trow.ctypes.data, tcol.ctypes.data, tval.ctypes.data)
    return trow, tcol[:col.size].copy(), tval[:col.size].copy()


class Control:
    """Tyings::Control(coor, dofs) (TyingsPeriodic.h:356-437): ndim control nodes (coordinates
    0) whose ndim x ndim dofs follow the existing ones."""

    def __init__(self, coor, dofs):
        coor = np.asarray(coor, dtype=np.float64)
        dofs = np.asarray(dofs, dtype=np.int64)
        if coor.ndim != 2 or coor.shape != dofs.shape:
            raise ValueError("coor and dofs must have the same 2-d shape")
        nnode, ndim = coor.shape
        self._control_dofs = np.arange(ndim * ndim, dtype=np.int64).reshape(ndim, ndim) + dofs.max() + 1
        self._control_nodes = nnode + np.arange(ndim, dtype=np.int64)
        self._coor = np.concatenate([coor, np.zeros((ndim, ndim))])
        self._dofs = np.concatenate([dofs, self._control_dofs])

    def coor(self):
        return self._coor.copy()

    def dofs(self):
        return self._dofs.copy()

    def controlDofs(self):
        return self._control_dofs.copy()

    def controlNodes(self):
        return self._control_nodes.copy()


class Periodic:
    """Tyings::Periodic(coor, dofs, control_dofs, nodal_tyings[, iip]) (TyingsPeriodic.h:46-344).
    nodal_tyings [ntyings, 2] = (independent node, dependent node)."""

    def __init__(self, coor, dofs, control_dofs, nodal_tyings, iip=None):
        self._coor = np.ascontiguousarray(coor, dtype=np.float64)
        d = _dev.host_i32(dofs)
        ctrl = _dev.host_i32(control_dofs)
        ty = _dev.host_i32(nodal_tyings).reshape(-1, 2)
        iip = _dev.host_i32(np.zeros(0) if iip is None else iip).ravel()
        nnode, ndim = d.shape
        if self._coor.shape != d.shape or ctrl.shape != (ndim, ndim):
            raise ValueError("shape mismatch")
        self._ndim, self._nties = ndim, ty.shape[0]
        self._tyings = ty
        self._dofs = np.empty_like(d)
        self._control = np.empty_like(ctrl)
        counts = np.zeros(4, dtype=np.int64)
        _lib.call("gfgpu_host_tyings_periodic", d.ctypes.data, nnode, ndim, ctrl.ctypes.data,
                  ty.ctypes.data, ty.shape[0], iip.ctypes.data, iip.size, self._dofs.ctypes.data,
                  self._control.ctypes.data, counts.ctypes.data)
        self._nnu, self._nnp, self._nni, self._nnd = (int(c) for c in counts)
        cap = max(self._nties * ndim * (ndim + 1), 1)
        rowptr = np.empty(self._nnd + 1, dtype=np.int32)
        col = np.empty(cap, dtype=np.int32)
        val = np.empty(cap)
        nnz = C.c_int64(0)
        _lib.call("gfgpu_host_tyings_cdi", self._coor.ctypes.data, self._dofs.ctypes.data,
                  self._control.ctypes.data, ty.ctypes.data, self._nties, ndim,
                  rowptr.ctypes.data, col.ctypes.data, val.ctypes.data, C.addressof(nnz))
        k = int(nnz.value)
        self._cdi = (rowptr, col[:k].copy(), val[:k].copy())

    def nnd(self):
        return self._nnd

    def nni(self):
        return self._nni

    def nnu(self):
        return self._nnu

    def nnp(self):
        return self._nnp

    def dofs(self):
        return self._dofs.copy()

    def control(self):
        return self._control.copy()

    def nodal_tyings(self):
        return self._tyings.copy()

    def iid(self):
        return np.arange(self._nni, self._nni + self._nnd)

    def iii(self):
        return np.arange(self._nni)

    def iiu(self):
        return np.arange(self._nnu)

    def iip(self):
        return np.arange(self._nnu, self._nnu + self._nnp)

    def Cdi(self):
        return _csr(*self._cdi, shape=(self._nnd, self._nni))

    def Cdu(self):
        return self.Cdi()[:, :self._nnu].tocsr()

    def Cdp(self):
        return self.Cdi()[:, self._nnu:].tocsr()


def _tying_tables(Cdu, Cdp):
    """Device CSR of C_di = [C_du | C_dp] and of its transpose C_id."""
    import scipy.sparse as sp

    Cdi = sp.hstack([Cdu, Cdp]).tocsr()
    Cdi.sort_indices()
    nnd, nni = Cdi.shape
    rp = Cdi.indptr.astype(np.int32)
    col = Cdi.indices.astype(np.int32)
    val = Cdi.data.astype(np.float64)
    trp, tcol, tval = _transpose(rp, col, val, nnd, nni)
    dev = _dev.device()
    t = lambda a: torch.as_tensor(a, device=dev)  # noqa: E731
    return (t(rp), t(col), t(val)), (t(trp), t(tcol), t(tval))


class VectorPartitionedTyings(Vector):
    """VectorPartitionedTyings(conn, dofs, Cdu, Cdp, Cdi) (VectorPartitionedTyings.h:32-252);
    dofs: the renumbered Tyings::Periodic::dofs()."""

    def __init__(self, conn, dofs, Cdu, Cdp, Cdi=None):
        super().__init__(conn, dofs)
        self._nnu, self._nnp, self._nnd = Cdu.shape[1], Cdp.shape[1], Cdp.shape[0]
        self._nni = self._nnu + self._nnp
        if self._ndof != self._nni + self._nnd:
            raise ValueError("dofs do not match the tying matrices")
        (self._cdi, self._cid) = _tying_tables(Cdu, Cdp)
        self.tdofs = self.dofs_d.view(-1)
        self._work = torch.empty(max(self._nnd, 1), dtype=torch.float64, device=_dev.device())

    def nnd(self):
        return self._nnd

    def nni(self):
        return self._nni

    def nnu(self):
        return self._nnu

    def nnp(self):
        return self._nnp

    def iid(self):
        return np.arange(self._nni, self._nni + self._nnd)

    def iii(self):
        return np.arange(self._nni)

    def iiu(self):
        return np.arange(self._nnu)

    def iip(self):
        return np.arange(self._nnu, self._nni)

    def copy_p(self, dofval_src, dofval_dest):
        """VectorPartitionedTyings::copy_p (:146-160)."""
        dofval_dest[self._nnu:self._nni] = dofval_src[self._nnu:self._nni]
        return dofval_dest

    def asDofs_i(self, nodevec, dofval_i, apply_tyings=True):
        """VectorPartitionedTyings::asDofs_i (:208-239)."""
        nv = _dev.dev_f64(nodevec)
        _dev.check_shape(nv, (self._nnode, self._ndim), "asDofs_i")
        _dev.check_shape(dofval_i, (self._nni,), "asDofs_i")
        _lib.call("gfgpu_tyings_as_dofs_i", self.tdofs.data_ptr(), self._nnode, self._ndim,
                  self._nni, self._nnd, self._cid[0].data_ptr(), self._cid[1].data_ptr(),
                  self._cid[2].data_ptr(), nv.data_ptr(), int(bool(apply_tyings)),
                  dofval_i.data_ptr(), self._work.data_ptr(), _dev.stream())
        return dofval_i

    def AsDofs_i(self, nodevec):
        out = torch.empty(self._nni, dtype=torch.float64, device=_dev.device())
        return self.asDofs_i(nodevec, out)


class MatrixPartitionedTyings(Matrix):
    """MatrixPartitionedTyings(conn, dofs, Cdu, Cdp) (MatrixPartitionedTyings.h): one CSR in the
    tyings numbering [u, p, d]; its nine blocks are index ranges."""

    def __init__(self, conn, dofs, Cdu, Cdp):
        self._conn_h = _dev.host_i32(conn)
        self._dofs_h = _dev.host_i32(dofs)
        self._nelem, self._nne = self._conn_h.shape
        self._nnode, self._ndim = self._dofs_h.shape
        self._nnu, self._nnp, self._nnd = Cdu.shape[1], Cdp.shape[1], Cdp.shape[0]
        self._nni = self._nnu + self._nnp
        self._ndof = self._nni + self._nnd
        if int(self._dofs_h.max()) + 1 != self._ndof:
            raise ValueError("dofs do not match the tying matrices")
        self._setup(self._dofs_h)
        (self._cdi, self._cid) = _tying_tables(Cdu, Cdp)
        self.tdofs = _dev.dev_i32(self._dofs_h).view(-1)

    def nnu(self):
        return self._nnu

    def nnp(self):
        return self._nnp

    def nnd(self):
        return self._nnd

    def nni(self):
        return self._nni


class MatrixPartitionedTyingsSolver:
    """MatrixPartitionedTyingsSolver (MatrixPartitionedTyings.h): solve(A, b, x) on nodevec
    b, x; the reference factorises the condensed matrix (Eigen SimplicialLDLT); here a
    Jacobi-PCG on the condensed operator in FP64 to a relative residual `tol`."""

    def __init__(self, tol=1e-12, maxiter=1000000, check_every=16):
        self.tol, self.maxiter, self.check_every = float(tol), int(maxiter), int(check_every)
        self.iterations = 0
        self.relres = 0.0

    def solve(self, A, b, x):
        bd = _dev.dev_f64(b).contiguous()
        _dev.check_shape(bd, (A._nnode, A._ndim), "solve")
        _dev.check_shape(x, (A._nnode, A._ndim), "solve")
        nb = int(_lib.lib().gfgpu_tyings_solve_workspace_bytes(A._nnu, A._nnp, A._nnd))
        ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=_dev.device())
        it, rel = C.c_int64(0), C.c_double(0.0)
        _lib.call("gfgpu_tyings_solve", A.rowptr.data_ptr(), A.col.data_ptr(), A._val.data_ptr(),
                  A._cdi[0].data_ptr(), A._cdi[1].data_ptr(), A._cdi[2].data_ptr(),
                  A._cid[0].data_ptr(), A._cid[1].data_ptr(), A._cid[2].data_ptr(),
                  A.tdofs.data_ptr(), A._nnode, A._ndim, A._nnu, A._nnp, A._nnd, bd.data_ptr(),
                  x.data_ptr(), self.tol, self.maxiter, self.check_every, ws.data_ptr(),
                  _dev.stream(), C.addressof(it), C.addressof(rel))
        self.iterations, self.relres = int(it.value), float(rel.value)
        return x

    def Solve(self, A, b, x):
        x = _dev.dev_f64(x).clone()
        return self.solve(A, b, x)
