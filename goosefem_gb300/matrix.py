"""GooseFEM.MatrixDiagonal / MatrixDiagonalPartitioned on the GPU (mirror of
include/GooseFEM/MatrixDiagonal.h and MatrixDiagonalPartitioned.h).

The diagonal is assembled through a dof-centric CSR (the reference's serial order, bit-exact);
the inverse is recomputed lazily on the next solve after a change (MatrixDiagonal.h:268-280).
"""

import numpy as np
import torch

from . import _dev, _lib
from . import mesh as _mesh
from .element import isDiagonal


class MatrixDiagonal:
    """MatrixDiagonal(conn, dofs) (MatrixDiagonal.h:133-147)."""

    def __init__(self, conn, dofs):
        self._conn_h = _dev.host_i32(conn)
        self._dofs_h = _dev.host_i32(dofs)
        self._nelem, self._nne = self._conn_h.shape
        self._nnode, self._ndim = self._dofs_h.shape
        self._ndof = int(self._dofs_h.max()) + 1
        self.conn_d = _dev.dev_i32(self._conn_h)
        self.dofs_d = _dev.dev_i32(self._dofs_h)
        p, i = _dev.dof_csr(self._conn_h, self._dofs_h, self._ndof)
        self.csr_ptr, self.csr_idx = _dev.dev_i32(p), _dev.dev_i32(i)
        self._A = _dev.empty((self._ndof,))
        self._inv = _dev.empty((self._ndof,))
        self._changed = True

    def nelem(self):
        return self._nelem

    def nne(self):
        return self._nne

    def nnode(self):
        return self._nnode

    def ndim(self):
        return self._ndim

    def ndof(self):
        return self._ndof

    def dofs(self):
        return self._dofs_h.copy()

    def conn(self):
        return self._conn_h.copy()

    def shape_elemmat(self):
        k = self._nne * self._ndim
        return (self._nelem, k, k)

    def assemble(self, elemmat):
        """MatrixDiagonal::assemble (MatrixDiagonal.h:151-167)."""
        em = _dev.dev_f64(elemmat)
        _dev.check_shape(em, self.shape_elemmat(), "assemble")
        if not isDiagonal(em):
            raise RuntimeError("MatrixDiagonal::assemble: elemmat is not diagonal")
        _lib.call("gfgpu_diag_assemble", self.csr_ptr.data_ptr(), self.csr_idx.data_ptr(),
                  self._ndof, self._nne, self._ndim, em.data_ptr(), self._A.data_ptr(),
                  _dev.stream())
        self._changed = True

    def assemble_diagonal(self, elemvec):
        """MatrixDiagonal::assemble from the element matrices' diagonals only (an elemvec, e.g.
        Quadrature.Int_N_scalar_NT_dV_diag): the same sums in the same order as assemble()."""
        ev = _dev.dev_f64(elemvec)
        _dev.check_shape(ev, (self._nelem, self._nne, self._ndim), "assemble_diagonal")
        ptr, idx, out = self._assemble_target()
        _lib.call("gfgpu_assemble_dofs", ptr.data_ptr(), idx.data_ptr(), self._ndof, ev.data_ptr(),
                  out.data_ptr(), _dev.stream())
        self._changed = True

    def _assemble_target(self):
        return self.csr_ptr, self.csr_idx, self._A

    def set(self, A):
        A = _dev.dev_f64(A)
        _dev.check_shape(A, (self._ndof,), "set")
        self._A.copy_(A)
        self._changed = True

    def data(self):
        return self._A

    def Todense(self):
        return torch.diag(self._A)

    def _factorize(self):
        if self._changed:
            _lib.call("gfgpu_diag_factorize", self._A.data_ptr(), self._ndof, self._inv.data_ptr(),
                      _dev.stream())
            self._changed = False

    def inverse(self):
        self._factorize()
        return self._inv

    def dot(self, x, b):
        x = _dev.dev_f64(x)
        if x.dim() == 2:
            _lib.call("gfgpu_diag_dot_nodevec", self.dofs_d.data_ptr(), self._nnode, self._ndim,
                      self._A.data_ptr(), x.data_ptr(), b.data_ptr(), _dev.stream())
        else:
            _lib.call("gfgpu_dofval_mul", self._A.data_ptr(), x.data_ptr(), self._ndof,
                      b.data_ptr(), _dev.stream())
        return b

    def Dot(self, x):
        x = _dev.dev_f64(x)
        return self.dot(x, torch.empty_like(x))

    def solve(self, b, x):
        """MatrixDiagonal::solve (MatrixDiagonal.h:237-259)."""
        b = _dev.dev_f64(b)
        self._factorize()
        if b.dim() == 2:
            _lib.call("gfgpu_diag_solve_nodevec", self.dofs_d.data_ptr(), self._nnode, self._ndim,
                      self._ndof, self._inv.data_ptr(), b.data_ptr(), x.data_ptr(), _dev.stream())
        else:
            _lib.call("gfgpu_dofval_mul", self._inv.data_ptr(), b.data_ptr(), self._ndof,
                      x.data_ptr(), _dev.stream())
        return x

    def Solve(self, b):
        b = _dev.dev_f64(b)
        return self.solve(b, torch.empty_like(b))


class MatrixDiagonalPartitioned(MatrixDiagonal):
    """MatrixDiagonalPartitioned(conn, dofs, iip) (MatrixDiagonalPartitioned.h:42-452): the
    diagonal stored as [A_uu, A_pp] back to back in the partitioned numbering."""

    def __init__(self, conn, dofs, iip):
        super().__init__(conn, dofs)
        self._iip = _dev.host_i32(iip)
        self._iiu, self._part = _mesh.partition(self._dofs_h, self._iip)
        self._nnu, self._nnp = self._iiu.size, self._iip.size
        dof2part = np.empty(self._ndof, dtype=np.int32)
        dof2part[self._iiu] = np.arange(self._nnu, dtype=np.int32)
        dof2part[self._iip] = self._nnu + np.arange(self._nnp, dtype=np.int32)
        self.part_d = _dev.dev_i32(self._part)
        self.dof2part_d = _dev.dev_i32(dof2part)
        self.iiu_d = _dev.dev_i32(self._iiu)
        self.iip_d = _dev.dev_i32(self._iip)
        p, i = _dev.dof_csr(self._conn_h, self._part, self._ndof)
        self.pcsr_ptr, self.pcsr_idx = _dev.dev_i32(p), _dev.dev_i32(i)
        self._App = _dev.empty((self._ndof,))  # [Auu, App] back to back

    def nnu(self):
        return self._nnu

    def nnp(self):
        return self._nnp

    def iiu(self):
        return self._iiu.copy()

    def iip(self):
        return self._iip.copy()

    def part(self):
        return self._part.copy()

    def assemble(self, elemmat):
        """MatrixDiagonalPartitioned::assemble (MatrixDiagonalPartitioned.h:73-98)."""
        em = _dev.dev_f64(elemmat)
        _dev.check_shape(em, self.shape_elemmat(), "assemble")
        if not isDiagonal(em):
            raise RuntimeError("MatrixDiagonalPartitioned::assemble: elemmat is not diagonal")
        _lib.call("gfgpu_diag_assemble", self.pcsr_ptr.data_ptr(), self.pcsr_idx.data_ptr(),
                  self._ndof, self._nne, self._ndim, em.data_ptr(), self._App.data_ptr(),
                  _dev.stream())
        self._changed = True

    def _assemble_target(self):
        return self.pcsr_ptr, self.pcsr_idx, self._App

    def data_uu(self):
        return self._App[: self._nnu]

    def data_pp(self):
        return self._App[self._nnu:]

    def data(self):
        """MatrixDiagonalPartitioned::data (MatrixDiagonalPartitioned.h:142-155): the diagonal in
        the plain dof numbering."""
        out = _dev.empty((self._ndof,))
        _lib.call("gfgpu_from_partitioned", self.dof2part_d.data_ptr(), self._ndof, self._nnu,
                  self._nnp, self._App.data_ptr(), self._App[self._nnu:].data_ptr(),
                  out.data_ptr(), _dev.stream())
        return out

    def set(self, A):
        """MatrixDiagonalPartitioned::set (MatrixDiagonalPartitioned.h:121-135)."""
        A = _dev.dev_f64(A)
        _dev.check_shape(A, (self._ndof,), "set")
        s = _dev.stream()
        _lib.call("gfgpu_from_partitioned", self.iiu_d.data_ptr(), self._nnu, self._ndof, 0,
                  A.data_ptr(), None, self._App.data_ptr(), s)
        _lib.call("gfgpu_from_partitioned", self.iip_d.data_ptr(), self._nnp, self._ndof, 0,
                  A.data_ptr(), None, self._App[self._nnu:].data_ptr(), s)
        self._changed = True

    def _factorize(self):
        if self._changed:
            _lib.call("gfgpu_diag_factorize", self._App.data_ptr(), self._nnu,
                      self._inv.data_ptr(), _dev.stream())
            self._changed = False

    def _table(self, x):
        """(index table, rows, columns) of a nodevec or a dofval argument."""
        if x.dim() == 2:
            _dev.check_shape(x, (self._nnode, self._ndim), "MatrixDiagonalPartitioned")
            return self.part_d, self._nnode, self._ndim
        _dev.check_shape(x, (self._ndof,), "MatrixDiagonalPartitioned")
        return self.dof2part_d, self._ndof, 1

    def solve(self, b, x):
        """MatrixDiagonalPartitioned::solve, nodevec or dofval (MatrixDiagonalPartitioned.h:
        306-337): writes the unknown dofs of x only."""
        b = _dev.dev_f64(b)
        tab, n, m = self._table(b)
        _dev.check_shape(x, tuple(b.shape), "solve")
        self._factorize()
        _lib.call("gfgpu_diag_solve_nodevec", tab.data_ptr(), n, m, self._nnu,
                  self._inv.data_ptr(), b.data_ptr(), x.data_ptr(), _dev.stream())
        return x

    def Solve(self, b, x=None):
        """Solve with the prescribed dofs taken from `x` (zero if not given)."""
        b = _dev.dev_f64(b)
        x = torch.zeros_like(b) if x is None else _dev.dev_f64(x).clone()
        return self.solve(b, x)

    def reaction(self, x, b):
        """MatrixDiagonalPartitioned::reaction, nodevec or dofval (MatrixDiagonalPartitioned.h:
        378-403): b_p = A_pp x_p, other entries of b untouched."""
        x = _dev.dev_f64(x)
        tab, n, m = self._table(x)
        _dev.check_shape(b, tuple(x.shape), "reaction")
        _lib.call("gfgpu_diagp_reaction_nodevec", tab.data_ptr(), n, m, self._nnu,
                  self._App[self._nnu:].data_ptr(), x.data_ptr(), b.data_ptr(), _dev.stream())
        return b

    def Reaction(self, x, b):
        b = _dev.dev_f64(b).clone()
        return self.reaction(x, b)

    def dot(self, x, b):
        """MatrixDiagonalPartitioned::dot, nodevec or dofval (MatrixDiagonalPartitioned.h:
        189-225)."""
        x = _dev.dev_f64(x)
        tab, n, m = self._table(x)
        _dev.check_shape(b, tuple(x.shape), "dot")
        _lib.call("gfgpu_diag_dot_nodevec", tab.data_ptr(), n, m, self._App.data_ptr(),
                  x.data_ptr(), b.data_ptr(), _dev.stream())
        return b

    # ------------------------------------------------- partitioned (x_u, x_p) variants
    def _mul(self, a, x, n, name):
        x = _dev.dev_f64(x)
        _dev.check_shape(x, (n,), name)
        out = _dev.empty((n,))
        _lib.call("gfgpu_dofval_mul", a.data_ptr(), x.data_ptr(), n, out.data_ptr(), _dev.stream())
        return out

    def Dot_u(self, x_u, x_p):
        """b_u = A_uu x_u (MatrixDiagonalPartitioned.h:234-262)."""
        _dev.check_shape(x_p, (self._nnp,), "Dot_u")
        return self._mul(self._App, x_u, self._nnu, "Dot_u")

    def Dot_p(self, x_u, x_p):
        """b_p = A_pp x_p (MatrixDiagonalPartitioned.h:272-300)."""
        _dev.check_shape(x_u, (self._nnu,), "Dot_p")
        return self._mul(self._App[self._nnu:], x_p, self._nnp, "Dot_p")

    def Solve_u(self, b_u, x_p):
        """x_u = A_uu^-1 b_u (MatrixDiagonalPartitioned.h:343-372)."""
        _dev.check_shape(x_p, (self._nnp,), "Solve_u")
        self._factorize()
        return self._mul(self._inv, b_u, self._nnu, "Solve_u")

    def Reaction_p(self, x_u, x_p):
        """b_p = A_pp x_p (MatrixDiagonalPartitioned.h:405-421)."""
        _dev.check_shape(x_u, (self._nnu,), "Reaction_p")
        return self._mul(self._App[self._nnu:], x_p, self._nnp, "Reaction_p")


def _pattern(conn_h, dmap_h, nnode, n):
    """CSR pattern and per-nonzero triplet lists (gfgpu_host_matrix_pattern)."""
    import ctypes as C

    nelem, nne = conn_h.shape
    nd = dmap_h.shape[1]
    total = nelem * (nne * nd) ** 2
    rowptr = np.empty(n + 1, dtype=np.int32)
    col = np.empty(max(total, 1), dtype=np.int32)
    cptr = np.empty(total + 1, dtype=np.int32)
    cidx = np.empty(max(total, 1), dtype=np.int32)
    nnz = C.c_int64(0)
    _lib.call("gfgpu_host_matrix_pattern", conn_h.ctypes.data, dmap_h.ctypes.data, nelem, nne,
              nnode, nd, n, rowptr.ctypes.data, col.ctypes.data, cptr.ctypes.data,
              cidx.ctypes.data, C.addressof(nnz))
    k = int(nnz.value)
    return rowptr, col[:k].copy(), cptr[:k + 1].copy(), cidx[:total].copy()


class Matrix:
    """Matrix(conn, dofs) (Matrix.h:653-863): assembled sparse matrix in CSR on the device.
    assemble() sums the element-matrix entries of each nonzero in the triplet order of
    Matrix.h:704-733 (Eigen setFromTriplets), bit-exact in strict mode."""

    def __init__(self, conn, dofs):
        self._conn_h = _dev.host_i32(conn)
        self._dofs_h = _dev.host_i32(dofs)
        self._nelem, self._nne = self._conn_h.shape
        self._nnode, self._ndim = self._dofs_h.shape
        self._ndof = int(self._dofs_h.max()) + 1
        self._setup(self._dofs_h)

    def _setup(self, dmap):
        self._dmap = dmap
        rp, col, cptr, cidx = _pattern(self._conn_h, dmap, self._nnode, self._ndof)
        self._rowptr_h, self._col_h = rp, col
        self.rowptr, self.col = _dev.dev_i32(rp), _dev.dev_i32(col)
        self.cptr, self.cidx = _dev.dev_i32(cptr), _dev.dev_i32(cidx)
        self._nnz = int(col.size)
        self._val = torch.zeros(self._nnz, dtype=torch.float64, device=_dev.device())

    def nelem(self):
        return self._nelem

    def nne(self):
        return self._nne

    def nnode(self):
        return self._nnode

    def ndim(self):
        return self._ndim

    def ndof(self):
        return self._ndof

    def nnz(self):
        return self._nnz

    def shape_elemmat(self):
        k = self._nne * self._ndim
        return (self._nelem, k, k)

    def assemble(self, elemmat):
        em = _dev.dev_f64(elemmat)
        _dev.check_shape(em, self.shape_elemmat(), "assemble")
        if getattr(self, "_custom", False):  # set() / add() replaced the element pattern
            self._setup(self._dmap)
            self._custom = False
        _lib.call("gfgpu_matrix_assemble", self.cptr.data_ptr(), self.cidx.data_ptr(), self._nnz,
                  em.data_ptr(), self._val.data_ptr(), _dev.stream())

    @staticmethod
    def _triplets_csr(r, c, v, n):
        """CSR of triplets with equal (row, col) summed in their order (Eigen setFromTriplets)."""
        order = np.lexsort((np.arange(r.size), c, r))
        r, c, v = r[order], c[order], v[order]
        rowptr = np.zeros(n + 1, dtype=np.int64)
        cols, vals = [], []
        k = 0
        while k < r.size:
            j = k
            acc = v[k]
            while j + 1 < r.size and r[j + 1] == r[k] and c[j + 1] == c[k]:
                j += 1
                acc = acc + v[j]
            cols.append(c[k])
            vals.append(acc)
            rowptr[r[k] + 1] += 1
            k = j + 1
        return np.cumsum(rowptr), np.asarray(cols, dtype=np.int64), np.asarray(vals)

    def _replace(self, rowptr, col, val):
        self._rowptr_h = rowptr.astype(np.int32)
        self._col_h = col.astype(np.int32)
        self.rowptr = _dev.dev_i32(self._rowptr_h)
        self.col = _dev.dev_i32(self._col_h if col.size else np.zeros(1, np.int32))
        self._nnz = int(col.size)
        self._val = torch.as_tensor(val if val.size else np.zeros(1), dtype=torch.float64,
                                    device=_dev.device()).contiguous()
        self._custom = True

    def _block(self, rows, cols, matrix):
        rows = np.asarray(rows, dtype=np.int64).ravel()
        cols = np.asarray(cols, dtype=np.int64).ravel()
        m = np.asarray(matrix.cpu() if isinstance(matrix, torch.Tensor) else matrix, dtype=np.float64)
        if m.shape != (rows.size, cols.size):
            raise ValueError("matrix must be [rows.size, cols.size]")
        if rows.size and (rows.max() >= self._ndof or cols.max() >= self._ndof):
            raise ValueError("row / column out of range")
        r = np.repeat(rows, cols.size)
        c = np.tile(cols, rows.size)
        return self._triplets_csr(r, c, m.ravel(), self._ndof)

    def set(self, rows, cols, matrix):
        """Matrix::set (Matrix.h:737-764): the matrix becomes the given block (setFromTriplets)."""
        self._replace(*self._block(rows, cols, matrix))

    def add(self, rows, cols, matrix):
        """Matrix::add (Matrix.h:766-790): the given block is added (sparse sum)."""
        rp_b, col_b, val_b = self._block(rows, cols, matrix)
        rp_a, col_a, val_a = self._csr_host()
        rp_a = rp_a.astype(np.int64)
        ra = np.repeat(np.arange(self._ndof), np.diff(rp_a))
        rb = np.repeat(np.arange(self._ndof), np.diff(rp_b))
        # union: A entries first, then B, so that equal entries are summed as a + b
        r = np.concatenate([ra, rb])
        c = np.concatenate([col_a[:ra.size].astype(np.int64), col_b])
        v = np.concatenate([val_a[:ra.size], val_b])
        self._replace(*self._triplets_csr(r, c, v, self._ndof))

    def data(self):
        """(rowptr, col, val) of the CSR (device)."""
        return self.rowptr, self.col, self._val

    def _csr_host(self):
        return self._rowptr_h, self._col_h, self._val.cpu().numpy()

    def Todense(self):
        """Matrix::Todense (Matrix.h:350-372), host array in the original dof numbering."""
        rp, col, val = self._csr_host()
        A = np.zeros((self._ndof, self._ndof))
        rows = np.repeat(np.arange(self._ndof), np.diff(rp))
        A[rows, col] = val
        return A

    def _dofval(self, x):
        from .vector import Vector

        x = _dev.dev_f64(x)
        if x.dim() == 1:
            return x, None
        v = Vector(self._conn_h, self._dofs_h)
        return v.AsDofs(x), v

    def Dot(self, x):
        """Matrix::Dot (Matrix.h:376-409), dofval or nodevec."""
        xd, v = self._dofval(x)
        b = torch.empty(self._ndof, dtype=torch.float64, device=xd.device)
        _lib.call("gfgpu_matrix_dot_dofval", self.rowptr.data_ptr(), self.col.data_ptr(),
                  self._val.data_ptr(), self._ndof, xd.contiguous().data_ptr(), b.data_ptr(),
                  _dev.stream())
        return b if v is None else v.AsNode(b)


class MatrixPartitioned(Matrix):
    """MatrixPartitioned(conn, dofs, iip) (MatrixPartitioned.h:34-460): one CSR in the
    partitioned numbering (unknowns first); the blocks uu, up, pu, pp are its index ranges."""

    def __init__(self, conn, dofs, iip):
        self._conn_h = _dev.host_i32(conn)
        self._dofs_h = _dev.host_i32(dofs)
        self._nelem, self._nne = self._conn_h.shape
        self._nnode, self._ndim = self._dofs_h.shape
        self._ndof = int(self._dofs_h.max()) + 1
        self._iip = _dev.host_i32(iip)
        self._iiu, self._part = _mesh.partition(self._dofs_h, self._iip)
        self._nnu, self._nnp = int(self._iiu.size), int(self._iip.size)
        self._iperm_h = np.concatenate([self._iiu, self._iip]).astype(np.int32)
        self.iperm = _dev.dev_i32(self._iperm_h)
        self._setup(self._part)

    def nnu(self):
        return self._nnu

    def nnp(self):
        return self._nnp

    def iiu(self):
        return self._iiu.copy()

    def iip(self):
        return self._iip.copy()

    def _block(self, rows, cols, matrix):
        """set / add blocks (MatrixPartitioned.h:213-320) in the partitioned numbering."""
        part1d = np.empty(self._ndof, dtype=np.int64)
        part1d[self._iperm_h] = np.arange(self._ndof)
        rows = part1d[np.asarray(rows, dtype=np.int64).ravel()]
        cols = part1d[np.asarray(cols, dtype=np.int64).ravel()]
        return super()._block(rows, cols, matrix)

    def Todense(self):
        """MatrixPartitioned::Todense (MatrixPartitioned.h:324-351), original numbering."""
        rp, col, val = self._csr_host()
        A = np.zeros((self._ndof, self._ndof))
        rows = np.repeat(np.arange(self._ndof), np.diff(rp))
        A[self._iperm_h[rows], self._iperm_h[col]] = val
        return A

    def Dot(self, x):
        """MatrixPartitioned::Dot (MatrixPartitioned.h:354-398), dofval or nodevec."""
        xd, v = self._dofval(x)
        b = torch.empty(self._ndof, dtype=torch.float64, device=xd.device)
        _lib.call("gfgpu_matrixp_dot_dofval", self.rowptr.data_ptr(), self.col.data_ptr(),
                  self._val.data_ptr(), self._ndof, self._nnu, self.iperm.data_ptr(),
                  xd.contiguous().data_ptr(), b.data_ptr(), _dev.stream())
        return b if v is None else v.AsNode(b)

    def Reaction(self, x, b):
        """MatrixPartitioned::Reaction (MatrixPartitioned.h:401-433): copy of b with
        b_p = A_pu x_u + A_pp x_p, dofval or nodevec."""
        xd, v = self._dofval(x)
        bd, _ = self._dofval(b)
        bd = bd.clone()
        _lib.call("gfgpu_matrixp_reaction_dofval", self.rowptr.data_ptr(), self.col.data_ptr(),
                  self._val.data_ptr(), self._ndof, self._nnu, self.iperm.data_ptr(),
                  xd.contiguous().data_ptr(), bd.data_ptr(), _dev.stream())
        return bd if v is None else v.AsNode(bd)


class MatrixPartitionedSolver:
    """MatrixPartitionedSolver (MatrixPartitioned.h:471-642): x_u = A_uu^-1 (b_u - A_up x_p).
    The reference factorises A_uu (Eigen SimplicialLDLT: any symmetric nonsingular A_uu); here
    a Krylov solve of the assembled A_uu in FP64 to a relative residual `tol`: method "minres"
    (default; gfgpu_matrixp_solve_minres, indefinite allowed) or "pcg" (Jacobi-PCG,
    gfgpu_matrixp_solve, SPD only)."""

    def __init__(self, tol=1e-12, maxiter=1000000, check_every=16, method="minres"):
        if method not in ("minres", "pcg"):
            raise ValueError("method is 'minres' or 'pcg'")
        self.tol, self.maxiter, self.check_every = float(tol), int(maxiter), int(check_every)
        self.method = method
        self.iterations = 0
        self.relres = 0.0

    def Solve(self, A, b, x):
        """Copy of x with the unknown dofs solved (dofval or nodevec; x holds x_p)."""
        import ctypes as C

        xd, v = A._dofval(x)
        bd, _ = A._dofval(b)
        xd = xd.clone().contiguous()
        fn = "gfgpu_matrixp_solve_minres" if self.method == "minres" else "gfgpu_matrixp_solve"
        nb = int(getattr(_lib.lib(), fn + "_workspace_bytes")(A._nnu))
        ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=xd.device)
        it, rel = C.c_int64(0), C.c_double(0.0)
        _lib.call(fn, A.rowptr.data_ptr(), A.col.data_ptr(), A._val.data_ptr(),
                  A._ndof, A._nnu, A.iperm.data_ptr(), bd.contiguous().data_ptr(), xd.data_ptr(),
                  self.tol, self.maxiter, self.check_every, ws.data_ptr(), _dev.stream(),
                  C.addressof(it), C.addressof(rel))
        self.iterations, self.relres = int(it.value), float(rel.value)
        return xd if v is None else v.AsNode(xd)

    def solve(self, A, b, x):
        out = self.Solve(A, b, x)
        x.copy_(out)
        return x


class MatrixSolver:
    """MatrixSolver (Matrix.h:866-912): x = A^-1 b for a Matrix. The reference factorises A
    (Eigen SimplicialLDLT: any symmetric, possibly indefinite, nonsingular matrix); here MINRES
    with the preconditioner diag(|A_ii|) in FP64 to the relative residual `tol`
    (gfgpu_matrix_solve)."""

    def __init__(self, tol=1e-12, maxiter=1000000, check_every=16):
        self.tol, self.maxiter, self.check_every = float(tol), int(maxiter), int(check_every)
        self.iterations = 0
        self.relres = 0.0

    def Solve(self, A, b, x0=None):
        """dofval or nodevec b; returns x (x0: optional initial guess)."""
        import ctypes as C

        bd, v = A._dofval(b)
        bd = bd.contiguous()
        if x0 is None:
            xd = torch.zeros(A._ndof, dtype=torch.float64, device=bd.device)
        else:
            xd, _ = A._dofval(x0)
            xd = xd.clone().contiguous()
        nb = int(_lib.lib().gfgpu_matrix_solve_workspace_bytes(A._ndof))
        ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=bd.device)
        it, rel = C.c_int64(0), C.c_double(0.0)
        _lib.call("gfgpu_matrix_solve", A.rowptr.data_ptr(), A.col.data_ptr(), A._val.data_ptr(),
                  A._ndof, bd.data_ptr(), xd.data_ptr(), self.tol, self.maxiter, self.check_every,
                  ws.data_ptr(), _dev.stream(), C.addressof(it), C.addressof(rel))
        self.iterations, self.relres = int(it.value), float(rel.value)
        return xd if v is None else v.AsNode(xd)

    def solve(self, A, b, x):
        out = self.Solve(A, b, x)
        x.copy_(out)
        return x
