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
    """MatrixDiagonalPartitioned(conn, dofs, iip) (MatrixDiagonalPartitioned.h:42-70)."""

    def __init__(self, conn, dofs, iip):
        super().__init__(conn, dofs)
        self._iip = _dev.host_i32(iip)
        self._iiu, self._part = _mesh.partition(self._dofs_h, self._iip)
        self._nnu, self._nnp = self._iiu.size, self._iip.size
        self.part_d = _dev.dev_i32(self._part)
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

    def data_uu(self):
        return self._App[: self._nnu]

    def data_pp(self):
        return self._App[self._nnu:]

    def data(self):
        out = torch.zeros(self._ndof, dtype=torch.float64, device=self._App.device)
        out[torch.as_tensor(self._iiu, device=out.device).long()] = self.data_uu()
        out[torch.as_tensor(self._iip, device=out.device).long()] = self.data_pp()
        return out

    def set(self, A):
        A = _dev.dev_f64(A)
        self._App[: self._nnu] = A[torch.as_tensor(self._iiu, device=A.device).long()]
        self._App[self._nnu:] = A[torch.as_tensor(self._iip, device=A.device).long()]
        self._changed = True

    def _factorize(self):
        if self._changed:
            _lib.call("gfgpu_diag_factorize", self._App.data_ptr(), self._nnu,
                      self._inv.data_ptr(), _dev.stream())
            self._changed = False

    def solve(self, b, x):
        """MatrixDiagonalPartitioned::solve nodevec (MatrixDiagonalPartitioned.h:306-322):
        writes the unknown dofs of x only."""
        b = _dev.dev_f64(b)
        self._factorize()
        _lib.call("gfgpu_diag_solve_nodevec", self.part_d.data_ptr(), self._nnode, self._ndim,
                  self._nnu, self._inv.data_ptr(), b.data_ptr(), x.data_ptr(), _dev.stream())
        return x

    def Solve(self, b, x):
        x = _dev.dev_f64(x).clone()
        return self.solve(b, x)

    def reaction(self, x, b):
        """MatrixDiagonalPartitioned::reaction nodevec (MatrixDiagonalPartitioned.h:378-392)."""
        x = _dev.dev_f64(x)
        _lib.call("gfgpu_diagp_reaction_nodevec", self.part_d.data_ptr(), self._nnode, self._ndim,
                  self._nnu, self._App[self._nnu:].data_ptr(), x.data_ptr(), b.data_ptr(),
                  _dev.stream())
        return b

    def Reaction(self, x, b):
        b = _dev.dev_f64(b).clone()
        return self.reaction(x, b)

    def dot(self, x, b):
        """MatrixDiagonalPartitioned::dot nodevec (MatrixDiagonalPartitioned.h:189-205)."""
        x = _dev.dev_f64(x)
        _lib.call("gfgpu_diag_dot_nodevec", self.part_d.data_ptr(), self._nnode, self._ndim,
                  self._App.data_ptr(), x.data_ptr(), b.data_ptr(), _dev.stream())
        return b
