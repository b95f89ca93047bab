"""GooseFEM.Vector / VectorPartitioned on the GPU (mirror of include/GooseFEM/Vector.h and
VectorPartitioned.h).

Storage names as in the reference: "dofval" [ndof], "nodevec" [nnode, ndim],
"elemvec" [nelem, nne, ndim]. Capitalised methods allocate and return a device tensor,
lower-case methods write into a caller-provided tensor (Element.h:597-616 pattern).
Assembly is a deterministic gather over a dof-centric CSR in the reference's serial order.
"""

import numpy as np
import torch

from . import _dev, _lib
from . import mesh as _mesh


class Vector:
    """Vector(conn, dofs) (Vector.h:34-47)."""

    def __init__(self, conn, dofs):
        conn_h = _dev.host_i32(conn)
        dofs_h = _dev.host_i32(dofs)
        if conn_h.ndim != 2 or dofs_h.ndim != 2:
            raise ValueError("conn and dofs must be 2-d")
        self._nelem, self._nne = conn_h.shape
        self._nnode, self._ndim = dofs_h.shape
        self._ndof = int(dofs_h.max()) + 1 if dofs_h.size else 0
        if conn_h.size and int(conn_h.max()) + 1 > self._nnode:
            raise ValueError("conn refers to a node beyond dofs")
        if self._ndof > self._nnode * self._ndim:
            raise ValueError("ndof > nnode * ndim")
        self._conn_h, self._dofs_h = conn_h, dofs_h
        self.conn_d = _dev.dev_i32(conn_h)
        self.dofs_d = _dev.dev_i32(dofs_h)
        p, i = _dev.dof_csr(conn_h, dofs_h, self._ndof)
        self.csr_ptr, self.csr_idx = _dev.dev_i32(p), _dev.dev_i32(i)
        p, i = _dev.dof_csr_nodevec(dofs_h, self._ndof)
        self.csrn_ptr, self.csrn_idx = _dev.dev_i32(p), _dev.dev_i32(i)
        self.last_elem = torch.empty(self._ndof, dtype=torch.int32, device=_dev.device())
        self.last_node = torch.empty(self._ndof, dtype=torch.int32, device=_dev.device())
        s = _dev.stream()
        _lib.call("gfgpu_csr_last", self.csr_ptr.data_ptr(), self.csr_idx.data_ptr(), self._ndof,
                  self.last_elem.data_ptr(), s)
        _lib.call("gfgpu_csr_last", self.csrn_ptr.data_ptr(), self.csrn_idx.data_ptr(), self._ndof,
                  self.last_node.data_ptr(), s)

    # ------------------------------------------------------------------ sizes
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

    def conn(self):
        return self._conn_h.copy()

    def dofs(self):
        return self._dofs_h.copy()

    def shape_dofval(self):
        return (self._ndof,)

    def shape_nodevec(self):
        return (self._nnode, self._ndim)

    def shape_elemvec(self):
        return (self._nelem, self._nne, self._ndim)

    def shape_elemmat(self):
        n = self._nne * self._ndim
        return (self._nelem, n, n)

    def allocate_dofval(self, val=None):
        t = _dev.empty(self.shape_dofval())
        return t if val is None else t.fill_(val)

    def allocate_nodevec(self, val=None):
        t = _dev.empty(self.shape_nodevec())
        return t if val is None else t.fill_(val)

    def allocate_elemvec(self, val=None):
        t = _dev.empty(self.shape_elemvec())
        return t if val is None else t.fill_(val)

    def allocate_elemmat(self, val=None):
        t = _dev.empty(self.shape_elemmat())
        return t if val is None else t.fill_(val)

    # ------------------------------------------------------------------ conversions
    def _kind(self, arg):
        shp = tuple(arg.shape)
        if shp == self.shape_dofval() and len(shp) == 1:
            return "dofval"
        if shp == self.shape_nodevec():
            return "nodevec"
        if shp == self.shape_elemvec():
            return "elemvec"
        raise RuntimeError(f"Vector: unknown storage for shape {shp}")

    def asElement(self, arg, ret):
        """Vector::asElement (Vector.h:681-697 nodevec, :659-675 dofval)."""
        arg = _dev.dev_f64(arg)
        _dev.check_shape(ret, self.shape_elemvec(), "asElement")
        if self._kind(arg) == "nodevec":
            _lib.call("gfgpu_as_element", self.conn_d.data_ptr(), self._nelem, self._nne,
                      self._ndim, arg.data_ptr(), ret.data_ptr(), _dev.stream())
        else:
            _lib.call("gfgpu_as_element_dofval", self.conn_d.data_ptr(), self.dofs_d.data_ptr(),
                      self._nelem, self._nne, self._ndim, arg.data_ptr(), ret.data_ptr(),
                      _dev.stream())
        return ret

    def AsElement(self, arg):
        return self.asElement(arg, self.allocate_elemvec())

    def asNode(self, arg, ret):
        """Vector::asNode dofval -> nodevec (Vector.h:615-629)."""
        arg = _dev.dev_f64(arg)
        _dev.check_shape(ret, self.shape_nodevec(), "asNode")
        if self._kind(arg) == "dofval":
            _lib.call("gfgpu_as_node", self.dofs_d.data_ptr(), self._nnode, self._ndim,
                      arg.data_ptr(), ret.data_ptr(), _dev.stream())
        else:  # elemvec -> nodevec (Vector.h:634-652): via dofval
            d = self.AsDofs(arg)
            self.asNode(d, ret)
        return ret

    def AsNode(self, arg):
        return self.asNode(arg, self.allocate_nodevec())

    def asDofs(self, arg, ret):
        """Vector::asDofs (Vector.h:569-608): last writer wins, unwritten dofs are 0."""
        arg = _dev.dev_f64(arg)
        _dev.check_shape(ret, self.shape_dofval(), "asDofs")
        last = self.last_node if self._kind(arg) == "nodevec" else self.last_elem
        _lib.call("gfgpu_as_dofs", last.data_ptr(), self._ndof, arg.data_ptr(), ret.data_ptr(),
                  _dev.stream())
        return ret

    def AsDofs(self, arg):
        return self.asDofs(arg, self.allocate_dofval())

    def assembleDofs(self, arg, ret):
        """Vector::assembleDofs (Vector.h:703-741), deterministic gather."""
        arg = _dev.dev_f64(arg)
        _dev.check_shape(ret, self.shape_dofval(), "assembleDofs")
        if self._kind(arg) == "nodevec":
            p, i = self.csrn_ptr, self.csrn_idx
        else:
            p, i = self.csr_ptr, self.csr_idx
        _lib.call("gfgpu_assemble_dofs", p.data_ptr(), i.data_ptr(), self._ndof, arg.data_ptr(),
                  ret.data_ptr(), _dev.stream())
        return ret

    def AssembleDofs(self, arg):
        return self.assembleDofs(arg, self.allocate_dofval())

    def assembleNode(self, arg, ret):
        """Vector::assembleNode (Vector.h:747-757)."""
        arg = _dev.dev_f64(arg)
        _dev.check_shape(arg, self.shape_elemvec(), "assembleNode")
        _dev.check_shape(ret, self.shape_nodevec(), "assembleNode")
        _lib.call("gfgpu_assemble_node", self.csr_ptr.data_ptr(), self.csr_idx.data_ptr(),
                  self.dofs_d.data_ptr(), self._nnode, self._ndim, arg.data_ptr(), ret.data_ptr(),
                  _dev.stream())
        return ret

    def AssembleNode(self, arg):
        return self.assembleNode(arg, self.allocate_nodevec())

    def copy(self, src, dest):
        dest.copy_(_dev.dev_f64(src))
        return dest

    def Copy(self, src, dest):
        return self.copy(src, dest.clone())


class VectorPartitioned(Vector):
    """VectorPartitioned(conn, dofs, iip) (VectorPartitioned.h:45-661): dofs split into
    unknown (iiu) and prescribed (iip) parts."""

    def __init__(self, conn, dofs, iip):
        super().__init__(conn, dofs)
        iip = _dev.host_i32(iip)
        self._iiu, self._part = _mesh.partition(self._dofs_h, iip)
        self._iip = iip.copy()
        self.iiu_d = _dev.dev_i32(self._iiu)
        self.iip_d = _dev.dev_i32(self._iip)
        self.part_d = _dev.dev_i32(self._part)

    def nnu(self):
        return self._iiu.size

    def nnp(self):
        return self._iip.size

    def iiu(self):
        return self._iiu.copy()

    def iip(self):
        return self._iip.copy()

    def dofs_is_u(self):
        return self._part < self.nnu()

    def dofs_is_p(self):
        return self._part >= self.nnu()

    def AsDofs_u(self, arg):
        return self.AsDofs(arg)[self.iiu_d.long()]

    def AsDofs_p(self, arg):
        return self.AsDofs(arg)[self.iip_d.long()]

    def Copy_u(self, nodevec_src, nodevec_dest):
        """VectorPartitioned::copy_u (VectorPartitioned.h:198): unknown dofs from src."""
        out = _dev.dev_f64(nodevec_dest).clone()
        mask = torch.as_tensor(self._part < self.nnu(), device=out.device)
        src = _dev.dev_f64(nodevec_src)
        out[mask] = src[mask]
        return out

    def Copy_p(self, nodevec_src, nodevec_dest):
        """VectorPartitioned::copy_p (VectorPartitioned.h:251): prescribed dofs from src."""
        out = _dev.dev_f64(nodevec_dest).clone()
        mask = torch.as_tensor(self._part >= self.nnu(), device=out.device)
        src = _dev.dev_f64(nodevec_src)
        out[mask] = src[mask]
        return out
