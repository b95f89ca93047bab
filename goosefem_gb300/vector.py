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
    unknown (iiu) and prescribed (iip) parts; `part` [nnode, ndim] numbers every dof by its
    position in [iiu, iip]."""

    def __init__(self, conn, dofs, iip):
        super().__init__(conn, dofs)
        iip = _dev.host_i32(iip)
        self._iiu, self._part = _mesh.partition(self._dofs_h, iip)
        self._iip = iip.copy()
        dof2part = np.empty(self._ndof, dtype=np.int32)
        dof2part[self._iiu] = np.arange(self._iiu.size, dtype=np.int32)
        dof2part[self._iip] = self._iiu.size + np.arange(self._iip.size, dtype=np.int32)
        self.iiu_d = _dev.dev_i32(self._iiu)
        self.iip_d = _dev.dev_i32(self._iip)
        self.part_d = _dev.dev_i32(self._part)
        self.dof2part_d = _dev.dev_i32(dof2part)

    def nnu(self):
        return self._iiu.size

    def nnp(self):
        return self._iip.size

    def iiu(self):
        return self._iiu.copy()

    def iip(self):
        return self._iip.copy()

    def dofs_is_u(self):
        """VectorPartitioned::dofs_is_u (VectorPartitioned.h:126-140)."""
        return self._part < self.nnu()

    def dofs_is_p(self):
        """VectorPartitioned::dofs_is_p (VectorPartitioned.h:147-161)."""
        return self._part >= self.nnu()

    # -------------------------------------------------------------- copy_u / copy_p
    def _copy_part(self, src, dest, lo, hi, name):
        src = _dev.dev_f64(src)
        _dev.check_shape(src, self.shape_nodevec(), name)
        _dev.check_shape(dest, self.shape_nodevec(), name)
        _lib.call("gfgpu_copy_partitioned_nodevec", self.part_d.data_ptr(), self._nnode,
                  self._ndim, lo, hi, src.data_ptr(), dest.data_ptr(), _dev.stream())
        return dest

    def copy_u(self, nodevec_src, nodevec_dest):
        """VectorPartitioned::copy_u (VectorPartitioned.h:198-216): unknown dofs of
        `nodevec_dest` overwritten from `nodevec_src`, in place."""
        return self._copy_part(nodevec_src, nodevec_dest, 0, self.nnu(), "copy_u")

    def copy_p(self, nodevec_src, nodevec_dest):
        """VectorPartitioned::copy_p (VectorPartitioned.h:251-269): prescribed dofs."""
        return self._copy_part(nodevec_src, nodevec_dest, self.nnu(), self._ndof, "copy_p")

    def Copy_u(self, nodevec_src, nodevec_dest):
        """VectorPartitioned::Copy_u (VectorPartitioned.h:176-184)."""
        return self.copy_u(nodevec_src, _dev.dev_f64(nodevec_dest).clone())

    def Copy_p(self, nodevec_src, nodevec_dest):
        """VectorPartitioned::Copy_p (VectorPartitioned.h:229-237)."""
        return self.copy_p(nodevec_src, _dev.dev_f64(nodevec_dest).clone())

    # ------------------------------------------------------ from partitioned storage
    def _uv(self, dofval_u, dofval_p, name):
        u, p = _dev.dev_f64(dofval_u), _dev.dev_f64(dofval_p)
        _dev.check_shape(u, (self.nnu(),), name)
        _dev.check_shape(p, (self.nnp(),), name)
        return u, p

    def dofsFromParitioned(self, dofval_u, dofval_p, dofval):
        """VectorPartitioned::dofsFromParitioned (VectorPartitioned.h:293-314); the reference's
        spelling is kept."""
        u, p = self._uv(dofval_u, dofval_p, "dofsFromParitioned")
        _dev.check_shape(dofval, self.shape_dofval(), "dofsFromParitioned")
        _lib.call("gfgpu_from_partitioned", self.dof2part_d.data_ptr(), self._ndof, self.nnu(),
                  self.nnp(), u.data_ptr(), p.data_ptr(), dofval.data_ptr(), _dev.stream())
        return dofval

    def DofsFromParitioned(self, dofval_u, dofval_p):
        return self.dofsFromParitioned(dofval_u, dofval_p, self.allocate_dofval())

    def nodeFromPartitioned(self, dofval_u, dofval_p, nodevec):
        """VectorPartitioned::nodeFromPartitioned (VectorPartitioned.h:344-365)."""
        u, p = self._uv(dofval_u, dofval_p, "nodeFromPartitioned")
        _dev.check_shape(nodevec, self.shape_nodevec(), "nodeFromPartitioned")
        _lib.call("gfgpu_from_partitioned", self.part_d.data_ptr(), self._nnode * self._ndim,
                  self.nnu(), self.nnp(), u.data_ptr(), p.data_ptr(), nodevec.data_ptr(),
                  _dev.stream())
        return nodevec

    def NodeFromPartitioned(self, dofval_u, dofval_p):
        return self.nodeFromPartitioned(dofval_u, dofval_p, self.allocate_nodevec())

    def elementFromPartitioned(self, dofval_u, dofval_p, elemvec):
        """VectorPartitioned::elementFromPartitioned (VectorPartitioned.h:395-418)."""
        u, p = self._uv(dofval_u, dofval_p, "elementFromPartitioned")
        _dev.check_shape(elemvec, self.shape_elemvec(), "elementFromPartitioned")
        _lib.call("gfgpu_from_partitioned_elemvec", self.conn_d.data_ptr(), self.part_d.data_ptr(),
                  self._nelem, self._nne, self._ndim, self.nnu(), self.nnp(), u.data_ptr(),
                  p.data_ptr(), elemvec.data_ptr(), _dev.stream())
        return elemvec

    def ElementFromPartitioned(self, dofval_u, dofval_p):
        return self.elementFromPartitioned(dofval_u, dofval_p, self.allocate_elemvec())

    # ----------------------------------------------------------- asDofs_u / asDofs_p
    def _as_dofs_sub(self, arg, ret, sel, n, name):
        arg = _dev.dev_f64(arg)
        _dev.check_shape(ret, (n,), name)
        if self._kind(arg) != "dofval":
            arg = self.AsDofs(arg)  # last writer wins, as the reference's serial loops
        _lib.call("gfgpu_from_partitioned", sel.data_ptr(), n, self._ndof, 0, arg.data_ptr(), None,
                  ret.data_ptr(), _dev.stream())
        return ret

    def asDofs_u(self, arg, dofval_u):
        """VectorPartitioned::asDofs_u of a dofval, nodevec or elemvec
        (VectorPartitioned.h:428-539)."""
        return self._as_dofs_sub(arg, dofval_u, self.iiu_d, self.nnu(), "asDofs_u")

    def asDofs_p(self, arg, dofval_p):
        """VectorPartitioned::asDofs_p (VectorPartitioned.h:549-660)."""
        return self._as_dofs_sub(arg, dofval_p, self.iip_d, self.nnp(), "asDofs_p")

    def AsDofs_u(self, arg):
        return self.asDofs_u(arg, _dev.empty((self.nnu(),)))

    def AsDofs_p(self, arg):
        return self.asDofs_p(arg, _dev.empty((self.nnp(),)))
