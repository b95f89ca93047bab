"""GooseFEM.Element.Quad4 / Hex8 quadrature on the GPU (mirror of include/GooseFEM/Element.h,
ElementQuad4.h and ElementHex8.h).

Quadrature(x[, xi, w]) computes the shape functions, the shape-function gradients dNx
[nelem, nip, nne, ndim] and the integration volumes dV [nelem, nip] on the device at
construction, then exposes the element-by-element operators of QuadratureBaseCartesian.
"""

import ctypes as C
import math

import numpy as np
import torch

from . import _dev, _lib


class _Rule:
    def __init__(self, xi, w):
        self._xi = np.asarray(xi, dtype=np.float64)
        self._w = np.asarray(w, dtype=np.float64)

    def nip(self):
        return self._w.size

    def xi(self):
        return self._xi.copy()

    def w(self):
        return self._w.copy()


def _quad4_gauss():
    g = 1.0 / math.sqrt(3.0)
    return _Rule([[-g, -g], [+g, -g], [+g, +g], [-g, +g]], [1.0] * 4)


def _quad4_nodal():
    return _Rule([[-1.0, -1.0], [+1.0, -1.0], [+1.0, +1.0], [-1.0, +1.0]], [1.0] * 4)


def _quad4_midpoint():
    return _Rule([[0.0, 0.0]], [1.0])


_HEX_S = [[-1, -1, -1], [+1, -1, -1], [+1, +1, -1], [-1, +1, -1],
          [-1, -1, +1], [+1, -1, +1], [+1, +1, +1], [-1, +1, +1]]


def _hex8_gauss():
    g = 1.0 / math.sqrt(3.0)
    return _Rule([[s * g for s in r] for r in _HEX_S], [1.0] * 8)


def _hex8_nodal():
    return _Rule([[float(s) for s in r] for r in _HEX_S], [1.0] * 8)


class _QuadratureBase:
    _nne = None
    _ndim = None
    _tdim = None
    _fn = None

    def __init__(self, x, xi=None, w=None):
        if xi is None:
            rule = self._gauss()
            xi, w = rule.xi(), rule.w()
        self._x = _dev.dev_f64(x)
        if self._x.dim() != 3 or tuple(self._x.shape[1:]) != (self._nne, self._ndim):
            raise ValueError(f"x must be an elemvec [nelem, {self._nne}, {self._ndim}]")
        self._xi = _dev.dev_f64(xi)
        self._w = _dev.dev_f64(w)
        self._nip = int(self._w.numel())
        if tuple(self._xi.shape) != (self._nip, self._ndim):
            raise ValueError("xi must be [nip, ndim]")
        self._nelem = int(self._x.shape[0])
        self._N = _dev.empty((self._nip, self._nne))
        self._dNxi = _dev.empty((self._nip, self._nne, self._ndim))
        self._dNx = _dev.empty((self._nelem, self._nip, self._nne, self._ndim))
        self._vol = _dev.empty((self._nelem, self._nip))
        self._compute_dN()

    def _compute_dN(self):
        _lib.call(self._fn, self._x.data_ptr(), self._nelem, self._xi.data_ptr(),
                  self._w.data_ptr(), self._nip, self._N.data_ptr(), self._dNxi.data_ptr(),
                  self._dNx.data_ptr(), self._vol.data_ptr(), _dev.stream())

    def update_x(self, x):
        """QuadratureBaseCartesian::update_x (Element.h:564-569)."""
        x = _dev.dev_f64(x)
        _dev.check_shape(x, self._x.shape, "update_x")
        self._x.copy_(x)
        self._compute_dN()

    # sizes and shapes (Element.h:151-534)
    def nelem(self):
        return self._nelem

    def nne(self):
        return self._nne

    def ndim(self):
        return self._ndim

    def tdim(self):
        return self._ndim if self._tdim is None else self._tdim

    def nip(self):
        return self._nip

    def shape_elemvec(self, n=None):
        return (self._nelem, self._nne, self._ndim if n is None else n)

    def shape_elemmat(self):
        k = self._nne * self._ndim
        return (self._nelem, k, k)

    def shape_qtensor(self, rank=0, n=None):
        return (self._nelem, self._nip) + (self.tdim() if n is None else n,) * rank

    def shape_qscalar(self):
        return (self._nelem, self._nip)

    def shape_qvector(self, n=None):
        return (self._nelem, self._nip, self._ndim if n is None else n)

    def allocate_qtensor(self, rank=0, val=None):
        t = _dev.empty(self.shape_qtensor(rank))
        return t if val is None else t.fill_(val)

    def allocate_qscalar(self, val=None):
        return self.allocate_qtensor(0, val)

    def allocate_elemvec(self, val=None):
        t = _dev.empty(self.shape_elemvec())
        return t if val is None else t.fill_(val)

    def allocate_elemmat(self, val=None):
        t = _dev.empty(self.shape_elemmat())
        return t if val is None else t.fill_(val)

    def asTensor(self, qscalar, qtensor):
        """QuadratureBase::asTensor (Element.h:215-220): qscalar repeated over the tensor
        components of `qtensor` [nelem, nip, tdim, ...]."""
        src = _dev.dev_f64(qscalar)
        _dev.check_shape(src, self.shape_qscalar(), "asTensor")
        if tuple(qtensor.shape[:2]) != self.shape_qscalar():
            raise ValueError(f"asTensor: shape {tuple(qtensor.shape)} is not a qtensor")
        k = int(np.prod(qtensor.shape[2:], dtype=np.int64))
        _lib.call("gfgpu_broadcast", src.data_ptr(), self._nelem * self._nip, k, qtensor.data_ptr(),
                  _dev.stream())
        return qtensor

    def AsTensor(self, rank, qscalar):
        """QuadratureBase::AsTensor(rank, qscalar) (Element.h:241-246)."""
        return self.asTensor(qscalar, self.allocate_qtensor(rank))

    def GradN(self):
        return self._dNx

    def dV(self):
        return self._vol

    def N(self):
        return self._N

    # ------------------------------------------------------------------ operators
    def interpQuad_vector(self, elemvec, qvector):
        ev = _dev.dev_f64(elemvec)
        n = int(ev.shape[2])
        _dev.check_shape(ev, self.shape_elemvec(n), "interpQuad_vector")
        _dev.check_shape(qvector, self.shape_qvector(n), "interpQuad_vector")
        _lib.call("gfgpu_interp_quad_vector", self._N.data_ptr(), ev.data_ptr(), self._nelem,
                  self._nne, self._nip, n, qvector.data_ptr(), _dev.stream())
        return qvector

    def InterpQuad_vector(self, elemvec):
        ev = _dev.dev_f64(elemvec)
        return self.interpQuad_vector(ev, _dev.empty(self.shape_qvector(int(ev.shape[2]))))

    def _grad(self, fn, elemvec, qtensor):
        ev = _dev.dev_f64(elemvec)
        _dev.check_shape(ev, self.shape_elemvec(), fn)
        _dev.check_shape(qtensor, self.shape_qtensor(2), fn)
        _lib.call(fn, self._dNx.data_ptr(), ev.data_ptr(), self._nelem, self._nne, self._nip,
                  self._ndim, qtensor.data_ptr(), _dev.stream())
        return qtensor

    def gradN_vector(self, elemvec, qtensor):
        return self._grad("gfgpu_grad_n_vector", elemvec, qtensor)

    def GradN_vector(self, elemvec):
        return self.gradN_vector(elemvec, self.allocate_qtensor(2))

    def gradN_vector_T(self, elemvec, qtensor):
        return self._grad("gfgpu_grad_n_vector_T", elemvec, qtensor)

    def GradN_vector_T(self, elemvec):
        return self.gradN_vector_T(elemvec, self.allocate_qtensor(2))

    def symGradN_vector(self, elemvec, qtensor):
        return self._grad("gfgpu_sym_grad_n_vector", elemvec, qtensor)

    def SymGradN_vector(self, elemvec):
        return self.symGradN_vector(elemvec, self.allocate_qtensor(2))

    def int_N_vector_dV(self, qvector, elemvec):
        qv = _dev.dev_f64(qvector)
        n = int(qv.shape[2])
        _dev.check_shape(qv, self.shape_qvector(n), "int_N_vector_dV")
        _dev.check_shape(elemvec, self.shape_elemvec(n), "int_N_vector_dV")
        _lib.call("gfgpu_int_n_vector_dv", self._N.data_ptr(), self._vol.data_ptr(), qv.data_ptr(),
                  self._nelem, self._nne, self._nip, n, elemvec.data_ptr(), _dev.stream())
        return elemvec

    def Int_N_vector_dV(self, qvector):
        qv = _dev.dev_f64(qvector)
        return self.int_N_vector_dV(qv, _dev.empty(self.shape_elemvec(int(qv.shape[2]))))

    def int_N_scalar_NT_dV(self, qscalar, elemmat):
        qs = _dev.dev_f64(qscalar)
        _dev.check_shape(qs, self.shape_qscalar(), "int_N_scalar_NT_dV")
        _dev.check_shape(elemmat, self.shape_elemmat(), "int_N_scalar_NT_dV")
        _lib.call("gfgpu_int_n_scalar_nt_dv", self._N.data_ptr(), self._vol.data_ptr(),
                  qs.data_ptr(), self._nelem, self._nne, self._nip, self._ndim,
                  elemmat.data_ptr(), _dev.stream())
        return elemmat

    def Int_N_scalar_NT_dV(self, qscalar):
        return self.int_N_scalar_NT_dV(qscalar, self.allocate_elemmat())

    def int_N_scalar_NT_dV_diag(self, qscalar, elemvec, check=True):
        """Diagonal of Int_N_scalar_NT_dV as an elemvec (elemvec(e,m,i) = elemmat(e, m*ndim+i,
        m*ndim+i)), without forming the element matrices (gfgpu_int_n_scalar_nt_dv_diag). With
        check=True the off-diagonal entries are formed on the fly and a non-diagonal result
        (Element::isDiagonal) raises, as MatrixDiagonal::assemble would."""
        qs = _dev.dev_f64(qscalar)
        _dev.check_shape(qs, self.shape_qscalar(), "int_N_scalar_NT_dV_diag")
        _dev.check_shape(elemvec, self.shape_elemvec(), "int_N_scalar_NT_dV_diag")
        flag = C.c_int(0)
        _lib.call("gfgpu_int_n_scalar_nt_dv_diag", self._N.data_ptr(), self._vol.data_ptr(),
                  qs.data_ptr(), self._nelem, self._nne, self._nip, self._ndim,
                  elemvec.data_ptr(), C.addressof(flag) if check else None, _dev.stream())
        if check and not flag.value:
            raise RuntimeError("Int_N_scalar_NT_dV_diag: the element matrices are not diagonal")
        return elemvec

    def Int_N_scalar_NT_dV_diag(self, qscalar, check=True):
        return self.int_N_scalar_NT_dV_diag(qscalar, self.allocate_elemvec(), check)

    def int_gradN_dot_tensor2_dV(self, qtensor, elemvec):
        qt = _dev.dev_f64(qtensor)
        _dev.check_shape(qt, self.shape_qtensor(2), "int_gradN_dot_tensor2_dV")
        _dev.check_shape(elemvec, self.shape_elemvec(), "int_gradN_dot_tensor2_dV")
        _lib.call("gfgpu_int_grad_n_dot_tensor2_dv", self._dNx.data_ptr(), self._vol.data_ptr(),
                  qt.data_ptr(), self._nelem, self._nne, self._nip, self._ndim,
                  elemvec.data_ptr(), _dev.stream())
        return elemvec

    def Int_gradN_dot_tensor2_dV(self, qtensor):
        return self.int_gradN_dot_tensor2_dV(qtensor, self.allocate_elemvec())

    def int_gradN_dot_tensor4_dot_gradNT_dV(self, qtensor, elemmat):
        qt = _dev.dev_f64(qtensor)
        _dev.check_shape(qt, self.shape_qtensor(4), "int_gradN_dot_tensor4_dot_gradNT_dV")
        _dev.check_shape(elemmat, self.shape_elemmat(), "int_gradN_dot_tensor4_dot_gradNT_dV")
        _lib.call("gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv", self._dNx.data_ptr(),
                  self._vol.data_ptr(), qt.data_ptr(), self._nelem, self._nne, self._nip,
                  self._ndim, elemmat.data_ptr(), _dev.stream())
        return elemmat

    def Int_gradN_dot_tensor4_dot_gradNT_dV(self, qtensor):
        return self.int_gradN_dot_tensor4_dot_gradNT_dV(qtensor, self.allocate_elemmat())


class _NS:
    pass


class Quad4:
    """Element::Quad4 (ElementQuad4.h)."""

    Gauss = _NS()
    Nodal = _NS()
    MidPoint = _NS()

    class Quadrature(_QuadratureBase):
        _nne, _ndim, _fn = 4, 2, "gfgpu_quad4_compute_dN"

        @staticmethod
        def _gauss():
            return _quad4_gauss()


class _QuadraturePlanar(_QuadratureBase):
    """Element::Quad4::QuadraturePlanar (ElementQuad4Planar.h:38-335): Quad4 with 3x3
    quadrature-point tensors (plane strain) and the out-of-plane thickness in dV."""

    _nne, _ndim, _tdim = 4, 2, 3

    def __init__(self, x, xi=None, w=None, thick=1.0):
        self._thick = float(thick)
        super().__init__(x, xi, w)

    @staticmethod
    def _gauss():
        return _quad4_gauss()

    def _compute_dN(self):
        _lib.call("gfgpu_quad4_planar_compute_dN", self._x.data_ptr(), self._nelem,
                  self._xi.data_ptr(), self._w.data_ptr(), self._nip, self._thick,
                  self._N.data_ptr(), self._dNxi.data_ptr(), self._dNx.data_ptr(),
                  self._vol.data_ptr(), _dev.stream())

    def _grad(self, fn, elemvec, qtensor):
        ev = _dev.dev_f64(elemvec)
        _dev.check_shape(ev, self.shape_elemvec(), fn)
        _dev.check_shape(qtensor, self.shape_qtensor(2), fn)
        _lib.call(fn + "_planar", self._dNx.data_ptr(), ev.data_ptr(), self._nelem, self._nip,
                  qtensor.data_ptr(), _dev.stream())
        return qtensor

    def int_gradN_dot_tensor2_dV(self, qtensor, elemvec):
        qt = _dev.dev_f64(qtensor)
        _dev.check_shape(qt, self.shape_qtensor(2), "int_gradN_dot_tensor2_dV")
        _dev.check_shape(elemvec, self.shape_elemvec(), "int_gradN_dot_tensor2_dV")
        _lib.call("gfgpu_int_grad_n_dot_tensor2_dv_planar", self._dNx.data_ptr(),
                  self._vol.data_ptr(), qt.data_ptr(), self._nelem, self._nip, elemvec.data_ptr(),
                  _dev.stream())
        return elemvec

    def int_gradN_dot_tensor4_dot_gradNT_dV(self, qtensor, elemmat):
        qt = _dev.dev_f64(qtensor)
        _dev.check_shape(qt, self.shape_qtensor(4), "int_gradN_dot_tensor4_dot_gradNT_dV")
        _dev.check_shape(elemmat, self.shape_elemmat(), "int_gradN_dot_tensor4_dot_gradNT_dV")
        _lib.call("gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv_planar", self._dNx.data_ptr(),
                  self._vol.data_ptr(), qt.data_ptr(), self._nelem, self._nip,
                  elemmat.data_ptr(), _dev.stream())
        return elemmat


Quad4.QuadraturePlanar = _QuadraturePlanar


class Hex8:
    """Element::Hex8 (ElementHex8.h)."""

    Gauss = _NS()
    Nodal = _NS()

    class Quadrature(_QuadratureBase):
        _nne, _ndim, _fn = 8, 3, "gfgpu_hex8_compute_dN"

        @staticmethod
        def _gauss():
            return _hex8_gauss()


for _ns, _rule in ((Quad4.Gauss, _quad4_gauss), (Quad4.Nodal, _quad4_nodal),
                   (Quad4.MidPoint, _quad4_midpoint), (Hex8.Gauss, _hex8_gauss),
                   (Hex8.Nodal, _hex8_nodal)):
    _ns.xi = (lambda r=_rule: r().xi())
    _ns.w = (lambda r=_rule: r().w())
    _ns.nip = (lambda r=_rule: r().nip())


def isDiagonal(elemmat):
    """Element::isDiagonal (Element.h:122-145)."""
    em = _dev.dev_f64(elemmat)
    res = C.c_int(0)
    _lib.call("gfgpu_is_diagonal", em.data_ptr(), int(em.shape[0]), int(em.shape[1]),
              C.addressof(res), _dev.stream())
    return bool(res.value)
