"""Linear elastic stress and the fused explicit velocity-Verlet integrator on the GPU.

The integrator runs the loop of docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157
(scheme: docs/examples/dynamics_inertia-damping.rst:6-66) with a nodal viscous damping force
-eta * v in the residual, a lumped mass from Int_N_scalar_NT_dV with nodal quadrature, and
fixed DOFs handled as MatrixDiagonalPartitioned does (the solve leaves them untouched).
"""

import ctypes as C
import math

import numpy as np
import torch

from . import _dev, _lib
from . import mesh as _mesh
from .element import Quad4, Hex8

# Relative tolerance of the uniform-box detection (gfgpu_verlet_detect_uniform): a mesh whose dNx
# or vol differ from the box model by more than this (relative to the largest |dNx|) takes the
# general per-Gauss-point kernel. The closed form's error on an almost-uniform mesh is of the
# order of that deviation, so the floor sits an order of magnitude inside the 1e-12 parity bound.
UNIFORM_RTOL = 1e-13


def uniform_rtol(coor, conn):
    """Detection tolerance for a mesh: the floor UNIFORM_RTOL, or twice the rounding noise that
    compute_dN itself leaves on an exact grid of this extent, whichever is larger. The Jacobian
    sums terms of the size of the coordinates that cancel to the element size, so the reference's
    own dNx / vol deviate from the exact box by about eps * max|x| / h (measured on Regular unit
    grids: 1.4e-14 at 64^2, 5.7e-14 at 256^2, 2.3e-13 at 1024^2, 5.1e-13 at 2048^2); twice that
    (9.1e-13 at 2048^2) separates rounding from geometry. Larger meshes than 2048 elements per
    edge therefore tolerate more than the parity bound, in proportion to that rounding noise."""
    x = coor.detach().cpu().numpy() if isinstance(coor, torch.Tensor) else np.asarray(coor)
    c0 = conn[0].detach().cpu().numpy() if isinstance(conn, torch.Tensor) else np.asarray(conn)[0]
    e0 = x[c0]
    h = float(np.min(e0.max(axis=0) - e0.min(axis=0)))
    if not h > 0.0:
        return UNIFORM_RTOL
    return max(UNIFORM_RTOL, 2.0 * np.finfo(np.float64).eps * float(np.abs(x).max()) / h)


def elastic_stress(eps, K, G, sig=None):
    """sigma = K tr(eps) I + 2 G dev(eps) per Gauss point, K and G per element [nelem]
    (plane strain for 2-d tensors; convention of docs/theory/examples/
    cartesian_linear-elasticity.py:146-186)."""
    eps = _dev.dev_f64(eps)
    K = _dev.dev_f64(K)
    G = _dev.dev_f64(G)
    nelem, nip, nd, _ = eps.shape
    if sig is None:
        sig = torch.empty_like(eps)
    _lib.call("gfgpu_elastic_stress", eps.data_ptr(), K.data_ptr(), G.data_ptr(), nelem, nip, nd,
              sig.data_ptr(), _dev.stream())
    return sig


class VelocityVerlet:
    """Explicit dynamics of a linear elastic Quad4/Hex8 mesh, fully device resident.

    Parameters
    ----------
    coor, conn, dofs : mesh tables (host or device)
    K, G : per-element bulk and shear moduli [nelem]
    rho : density (scalar) used for the lumped mass
    dt, eta : time step and nodal viscous damping coefficient
    iip : prescribed (fixed) dofs, or None
    fext : external force nodevec, or None
    uniform : "auto" (detect congruent axis-aligned elements), True or False
    arithmetic : "fp64" (default: FP64 kernels) or "pair": the increments run in float-float
        arithmetic (two FP32 numbers per value, ~48-bit significands; gfgpu_verlet_precompute_pair):
        one fused kernel per increment on a Mesh::Quad4::Regular mesh of square elements with
        lumped-mass classes, an element kernel (square closed form or stored element stiffness)
        and a dof-CSR node kernel on any other Quad4 mesh; agreement with the FP64 path ~1e-14 per
        increment. Hex8 meshes raise with "pair". "mixed" (uniform square Quad4 meshes): the FP64
        state and node kernels, the element forces from the pair closed form on node differences
        formed in FP64 (gfgpu_pcg_precompute_pair), so that an applied affine displacement
        cancels as in FP64.
    """

    def __init__(self, coor, conn, dofs, K, G, rho=1.0, dt=None, eta=0.0, iip=None, fext=None,
                 uniform="auto", arithmetic="fp64"):
        from .vector import Vector
        from .matrix import MatrixDiagonal, MatrixDiagonalPartitioned

        conn_h = _dev.host_i32(conn)
        dofs_h = _dev.host_i32(dofs)
        nelem, nne = conn_h.shape
        nnode, nd = dofs_h.shape
        self.nelem, self.nnode, self.nne, self.ndim = nelem, nnode, nne, nd
        E = Quad4 if nne == 4 else Hex8
        self.vector = Vector(conn_h, dofs_h)
        x = self.vector.AsElement(_dev.dev_f64(coor))
        self.quad = E.Quadrature(x)
        nodal = E.Quadrature(x, E.Nodal.xi(), E.Nodal.w())
        rho_q = torch.full((nelem, nodal.nip()), float(rho), dtype=torch.float64,
                           device=_dev.device())
        # lumped mass: the element matrices' diagonals only (checked diagonal on the fly), no
        # [nelem, nne*ndim, nne*ndim] intermediate
        Md = nodal.Int_N_scalar_NT_dV_diag(rho_q)
        if iip is None or len(iip) == 0:
            self.mass = MatrixDiagonal(conn_h, dofs_h)
            part = dofs_h
            nnu = self.mass.ndof()
        else:
            self.mass = MatrixDiagonalPartitioned(conn_h, dofs_h, iip)
            part = self.mass.part()
            nnu = self.mass.nnu()
        self.mass.assemble_diagonal(Md)
        inv = self.mass.inverse()
        del Md, nodal, rho_q
        self.part_d = _dev.dev_i32(part)
        self.inv = inv
        self.K = _dev.dev_f64(K)
        self.G = _dev.dev_f64(G)
        self.fext = None if fext is None else _dev.dev_f64(fext)
        self.dt = float(dt)
        self.eta = float(eta)

        d = _lib.VerletDesc()
        d.nelem, d.nnode, d.nne, d.ndim, d.nip = nelem, nnode, nne, nd, self.quad.nip()
        d.conn = self.vector.conn_d.data_ptr()
        d.dofs = self.vector.dofs_d.data_ptr()
        d.csr_ptr = self.vector.csr_ptr.data_ptr()
        d.csr_idx = self.vector.csr_idx.data_ptr()
        d.part = self.part_d.data_ptr()
        d.nnu = nnu
        d.inv = self.inv.data_ptr()
        d.dNx = self.quad.GradN().data_ptr()
        d.vol = self.quad.dV().data_ptr()
        d.K = self.K.data_ptr()
        d.G = self.G.data_ptr()
        d.fext = None if self.fext is None else self.fext.data_ptr()
        d.dt, d.eta = self.dt, self.eta
        d.uniform = 0
        self.desc = d
        if uniform is True or uniform == "auto":
            g0 = self.quad.GradN()[0].detach().cpu().numpy().copy()
            v0 = self.quad.dV()[0].detach().cpu().numpy().copy()
            _lib.call("gfgpu_verlet_detect_uniform", C.addressof(d), g0.ctypes.data,
                      v0.ctypes.data, uniform_rtol(coor, conn_h), _dev.stream())
            if uniform is True and not d.uniform:
                raise RuntimeError("mesh is not a uniform axis-aligned Quad4 mesh")
        self.coef = None
        square = d.uniform and nne == 4 and abs(d.hx - d.hy) <= 1e-12 * d.hx
        cube = (d.uniform and nne == 8 and abs(d.hx - d.hy) <= 1e-12 * d.hx
                and abs(d.hx - d.hz) <= 1e-12 * d.hx)
        if square or cube:
            self.coef = torch.empty((nelem, 4 if square else 8), dtype=torch.float64,
                                    device=_dev.device())
            _lib.call("gfgpu_verlet_precompute", C.addressof(d), self.coef.data_ptr(),
                      _dev.stream())
            d.coef = self.coef.data_ptr()
        self.classify()
        self._ell = None
        if nne == 4:
            if not self._detect_regular(conn_h):
                self._build_ell()
        self.coef_pair = None
        if arithmetic == "pair":
            self.use_pair()
        elif arithmetic == "mixed":
            self.use_mixed()
        elif arithmetic != "fp64":
            raise ValueError("arithmetic must be 'fp64', 'pair' or 'mixed'")
        self._alloc_ws()

    def _alloc_ws(self):
        self.ws = torch.empty(int(_lib.lib().gfgpu_verlet_workspace_bytes(C.addressof(self.desc))) // 8,
                              dtype=torch.float64, device=_dev.device())

    def use_pair(self):
        """Float-float increments (gfgpu_verlet_precompute_pair, for the descriptor as it is now:
        Regular square-element tile kernel, square closed form + CSR, or element stiffness + CSR);
        raises GFGPUError (GFGPU_ERR_UNSUPPORTED) for Hex8 meshes."""
        self.desc.coef_pair = None
        n = int(_lib.lib().gfgpu_verlet_pair_coef_floats(C.addressof(self.desc)))
        cp = torch.empty(max(n, 4), dtype=torch.float32, device=_dev.device())
        _lib.call("gfgpu_verlet_precompute_pair", C.addressof(self.desc), cp.data_ptr(),
                  _dev.stream())
        self.coef_pair = cp
        self.desc.coef_pair = self.coef_pair.data_ptr()
        if hasattr(self, "ws"):
            self._alloc_ws()

    def use_fp64(self):
        """FP64 kernels (the default)."""
        self.desc.coef_pair = None
        self.desc.pcg_pair = None

    def use_mixed(self):
        """FP64 state and node kernels with the element forces of the pair closed form (uniform
        square Quad4 meshes; strict mode ignores it)."""
        self.use_fp64()
        n = int(_lib.lib().gfgpu_pcg_pair_coef_floats(C.addressof(self.desc)))
        if n == 0 or self.desc.nne != 4:
            raise RuntimeError("mixed arithmetic needs a uniform square Quad4 mesh")
        self.coef_mixed = torch.empty(n, dtype=torch.float32, device=_dev.device())
        _lib.call("gfgpu_pcg_precompute_pair", C.addressof(self.desc), self.coef_mixed.data_ptr(),
                  _dev.stream())

    @property
    def arithmetic(self):
        if self.desc.coef_pair:
            return "pair"
        return "mixed" if self.desc.pcg_pair else "fp64"

    @property
    def uniform(self):
        return bool(self.desc.uniform)

    def classify(self):
        """Lumped-mass classes for the closed-form node update (gfgpu_verlet_classify): used
        when the free dofs take at most 16 distinct inverse masses. Returns whether it applies."""
        n = self.desc.nnode * self.desc.ndim
        self._mclass = torch.empty(n, dtype=torch.uint8, device=_dev.device())
        self._mclass_inv = np.zeros(16)
        try:
            _lib.call("gfgpu_verlet_classify", C.addressof(self.desc), self._mclass.data_ptr(),
                      self._mclass_inv.ctypes.data, _dev.stream())
            return True
        except _lib.GFGPUError as e:
            if e.code != -7:
                raise
            self._mclass = None
            return False

    def _detect_regular(self, conn):
        """Mesh::Quad4::Regular numbering (gfgpu_verlet_detect_regular, checked on the device):
        the first element (0, 1, nx + 2, nx + 1) gives nx; the coordinates play no part, so a
        distorted Regular mesh is found too."""
        c0 = conn[0]
        nx = int(c0[3]) - 1
        if (nx > 0 and int(c0[0]) == 0 and int(c0[1]) == 1 and int(c0[2]) == nx + 2
                and self.desc.nelem % nx == 0):
            _lib.call("gfgpu_verlet_detect_regular", C.addressof(self.desc), nx,
                      self.desc.nelem // nx, _dev.stream())
        return self.desc.reg_nx > 0

    def _build_ell(self):
        """The node kernels' gather table (gfgpu_verlet_build_ell): at most 4 element
        contributions per dof; same entries and order as the dof CSR, one 16-byte load."""
        n = self.desc.nnode * self.desc.ndim
        t = torch.empty(max(n, 1) * 4, dtype=torch.int32, device=_dev.device())
        try:
            _lib.call("gfgpu_verlet_build_ell", C.addressof(self.desc), t.data_ptr(), _dev.stream())
            self._ell = t
        except _lib.GFGPUError:
            self.desc.ell = None

    def use_csr_gather(self):
        """Node kernel through the dof CSR even on a Regular mesh, without the gather table (FP64
        kernels)."""
        self.use_fp64()
        self.desc.reg_nx = 0
        self.desc.reg_ny = 0
        self.desc.ell = None

    def use_per_dof_mass(self):
        """Node update with the inverse mass read per dof (no mass classes; FP64 kernels)."""
        self.use_fp64()
        self.desc.mclass = None
        self.desc.mclass_inv = None
        self.desc.ncls = 0

    @property
    def path(self):
        if not self.desc.uniform:
            return "general-pair" if self.desc.coef_pair else "general"
        if self.desc.coef_pair:
            return {1: "uniform-square-pair", 2: "uniform-square-pair-csr"}.get(self.desc.pair_mode, "general-pair")
        if self.desc.pcg_pair and self.desc.nne == 4:
            return "uniform-square-mixed"
        if self.desc.coef:
            return "uniform-square" if self.desc.nne == 4 else "uniform-cube"
        return "uniform"

    def use_general_path(self):
        self.use_fp64()
        self.desc.uniform = 0
        self.desc.coef = None

    def use_uniform_onthefly(self):
        """Uniform closed form with K, G read every increment (no precomputed coefficients)."""
        self.use_fp64()
        self.desc.coef = None

    def step(self, u, v, a, nsteps=1):
        """Advance nsteps increments in place (u, v, a: device nodevec float64)."""
        for t in (u, v, a):
            _dev.check_shape(t, (self.nnode, self.ndim), "VelocityVerlet.step")
            if t.dtype != torch.float64 or not t.is_contiguous() or not t.is_cuda:
                raise ValueError("u, v, a must be contiguous float64 CUDA tensors")
        _lib.call("gfgpu_verlet_step", C.addressof(self.desc), u.data_ptr(), v.data_ptr(),
                  a.data_ptr(), int(nsteps), self.ws.data_ptr(), _dev.stream())

    def Step(self, u, v, a, nsteps=1, out=None):
        """Capital form of step (GooseFEM's allocate-and-return convention): u, v, a are host
        nodevecs (numpy or torch, pinned torch tensors copy asynchronously); the state is copied
        to device buffers of this object, advanced nsteps increments, and returned as a tuple of
        new pinned host tensors (or written into `out`, a previous result). Synchronises."""
        shape = (self.nnode, self.ndim)
        if getattr(self, "_dstate", None) is None:
            self._dstate = [torch.empty(shape, dtype=torch.float64, device=_dev.device())
                            for _ in range(3)]
        for d, h in zip(self._dstate, (u, v, a)):
            h = torch.as_tensor(h, dtype=torch.float64)
            _dev.check_shape(h, shape, "VelocityVerlet.Step")
            d.copy_(h, non_blocking=True)
        self.step(*self._dstate, nsteps)
        if out is None:
            out = tuple(torch.empty(shape, dtype=torch.float64).pin_memory() for _ in range(3))
        for o, d in zip(out, self._dstate):
            o.copy_(d, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out

    def internal_force(self, u, fint=None):
        u = _dev.dev_f64(u)
        if fint is None:
            fint = torch.empty_like(u)
        _lib.call("gfgpu_internal_force", C.addressof(self.desc), u.data_ptr(), fint.data_ptr(),
                  self.ws.data_ptr(), _dev.stream())
        return fint


def critical_dt(K, G, rho=1.0, h=1.0):
    """h / c_max with c = sqrt((K + 4G/3) / rho) (plane-strain P-wave speed)."""
    K = np.asarray(K, dtype=np.float64)
    G = np.asarray(G, dtype=np.float64)
    return h / math.sqrt(float(np.max(K + 4.0 * G / 3.0)) / rho)
