"""Static linear elastic solve with prescribed displacements, matrix-free on the GPU.

The reference solves A_uu x_u = b_u - A_up x_p with an assembled sparse matrix and a direct
factorisation (MatrixPartitioned.h:526-642). Here the stiffness action is the element kernel of the
explicit step plus the deterministic CSR gather, and the solve is Jacobi-preconditioned CG in FP64
(gfgpu_pcg_solve), optionally with the stiffness action in float-float arithmetic.
"""

import ctypes as C

import numpy as np
import torch

from . import _dev, _lib
from . import mesh as _mesh
from .element import Quad4, Hex8
from .dynamics import uniform_rtol


class ElasticStatic:
    """Matrix-free linear elastic operator of a Quad4/Hex8 mesh with prescribed dofs `iip`.

    K, G: per-element bulk and shear moduli. uniform: "auto" | True | False (closed-form element
    kernel for congruent axis-aligned elements, see gfgpu_verlet_detect_uniform).
    arithmetic: "fp64" (default) or "pair": the Jacobi-PCG (and flexible CG) iterations apply the
    stiffness in float-float arithmetic (gfgpu_pcg_precompute_pair; Regular cube Hex8 meshes and
    uniform square Quad4 meshes), everything else (solution, residuals, dot products, the initial
    and the true final residual) in FP64."""

    def __init__(self, coor, conn, dofs, K, G, iip, uniform="auto", arithmetic="fp64"):
        from .vector import Vector

        conn_h = _dev.host_i32(conn)
        dofs_h = _dev.host_i32(dofs)
        nelem, nne = conn_h.shape
        nnode, nd = dofs_h.shape
        self.nelem, self.nnode, self.nne, self.ndim = nelem, nnode, nne, nd
        E = Quad4 if nne == 4 else Hex8
        self.vector = Vector(conn_h, dofs_h)
        self.quad = E.Quadrature(self.vector.AsElement(_dev.dev_f64(coor)))
        self.iip = _dev.host_i32(iip)
        self.iiu, part = _mesh.partition(dofs_h, self.iip)
        self.part_d = _dev.dev_i32(part)
        self.K = _dev.dev_f64(K)
        self.G = _dev.dev_f64(G)
        d = _lib.VerletDesc()
        d.nelem, d.nnode, d.nne, d.ndim, d.nip = nelem, nnode, nne, nd, self.quad.nip()
        d.conn = self.vector.conn_d.data_ptr()
        d.dofs = self.vector.dofs_d.data_ptr()
        d.csr_ptr = self.vector.csr_ptr.data_ptr()
        d.csr_idx = self.vector.csr_idx.data_ptr()
        d.part = self.part_d.data_ptr()
        d.nnu = int(self.iiu.size)
        d.dNx = self.quad.GradN().data_ptr()
        d.vol = self.quad.dV().data_ptr()
        d.K = self.K.data_ptr()
        d.G = self.G.data_ptr()
        d.dt = 1.0
        d.uniform = 0
        self.desc = d
        if uniform is True or uniform == "auto":
            g0 = self.quad.GradN()[0].detach().cpu().numpy().copy()
            v0 = self.quad.dV()[0].detach().cpu().numpy().copy()
            _lib.call("gfgpu_verlet_detect_uniform", C.addressof(d), g0.ctypes.data,
                      v0.ctypes.data, uniform_rtol(coor, conn_h), _dev.stream())
            if uniform is True and not d.uniform:
                raise RuntimeError("mesh is not uniform")
        # square Quad4 / cube Hex8 elements: precomputed per-element coefficients (34 / ~171 FP64
        # instructions per element in the operator instead of recombining K, G every application)
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
        # Mesh::Quad4/Hex8::Regular numbering with plain dofs: the operator's gather by index
        # arithmetic (gfgpu_verlet_detect_regular(_hex8), checked on the device; same bits as the
        # CSR)
        if nne == 8 and nd == 3:
            c = np.asarray(coor)
            nxg = int(np.argmax(c[:, 1] != c[0, 1])) if np.any(c[:, 1] != c[0, 1]) else c.shape[0]
            nyg = int(np.argmax(c[:, 2] != c[0, 2])) // max(nxg, 1) if np.any(c[:, 2] != c[0, 2]) else 0
            nx, ny = nxg - 1, nyg - 1
            if nx > 0 and ny > 0 and nelem % (nx * ny) == 0:
                _lib.call("gfgpu_verlet_detect_regular_hex8", C.addressof(d), nx, ny,
                          nelem // (nx * ny), _dev.stream())
        if nne == 4 and nd == 2:
            y = np.asarray(coor)[:, 1]
            run = int(np.argmax(y != y[0])) if np.any(y != y[0]) else y.size
            nx = run - 1
            if nx > 0 and nelem % nx == 0:
                _lib.call("gfgpu_verlet_detect_regular", C.addressof(d), nx, nelem // nx,
                          _dev.stream())
        self.coef_pair = None
        if arithmetic == "pair":
            self.use_pair()
        elif arithmetic != "fp64":
            raise ValueError("arithmetic must be 'fp64' or 'pair'")
        nbytes = int(_lib.lib().gfgpu_pcg_workspace_bytes(C.addressof(d)))
        self.ws = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=_dev.device())
        self.diag = torch.empty((nnode, nd), dtype=torch.float64, device=_dev.device())
        _lib.call("gfgpu_elastic_diagonal", C.addressof(d), self.diag.data_ptr(),
                  self.ws.data_ptr(), _dev.stream())

    def use_pair(self):
        """Float-float stiffness action in the PCG iterations (Regular cube Hex8 meshes, uniform
        square Quad4 meshes)."""
        n = int(_lib.lib().gfgpu_pcg_pair_coef_floats(C.addressof(self.desc)))
        if n == 0:
            raise RuntimeError("the pair operator needs a Regular cube Hex8 mesh (uniform, "
                               "index-arithmetic gather) or a uniform square Quad4 mesh")
        self.coef_pair = torch.empty(n, dtype=torch.float32, device=_dev.device())
        _lib.call("gfgpu_pcg_precompute_pair", C.addressof(self.desc), self.coef_pair.data_ptr(),
                  _dev.stream())

    def use_fp64(self):
        """FP64 stiffness action in the PCG iterations."""
        self.desc.pcg_pair = None
        self.coef_pair = None

    @property
    def arithmetic(self):
        return "pair" if self.desc.pcg_pair else "fp64"

    def use_csr_gather(self):
        """Gather the operator's element forces through the dof CSR even on a Regular mesh."""
        self.use_fp64()
        self.desc.reg_nx = 0
        self.desc.reg_ny = 0
        self.desc.reg_nz = 0

    @property
    def uniform(self):
        return bool(self.desc.uniform)

    def use_general_path(self):
        self.use_fp64()
        self.desc.uniform = 0

    def force(self, u):
        """Internal force (= stiffness action) of a displacement nodevec."""
        u = _dev.dev_f64(u)
        out = torch.empty_like(u)
        _lib.call("gfgpu_internal_force", C.addressof(self.desc), u.data_ptr(), out.data_ptr(),
                  self.ws.data_ptr(), _dev.stream())
        return out

    def solve(self, x, tol=1e-8, maxiter=100000, check_every=16):
        """Solve in place: x (device nodevec) holds the prescribed values and the initial guess.
        Returns (iterations, relative residual of the true residual)."""
        if not (x.is_cuda and x.dtype == torch.float64 and x.is_contiguous()):
            raise ValueError("x must be a contiguous float64 CUDA tensor")
        _dev.check_shape(x, (self.nnode, self.ndim), "solve")
        it = C.c_int64(0)
        rel = C.c_double(0.0)
        _lib.call("gfgpu_pcg_solve", C.addressof(self.desc), self.diag.data_ptr(), x.data_ptr(),
                  float(tol), int(maxiter), int(check_every), self.ws.data_ptr(), _dev.stream(),
                  C.addressof(it), C.addressof(rel))
        return int(it.value), float(rel.value)
