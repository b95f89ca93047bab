"""Learned preconditioner for the matrix-free static solve of a Regular Quad4 mesh.

The network (4 convolution layers 3x3, 32 channels, dilations 1, 2, 4, 1: a 17 x 17 node
receptive field; BF16 weights, FP32 accumulation; kernels in csrc/learned.cu) learns what
`inner` iterations of Jacobi-PCG add to a residual beyond the Jacobi step itself: for a residual
r the target is c - D^-1 r with c = PCG_inner(A, r) from zero (both scaled by the RMS of r).
That map is local (its support grows by one node per iteration), which a local network can
represent. The training pairs come from the plain solver: Jacobi-PCG runs on random loads (body
forces, boundary displacements, smooth fields, point loads) and its residuals are snapshotted.

The loss is the energy norm of the output error, sum e^T A e / sum t^T A t over the crops of a
batch, with A each crop's own stiffness: a network output error of high spatial frequency costs
what it costs the solver, which a mean-squared error under-weights.

The solve is a flexible CG in FP64 (gfgpu_fcg_solve) with two search directions per iteration,
D^-1 r and the network's correction RMS(r) * net(r / RMS(r)), A-orthogonalised against a ring of
earlier directions, with an exact line search along each. The Jacobi direction keeps the solve
convergent whatever the network returns; plain Jacobi-PCG remains the fallback and the check of
the answer (same FP64 true-residual test).
"""

import ctypes as C
import math

import numpy as np
import torch

from . import _dev, _lib
from .statics import ElasticStatic


class NNDesc(C.Structure):
    """Mirror of gfgpu_nn_desc (include/gfgpu.h)."""

    _fields_ = [("weights_bf16", C.c_void_p), ("params_f32", C.c_void_p),
                ("material", C.c_void_p), ("H", C.c_int32), ("W", C.c_int32)]


class CoarseDesc(C.Structure):
    """Mirror of gfgpu_coarse_desc (include/gfgpu.h)."""

    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("hc", C.c_int32), ("ncx", C.c_int32),
                ("ncy", C.c_int32), ("ld", C.c_int32), ("ainv", C.c_void_p), ("rhx", C.c_double),
                ("rlx", C.c_double),
                ("rhy", C.c_double), ("rly", C.c_double)]


def inclusion_material(nx, ny, seed, fraction=0.15, rmin=4.0, rmax=12.0, K0=1.0, G0=0.5, factor=10.0):
    """Two-phase element moduli: matrix (K0, G0) and circular inclusions (x factor), radius
    U[rmin, rmax] elements at seeded random centres, placed until the inclusion area (elements
    whose centre lies in a circle) reaches `fraction`."""
    rng = np.random.default_rng(seed)
    cx = (np.arange(nx) + 0.5)[None, :].repeat(ny, 0)
    cy = (np.arange(ny) + 0.5)[:, None].repeat(nx, 1)
    inside = np.zeros((ny, nx), dtype=bool)
    while inside.mean() < fraction:
        r = rng.uniform(rmin, rmax)
        x0, y0 = rng.uniform(0, nx), rng.uniform(0, ny)
        inside |= (cx - x0) ** 2 + (cy - y0) ** 2 <= r * r
    K = np.where(inside, K0 * factor, K0).ravel()
    G = np.where(inside, G0 * factor, G0).ravel()
    return K, G, inside


def static_bc(mesh, uy_top=-1e-2):
    """Bottom edge fixed, top edge uy prescribed (ux free): (iip, prescribed values)."""
    dofs = mesh.dofs()
    bot, top = mesh.nodesBottomEdge(), mesh.nodesTopEdge()
    iip = np.unique(np.concatenate([dofs[bot, :].ravel(), dofs[top, 1]]))
    xp = np.where(np.isin(iip, dofs[top, 1]), uy_top, 0.0)
    return iip, xp


class LearnedPreconditioner:
    """Network parameters, training pairs, training loop and the preconditioned FCG solve for one
    Regular Quad4 mesh (nx x ny elements, per-element K, G) with prescribed dofs iip."""

    def __init__(self, nx, ny, K, G, iip, seed=0, arithmetic="fp64"):
        from . import mesh as M

        self.nx, self.ny = int(nx), int(ny)
        self.H, self.W = self.ny + 1, self.nx + 1
        m = M.Quad4.Regular(nx, ny)
        self.mesh = m
        # arithmetic "pair": the stiffness action of the solvers' iterations in float-float pairs
        self.static = ElasticStatic(m.coor(), m.conn(), m.dofs(), K, G, iip, arithmetic=arithmetic)
        self.iip = np.asarray(iip)
        dev = _dev.device()
        self.free = torch.ones(self.H * self.W * 2, dtype=torch.bool, device=dev)
        self.free[torch.as_tensor(self.iip, device=dev).long()] = False
        self.nfree = int(self.free.sum())
        # nodal material channels: mean of the adjacent elements' K / max K and G / max G
        Kn = np.zeros(self.H * self.W)
        Gn = np.zeros(self.H * self.W)
        cnt = np.zeros(self.H * self.W)
        conn = m.conn()
        for k in range(4):
            np.add.at(Kn, conn[:, k], K)
            np.add.at(Gn, conn[:, k], G)
            np.add.at(cnt, conn[:, k], 1.0)
        mat = np.stack([Kn / cnt / np.max(K), Gn / cnt / np.max(G)], axis=1).astype(np.float32)
        self.material = torch.as_tensor(mat, device=dev).contiguous()
        # element moduli and free-dof mask for the energy-norm loss
        self.elem_kg = torch.as_tensor(np.stack([np.asarray(K), np.asarray(G)], 1).astype(np.float32),
                                       device=dev).contiguous()
        self.free_f = self.free.float().contiguous()
        self.minv = torch.where(self.free, 1.0 / self.static.diag.reshape(-1),
                                torch.zeros((), dtype=torch.float64, device=dev))
        # parameters: He initialisation, zero biases, a small last layer
        self.P = int(_lib.lib().gfgpu_nn_param_count())
        rng = np.random.default_rng(seed)
        p = np.zeros(self.P, dtype=np.float32)
        for layer, (cin, cout) in enumerate(((4, 32), (32, 32), (32, 32), (32, 2))):
            off = int(_lib.lib().gfgpu_nn_param_offset(layer, 0))
            std = math.sqrt(2.0 / (9 * cin)) * (0.1 if layer == 3 else 1.0)
            p[off:off + 9 * cin * cout] = rng.normal(0.0, std, 9 * cin * cout)
        self.params = torch.as_tensor(p, device=dev)
        self.wbf = self.params.to(torch.bfloat16)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.R = None
        self.T = None
        self.losses = []
        self.coarse = None

    # ------------------------------------------------------------------ helpers
    def _desc(self):
        return C.addressof(self.static.desc)

    def nn_desc(self):
        d = NNDesc()
        d.weights_bf16 = self.wbf.data_ptr()
        d.params_f32 = self.params.data_ptr()
        d.material = self.material.data_ptr()
        d.H, d.W = self.H, self.W
        self._nnd = d
        return d

    def _pcg_ws(self):
        nb = int(_lib.lib().gfgpu_pcg_workspace_bytes(self._desc()))
        return torch.empty(nb // 8 + 1, dtype=torch.float64, device=_dev.device())

    # ------------------------------------------------------------------ training pairs
    def _load(self, kind, gen, x):
        """A random load: the right-hand side (body force) and, in x, prescribed displacements.
        kind 0: uniform body force; 1: random prescribed displacements (boundary-concentrated
        load); 2: smooth random body force (Gaussian filter of white noise, random length);
        3: a few point forces."""
        dev = _dev.device()
        n = self.H * self.W * 2
        b = torch.zeros(n, dtype=torch.float64, device=dev)
        x.zero_()
        if kind == 0:
            b = torch.rand(n, generator=gen, dtype=torch.float64, device=dev) * 2.0 - 1.0
        elif kind == 1:
            iip = torch.as_tensor(self.iip, device=dev).long()
            v = torch.rand(iip.numel(), generator=gen, dtype=torch.float64, device=dev) * 2.0 - 1.0
            if float(torch.rand(1, generator=gen, device=dev)) < 0.5:
                v = torch.full_like(v, float(v[0]))
            x[iip] = v
        elif kind == 2:
            f = torch.randn((2, self.H, self.W), generator=gen, dtype=torch.float64, device=dev)
            L = 2.0 + 10.0 * float(torch.rand(1, generator=gen, device=dev))
            ky = torch.fft.fftfreq(self.H, device=dev, dtype=torch.float64)[:, None]
            kx = torch.fft.fftfreq(self.W, device=dev, dtype=torch.float64)[None, :]
            filt = torch.exp(-(ky ** 2 + kx ** 2) * (L * math.pi) ** 2)
            f = torch.fft.ifft2(torch.fft.fft2(f) * filt).real
            b = f.permute(1, 2, 0).reshape(-1).contiguous()
        else:
            k = int(torch.randint(1, 8, (1,), generator=gen, device=dev))
            idx = torch.randint(0, n, (k,), generator=gen, device=dev)
            b[idx] = torch.randn(k, generator=gen, dtype=torch.float64, device=dev)
        b[~self.free] = 0.0
        return b.contiguous()

    def make_pairs(self, nloads=64, snaps=64, every=16, inner=8, seed=1):
        """(residual, correction) pairs from the plain Jacobi-PCG solver on random loads: for the
        residual r after 0, every, 2 every, ... iterations the target is PCG_inner(A, r) - D^-1 r;
        both are divided by the RMS of r over the free dofs."""
        n = self.H * self.W * 2
        npairs = nloads * snaps
        dev = _dev.device()
        self.R = torch.empty((npairs, self.H, self.W, 2), dtype=torch.float32, device=dev)
        self.T = torch.empty_like(self.R)
        ws1, ws2 = self._pcg_ws(), self._pcg_ws()
        s = _dev.stream()
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        r_ptr = C.c_void_p(0)
        _lib.call("gfgpu_pcg_vector", self._desc(), ws1.data_ptr(), 0, C.addressof(r_ptr))
        r = torch.empty(n, dtype=torch.float64, device=dev)
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        c = torch.zeros(n, dtype=torch.float64, device=dev)
        k = 0
        for load in range(nloads):
            b = self._load(load % 4, gen, x)
            _lib.call("gfgpu_pcg_begin", self._desc(), self.static.diag.data_ptr(), b.data_ptr(),
                      x.data_ptr(), ws1.data_ptr(), s)
            for snap in range(snaps):
                if snap:
                    _lib.call("gfgpu_pcg_iterate", self._desc(), every, x.data_ptr(), ws1.data_ptr(), s)
                _lib.call("gfgpu_memcpy_d2d", r.data_ptr(), r_ptr.value, n * 8)
                sigma = torch.sqrt((r[self.free] ** 2).sum() / self.nfree)
                c.zero_()
                _lib.call("gfgpu_pcg_begin", self._desc(), self.static.diag.data_ptr(), r.data_ptr(),
                          c.data_ptr(), ws2.data_ptr(), s)
                _lib.call("gfgpu_pcg_iterate", self._desc(), inner, c.data_ptr(), ws2.data_ptr(), s)
                self.R[k] = (r / sigma).view(self.H, self.W, 2).float()
                self.T[k] = ((c - self.minv * r) / sigma).view(self.H, self.W, 2).float()
                k += 1
        return npairs

    def _residual(self, x, b):
        """r = b - A x on the free dofs (0 on prescribed), FP64."""
        f = self.static.force(x.view(self.H * self.W, 2)).view(-1)
        return torch.where(self.free, b - f, torch.zeros((), dtype=torch.float64, device=x.device))

    def _apply_free(self, v):
        """(A v) on the free dofs for v that is 0 on the prescribed dofs."""
        f = self.static.force(v.view(self.H * self.W, 2)).view(-1)
        return torch.where(self.free, f, torch.zeros((), dtype=torch.float64, device=v.device))

    def _lambda_max(self, iters=40, seed=5):
        """Largest eigenvalue of D^-1 A_uu (power iteration), cached."""
        if getattr(self, "_lmax", None) is None:
            gen = torch.Generator(device=_dev.device())
            gen.manual_seed(seed)
            v = torch.rand(self.H * self.W * 2, generator=gen, dtype=torch.float64,
                           device=_dev.device()) * self.free
            lam = 0.0
            for _ in range(iters):
                w = self.minv * self._apply_free(v)
                lam = float((v * w).sum() / (v * v).sum())
                v = w / torch.linalg.vector_norm(w)
            self._lmax = 1.05 * lam
        return self._lmax

    def chebyshev(self, r, degree=8, ratio=30.0):
        """Chebyshev semi-iteration for A_uu c = r, Jacobi-preconditioned, on the interval
        [lambda_max / ratio, lambda_max] of D^-1 A_uu: a fixed linear map whose support grows by
        one node per degree (17 x 17 nodes at degree 8)."""
        hi = self._lambda_max()
        lo = hi / ratio
        th, de = 0.5 * (hi + lo), 0.5 * (hi - lo)
        sig = th / de
        rho = 1.0 / sig
        x = torch.zeros_like(r)
        res = r.clone()
        d = self.minv * res / th
        for _ in range(degree):
            x += d
            res -= self._apply_free(d)
            rho_n = 1.0 / (2.0 * sig - rho)
            d = rho_n * rho * d + (2.0 * rho_n / de) * (self.minv * res)
            rho = rho_n
        return x

    def make_pairs_twolevel(self, nloads=64, snaps=48, every=4, seed=1, nkeep=4, target="cheb",
                            degree=8, post=False):
        """(residual, correction) pairs for the network as the fine-level part of the two-level
        preconditioner (coarse_setup first). For each random load the exact solution x* comes
        from the two-level solve to 1e-11; the snapshots x_k are the iterates of the same solver
        restarted every `every` iterations. For r_k = b - A x_k the target is, with target="cheb",
        what `degree` Chebyshev steps add beyond the Jacobi step, chebyshev(r_k) - D^-1 r_k (a
        linear map of the network's receptive field), or, with target="error", what the
        two-level direction misses of the exact error, (x* - x_k) - P A_c^-1 P^T r_k - D^-1 r_k;
        both are divided by the RMS of r_k over the free dofs. post=True takes as r_k the
        residual left after the line search along the two-level direction (the network's input
        in the solve with post=True; target "cheb" only)."""
        if self.coarse is None:
            raise RuntimeError("coarse_setup first")
        npairs = nloads * snaps
        dev = _dev.device()
        self.R = torch.empty((npairs, self.H, self.W, 2), dtype=torch.float32, device=dev)
        self.T = torch.empty_like(self.R)
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        n = self.H * self.W * 2
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        k = 0
        for load in range(nloads):
            b = self._load(load % 4, gen, x)
            xs = x.clone()
            for _ in range(3):  # restarts clear the drift of the recurrence residual
                try:
                    self.fcg(xs, tol=1e-11, use_nn=False, nkeep=nkeep, coarse=True, rhs=b)
                    break
                except _lib.GFGPUError as e:
                    if e.code != -8:
                        raise
            xk = x.clone()
            for snap in range(snaps):
                r = self._residual(xk, b)
                if post:  # the residual after the exact line search along the two-level direction
                    d1 = self.coarse_apply(r) + self.minv * r
                    q1 = self._apply_free(d1)
                    r = r - ((r * d1).sum() / (d1 * q1).sum()) * q1
                sigma = torch.sqrt((r[self.free] ** 2).sum() / self.nfree)
                if target == "cheb":
                    t = self.chebyshev(r, degree) - self.minv * r
                else:
                    t = (xs - xk) - self.coarse_apply(r) - self.minv * r
                self.R[k] = (r / sigma).view(self.H, self.W, 2).float()
                self.T[k] = (t / sigma).view(self.H, self.W, 2).float()
                k += 1
                try:
                    self.fcg(xk, tol=1e-14, use_nn=False, nkeep=nkeep, coarse=True, rhs=b,
                             maxiter=every)
                except _lib.GFGPUError as e:
                    if e.code != -8:  # maxiter reached: the expected exit
                        raise
        return npairs

    # ------------------------------------------------------------------ training
    def train(self, steps=2000, batch=32, crop=64, margin=8, lr=2e-3, seed=2, log_every=0,
              loss="energy"):
        """Adam on random crops of the stored pairs (cosine learning-rate decay). loss: "energy"
        (e^T A e / t^T A t per crop) or "mse"."""
        dev = _dev.device()
        B, S = int(batch), int(crop)
        X = torch.empty((B, S, S, 4), dtype=torch.float32, device=dev)
        Tc = torch.empty((B, S, S, 2), dtype=torch.float32, device=dev)
        energy = loss == "energy"
        Ec = torch.empty((B, S - 1, S - 1, 2), dtype=torch.float32, device=dev) if energy else None
        Fc = torch.empty((B, S, S, 2), dtype=torch.float32, device=dev) if energy else None
        lossv = torch.zeros(1, dtype=torch.float32, device=dev)
        nb = int(_lib.lib().gfgpu_nn_train_workspace_bytes(B, S, S))
        ws = torch.empty(nb // 4 + 64, dtype=torch.float32, device=dev)
        rng = np.random.default_rng(seed)
        npairs = self.R.shape[0]
        s = _dev.stream()
        ptr = lambda t: t.data_ptr() if t is not None else None
        for it in range(steps):
            pos = np.stack([rng.integers(0, npairs, B),
                            rng.integers(-margin, max(self.H - S + margin, -margin) + 1, B),
                            rng.integers(-margin, max(self.W - S + margin, -margin) + 1, B)],
                           axis=1).astype(np.int32)
            pos_d = torch.as_tensor(pos, device=dev)
            _lib.call("gfgpu_nn_gather_crops", self.R.data_ptr(), self.T.data_ptr(),
                      self.material.data_ptr(), self.elem_kg.data_ptr(), self.free_f.data_ptr(),
                      pos_d.data_ptr(), B, S, self.H, self.W, X.data_ptr(), Tc.data_ptr(), ptr(Ec),
                      ptr(Fc), s)
            _lib.call("gfgpu_nn_train_step", self.wbf.data_ptr(), self.params.data_ptr(),
                      X.data_ptr(), Tc.data_ptr(), ptr(Ec), ptr(Fc), B, S, margin,
                      self.grads.data_ptr(), lossv.data_ptr(), ws.data_ptr(), s)
            self.step += 1
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * it / max(steps, 1)))
            _lib.call("gfgpu_nn_adam", self.params.data_ptr(), self.grads.data_ptr(),
                      self.m.data_ptr(), self.v.data_ptr(), self.P, float(max(cur, lr * 0.02)),
                      0.9, 0.999, 1e-8, self.step, self.wbf.data_ptr(), s)
            if log_every and (it % log_every == 0 or it == steps - 1):
                self.losses.append((it, float(lossv.item())))
        return self.losses

    # ------------------------------------------------------------------ solves
    def initial_guess(self, xp):
        n = self.H * self.W * 2
        x = torch.zeros(n, dtype=torch.float64, device=_dev.device())
        x[torch.as_tensor(self.iip, device=x.device).long()] = torch.as_tensor(xp, device=x.device)
        return x

    def coarse_setup(self, hc=16):
        """Two-level correction (gfgpu_coarse_setup): Galerkin matrix of bilinear hats on every
        hc-th node, inverted once. Returns the FP64 coarse matrix (device) for checks."""
        g = CoarseDesc()
        _lib.call("gfgpu_coarse_grid", self.nx, self.ny, int(hc), C.addressof(g))
        nc = g.ncx * g.ncy * 2
        dev = _dev.device()
        self.ainv = torch.empty((nc, g.ld), dtype=torch.float32, device=dev)
        ac = torch.empty((nc, nc), dtype=torch.float64, device=dev)
        nb = int(_lib.lib().gfgpu_coarse_setup_workspace_bytes(self._desc(), C.addressof(g)))
        ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=dev)
        _lib.call("gfgpu_coarse_setup", self._desc(), C.addressof(g), self.ainv.data_ptr(),
                  ac.data_ptr(), ws.data_ptr(), _dev.stream())
        g.ainv = self.ainv.data_ptr()
        self.coarse = g
        return ac

    def coarse_apply(self, r):
        """z = P A_c^-1 P^T r on the free dofs (gfgpu_coarse_apply)."""
        r = _dev.dev_f64(r).contiguous()
        z = torch.empty_like(r)
        nc = self.coarse.ncx * self.coarse.ncy * 2
        ws = torch.empty(2 * ((nc * 8 + 255) // 256 * 256) // 8, dtype=torch.float64,
                         device=r.device)
        _lib.call("gfgpu_coarse_apply", self._desc(), C.addressof(self.coarse), r.data_ptr(),
                  z.data_ptr(), ws.data_ptr(), _dev.stream())
        return z

    def fcg(self, x, tol=1e-8, use_nn=True, maxiter=200000, nkeep=8, check_every=16,
            coarse=False, rhs=None, post=False):
        """Flexible CG (gfgpu_fcg_solve) in place on x (prescribed values + initial guess): with
        the network, two directions per iteration (D^-1 r and the network's correction); without,
        Jacobi only. coarse=True adds the two-level correction to the first direction
        (gfgpu_fcg_solve_coarse; coarse_setup first), which also takes an external load `rhs`;
        post=True applies the network to the residual left after the two-level step. Returns
        (iterations, relative true residual)."""
        ndir = 2 if use_nn else 1
        if coarse:
            nb = int(_lib.lib().gfgpu_fcg_coarse_workspace_bytes(
                self._desc(), self.H, self.W, nkeep, ndir, C.addressof(self.coarse)))
        else:
            nb = int(_lib.lib().gfgpu_fcg_workspace_bytes(self._desc(), self.H, self.W, nkeep, ndir))
        if nb <= 0:
            raise ValueError("nkeep out of range")
        ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=_dev.device())
        it = C.c_int64(0)
        rel = C.c_double(0.0)
        nnd = C.addressof(self.nn_desc()) if use_nn else None
        if coarse:
            _lib.call("gfgpu_fcg_solve_coarse", self._desc(), self.static.diag.data_ptr(), nnd,
                      C.addressof(self.coarse), int(bool(post)),
                      None if rhs is None else rhs.data_ptr(),
                      x.data_ptr(), float(tol), int(maxiter), int(nkeep),
                      int(check_every), ws.data_ptr(), _dev.stream(), C.addressof(it),
                      C.addressof(rel))
        else:
            _lib.call("gfgpu_fcg_solve", self._desc(), self.static.diag.data_ptr(), nnd,
                      x.data_ptr(), float(tol), int(maxiter), int(nkeep), int(check_every),
                      ws.data_ptr(), _dev.stream(), C.addressof(it), C.addressof(rel))
        return int(it.value), float(rel.value)

    def solve(self, x, tol=1e-8, maxiter=20000, nkeep=2, check_every=4):
        """The learned solve with Jacobi-PCG as its fallback: when the flexible CG with the
        network does not reach tol within maxiter iterations, Jacobi-PCG continues from its
        iterate. After coarse_setup the solve is the two-level one with the network as the
        post-smoother of the two-level step (train it on make_pairs_twolevel(post=True) pairs).
        Returns (network iterations, fallback iterations, relative true residual)."""
        x0 = x.clone()
        two = self.coarse is not None
        try:
            it, rel = self.fcg(x, tol=tol, use_nn=True, maxiter=maxiter, nkeep=nkeep,
                               check_every=check_every, coarse=two, post=two)
            return it, 0, rel
        except _lib.GFGPUError as e:
            if e.code not in (-8, -5):  # not converged / non-finite residual
                raise
        if not bool(torch.isfinite(x).all()):
            x.copy_(x0)
        itf, rel = self.jacobi_pcg(x, tol=tol)
        return maxiter, itf, rel

    def jacobi_pcg(self, x, tol=1e-8, check_every=16):
        return self.static.solve(x.view(self.H * self.W, 2), tol=tol, check_every=check_every)
