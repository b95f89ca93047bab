"""The learned preconditioner: the network's training kernels (mean-squared and energy-norm
losses) against the FP64 numpy oracle (oracle/nn.py), the crop gather, the tensor-core inference
against the FP32 path, the flexible CG against the direct solve, and what the trained network
gains over the same solver without it."""

import numpy as np
import pytest
import torch

from _common import rel_err

pytestmark = pytest.mark.gpu

DILS = (1, 2, 4, 1)
SHAPES = ((4, 32), (32, 32), (32, 32), (32, 2))


@pytest.fixture(scope="module")
def L():
    import goosefem_gb300  # noqa: F401  (loads the library)
    from goosefem_gb300 import _lib

    return _lib


def _random_params(L, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    P = int(L.lib().gfgpu_nn_param_count())
    p = np.zeros(P, dtype=np.float32)
    for k, (ci, co) in enumerate(SHAPES):
        w0 = int(L.lib().gfgpu_nn_param_offset(k, 0))
        b0 = int(L.lib().gfgpu_nn_param_offset(k, 1))
        p[w0:w0 + 9 * ci * co] = rng.normal(0, scale * np.sqrt(2.0 / (9 * ci)), 9 * ci * co)
        p[b0:b0 + co] = rng.normal(0, 0.1, co)
    pt = torch.as_tensor(p, device="cuda")
    wb = pt.to(torch.bfloat16)
    return pt, wb


def _oracle_params(L, pt, wb):
    """W as the BF16 values the kernels use (in FP64), biases FP32 -> FP64."""
    wq = wb.float().cpu().numpy().astype(np.float64)
    pf = pt.cpu().numpy().astype(np.float64)
    out = []
    for k, (ci, co) in enumerate(SHAPES):
        w0 = int(L.lib().gfgpu_nn_param_offset(k, 0))
        b0 = int(L.lib().gfgpu_nn_param_offset(k, 1))
        out.append((wq[w0:w0 + 9 * ci * co].reshape(9, ci, co), pf[b0:b0 + co]))
    return out


def test_training_gradients_match_oracle(L):
    from oracle import nn as O

    B, S, margin = 2, 14, 2
    pt, wb = _random_params(L, 0)
    rng = np.random.default_rng(1)
    X = rng.normal(size=(B, S, S, 4)).astype(np.float32)
    T = rng.normal(size=(B, S, S, 2)).astype(np.float32)
    Xd, Td = torch.as_tensor(X, device="cuda"), torch.as_tensor(T, device="cuda")
    grads = torch.zeros_like(pt)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    nb = int(L.lib().gfgpu_nn_train_workspace_bytes(B, S, S))
    ws = torch.empty(nb // 4 + 64, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    L.call("gfgpu_nn_train_step", wb.data_ptr(), pt.data_ptr(), Xd.data_ptr(), Td.data_ptr(), None,
           None, B, S, margin, grads.data_ptr(), loss.data_ptr(), ws.data_ptr(), s)
    params = _oracle_params(L, pt, wb)
    mask = np.zeros((B, S, S))
    mask[:, margin:S - margin, margin:S - margin] = 1.0
    lref, gref = O.loss_and_grads(X.astype(np.float64), T.astype(np.float64), mask, params, DILS)
    assert abs(float(loss.item()) - lref) <= 1e-5 * abs(lref)
    g = grads.cpu().numpy().astype(np.float64)
    for k, (ci, co) in enumerate(SHAPES):
        w0 = int(L.lib().gfgpu_nn_param_offset(k, 0))
        b0 = int(L.lib().gfgpu_nn_param_offset(k, 1))
        assert rel_err(g[w0:w0 + 9 * ci * co].reshape(9, ci, co), gref[k][0]) <= 1e-4, k
        assert rel_err(g[b0:b0 + co], gref[k][1]) <= 1e-4, k
    # the same step twice gives the same bits (fixed-order reductions)
    g1 = grads.clone()
    L.call("gfgpu_nn_train_step", wb.data_ptr(), pt.data_ptr(), Xd.data_ptr(), Td.data_ptr(), None,
           None, B, S, margin, grads.data_ptr(), loss.data_ptr(), ws.data_ptr(), s)
    assert torch.equal(g1, grads)


def test_energy_loss_gradients_match_oracle(L):
    """Energy-norm loss sum e^T A e / sum t^T A t over the crops (A assembled by the oracle's
    element integrals) and its gradients, with empty elements and prescribed dofs in the crops."""
    from oracle import nn as O

    B, S, margin = 3, 12, 2
    pt, wb = _random_params(L, 5)
    rng = np.random.default_rng(6)
    X = rng.normal(size=(B, S, S, 4)).astype(np.float32)
    T = rng.normal(size=(B, S, S, 2)).astype(np.float32)
    E = np.stack([rng.uniform(0.5, 10.0, (B, S - 1, S - 1)), rng.uniform(0.25, 5.0, (B, S - 1, S - 1))],
                 -1).astype(np.float32)
    E[0, :, :3] = 0.0  # outside the mesh
    F = (rng.uniform(size=(B, S, S, 2)) > 0.15).astype(np.float32)
    F[0, :, :3] = 0.0
    d = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    Xd, Td, Ed, Fd = d(X), d(T), d(E), d(F)
    grads = torch.zeros_like(pt)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    nb = int(L.lib().gfgpu_nn_train_workspace_bytes(B, S, S))
    ws = torch.empty(nb // 4 + 64, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    L.call("gfgpu_nn_train_step", wb.data_ptr(), pt.data_ptr(), Xd.data_ptr(), Td.data_ptr(),
           Ed.data_ptr(), Fd.data_ptr(), B, S, margin, grads.data_ptr(), loss.data_ptr(),
           ws.data_ptr(), s)
    lref, gref = O.energy_loss_and_grads(X.astype(np.float64), T.astype(np.float64),
                                         E.astype(np.float64), F.astype(np.float64), margin,
                                         _oracle_params(L, pt, wb), DILS)
    assert abs(float(loss.item()) - lref) <= 1e-5 * abs(lref)
    g = grads.cpu().numpy().astype(np.float64)
    for k, (ci, co) in enumerate(SHAPES):
        w0 = int(L.lib().gfgpu_nn_param_offset(k, 0))
        b0 = int(L.lib().gfgpu_nn_param_offset(k, 1))
        assert rel_err(g[w0:w0 + 9 * ci * co].reshape(9, ci, co), gref[k][0]) <= 1e-4, k
        assert rel_err(g[b0:b0 + co], gref[k][1]) <= 1e-4, k


def test_gather_crops(L):
    """Crops of pairs, material, element moduli and free masks, zero outside the mesh."""
    H, W, npairs, B, S = 9, 11, 3, 4, 6
    rng = np.random.default_rng(8)
    R = rng.normal(size=(npairs, H, W, 2)).astype(np.float32)
    T = rng.normal(size=(npairs, H, W, 2)).astype(np.float32)
    mat = rng.normal(size=(H, W, 2)).astype(np.float32)
    ekg = rng.normal(size=((H - 1) * (W - 1), 2)).astype(np.float32)
    free = (rng.uniform(size=H * W * 2) > 0.3).astype(np.float32)
    pos = np.array([[0, -2, -3], [2, 4, 7], [1, 0, 0], [2, -5, 9]], dtype=np.int32)
    Rd, Td, md, ed, fd, pd = (torch.as_tensor(a, device="cuda") for a in (R, T, mat, ekg, free, pos))
    X = torch.full((B, S, S, 4), 7.0, device="cuda")
    Tc = torch.full((B, S, S, 2), 7.0, device="cuda")
    Ec = torch.full((B, S - 1, S - 1, 2), 7.0, device="cuda")
    Fc = torch.full((B, S, S, 2), 7.0, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    L.call("gfgpu_nn_gather_crops", Rd.data_ptr(), Td.data_ptr(), md.data_ptr(), ed.data_ptr(),
           fd.data_ptr(), pd.data_ptr(), B, S, H, W, X.data_ptr(), Tc.data_ptr(), Ec.data_ptr(),
           Fc.data_ptr(), s)
    torch.cuda.synchronize()
    Xe = np.zeros((B, S, S, 4), np.float32)
    Te = np.zeros((B, S, S, 2), np.float32)
    Ee = np.zeros((B, S - 1, S - 1, 2), np.float32)
    Fe = np.zeros((B, S, S, 2), np.float32)
    ek = ekg.reshape(H - 1, W - 1, 2)
    fr = free.reshape(H, W, 2)
    for b, (k, y0, x0) in enumerate(pos):
        for y in range(S):
            for x in range(S):
                yy, xx = y0 + y, x0 + x
                if 0 <= yy < H and 0 <= xx < W:
                    Xe[b, y, x] = np.concatenate([R[k, yy, xx], mat[yy, xx]])
                    Te[b, y, x] = T[k, yy, xx]
                    Fe[b, y, x] = fr[yy, xx]
                if y < S - 1 and x < S - 1 and 0 <= yy < H - 1 and 0 <= xx < W - 1:
                    Ee[b, y, x] = ek[yy, xx]
    for got, exp in ((X, Xe), (Tc, Te), (Ec, Ee), (Fc, Fe)):
        assert np.array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("H,W", [(37, 45), (29, 301)])
def test_tensor_core_inference_matches_fp32_and_oracle(L, H, W):
    """Inference with the 32 -> 32 layers on tcgen05 (TMEM accumulators) and on mma.sync against
    the FP32 CUDA-core path and the FP64 oracle; grids narrower and wider than the 128-pixel
    tcgen05 tile, with a partial last tile."""
    from oracle import nn as O
    from goosefem_gb300.learned import NNDesc
    import ctypes as C

    pt, wb = _random_params(L, 3, scale=0.8)
    rng = np.random.default_rng(4)
    X0 = rng.normal(size=(H, W, 4)).astype(np.float32)
    Xd = torch.as_tensor(X0, device="cuda")
    mat = torch.zeros((H, W, 2), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    # FP32 path
    y32 = torch.empty((H, W, 2), dtype=torch.float32, device="cuda")
    nb = int(L.lib().gfgpu_nn_train_workspace_bytes(1, H, W))
    ws = torch.empty(nb // 4 + 64, dtype=torch.float32, device="cuda")
    L.call("gfgpu_nn_forward", wb.data_ptr(), pt.data_ptr(), Xd.data_ptr(), 1, H, W, y32.data_ptr(),
           ws.data_ptr(), s)
    # tensor-core path
    d = NNDesc()
    d.weights_bf16, d.params_f32, d.material, d.H, d.W = wb.data_ptr(), pt.data_ptr(), mat.data_ptr(), H, W
    nbi = int(L.lib().gfgpu_nn_infer_workspace_bytes(H, W))
    ws2 = torch.empty(nbi // 8 + 1, dtype=torch.float64, device="cuda")
    yref, _ = O.forward(X0[None].astype(np.float64), _oracle_params(L, pt, wb), DILS)
    assert rel_err(y32.cpu().numpy(), yref[0]) <= 1e-5
    out = {}
    try:
        for path in (0, 1, 2, 3):  # mma.sync, tcgen05, tcgen05 + TMA pipeline, + row reuse
            L.call("gfgpu_set_nn_tensor_path", path)
            ytc = torch.full((H, W, 2), float("nan"), dtype=torch.float32, device="cuda")
            L.call("gfgpu_nn_infer", C.addressof(d), Xd.data_ptr(), ytc.data_ptr(), ws2.data_ptr(), s)
            L.call("gfgpu_nn_tc_status")
            out[path] = ytc.cpu().numpy()
            # BF16 activations between the layers: agreement to the BF16 rounding level
            assert np.all(np.isfinite(out[path]))
            assert rel_err(out[path], yref[0]) <= 3e-2, path
    finally:
        L.call("gfgpu_set_nn_tensor_path", 2)  # the default
    # same products, different FP32 summation order
    assert rel_err(out[0], out[1]) <= 1e-2
    assert rel_err(out[0], out[2]) <= 1e-2
    # paths 2 and 3 run the same MMAs on the same rows in the same order
    assert np.array_equal(out[2], out[3])


@pytest.mark.parametrize("H,W", [(37, 45), (513, 513)])
def test_dependent_launches_give_the_same_bits(L, H, W):
    """The default network chain (path 2: tcgen05 + TMA layers) launched with programmatic
    dependent launch and with ordinary stream-ordered launches: identical bits, repeatedly (a layer
    that read its predecessor's output before griddepcontrol.wait, or wrote before it, would show
    up as a difference or as run-to-run variation)."""
    from goosefem_gb300.learned import NNDesc
    import ctypes as C

    pt, wb = _random_params(L, 5, scale=0.8)
    X0 = np.random.default_rng(6).normal(size=(H, W, 4)).astype(np.float32)
    Xd = torch.as_tensor(X0, device="cuda")
    mat = torch.zeros((H, W, 2), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    d = NNDesc()
    d.weights_bf16, d.params_f32, d.material, d.H, d.W = wb.data_ptr(), pt.data_ptr(), mat.data_ptr(), H, W
    ws = torch.empty(int(L.lib().gfgpu_nn_infer_workspace_bytes(H, W)) // 8 + 1, dtype=torch.float64,
                     device="cuda")
    out = []
    try:
        L.call("gfgpu_set_nn_tensor_path", 2)
        for pdl in (1, 0, 1, 0):
            L.call("gfgpu_set_nn_pdl", pdl)
            y = torch.full((H, W, 2), float("nan"), dtype=torch.float32, device="cuda")
            for _ in range(3):  # back-to-back applications: each one's first layer follows the last
                L.call("gfgpu_nn_infer", C.addressof(d), Xd.data_ptr(), y.data_ptr(), ws.data_ptr(), s)
            L.call("gfgpu_nn_tc_status")
            out.append(y.cpu().numpy())
    finally:
        L.call("gfgpu_set_nn_pdl", 1)
    assert np.all(np.isfinite(out[0]))
    for o in out[1:]:
        assert np.array_equal(o, out[0])


@pytest.fixture(scope="module")
def small_problem():
    from goosefem_gb300 import learned as LR
    from goosefem_gb300 import mesh as M

    nx = ny = 48
    K, G, _ = LR.inclusion_material(nx, ny, 7, rmin=2.0, rmax=5.0)
    m = M.Quad4.Regular(nx, ny)
    iip, xp = LR.static_bc(m)
    return nx, ny, K, G, iip, xp


def _direct(nx, ny, K, G, iip, xp):
    from oracle import gfref as R
    from oracle import statics as S

    coor, conn = R.quad4_regular(nx, ny)
    A = S.stiffness(coor, conn, K, G)
    return A, S.solve_partitioned(A, iip, xp)


def test_fcg_jacobi_matches_direct_solve(small_problem):
    from goosefem_gb300 import learned as LR
    from oracle import statics as S

    nx, ny, K, G, iip, xp = small_problem
    lp = LR.LearnedPreconditioner(nx, ny, K, G, iip)
    A, xr = _direct(nx, ny, K, G, iip, xp)
    x2 = lp.initial_guess(xp)
    it2, _ = lp.jacobi_pcg(x2)
    # the ring-based flexible CG with the Jacobi direction alone is Jacobi-PCG (exact
    # arithmetic), for any ring length, eager and replayed as a CUDA graph
    for nkeep, check_every in ((1, 1), (1, 16), (8, 16), (3, 5)):
        x = lp.initial_guess(xp)
        it, rel = lp.fcg(x, use_nn=False, nkeep=nkeep, check_every=check_every)
        xg = x.cpu().numpy()
        assert rel <= 1e-8 and S.residual(A, iip, xg) <= 1e-8
        assert np.linalg.norm(xg - xr) / np.linalg.norm(xr) <= 1e-6
        assert abs(it - it2) <= max(16, it2 // 20), (nkeep, it, it2)
    # the same call twice gives the same bits (fixed-order reductions, graph replay)
    xa, xb = lp.initial_guess(xp), lp.initial_guess(xp)
    lp.fcg(xa, use_nn=False, nkeep=4)
    lp.fcg(xb, use_nn=False, nkeep=4)
    assert torch.equal(xa, xb)


def test_untrained_network_still_converges(small_problem):
    """The Jacobi direction keeps the two-direction solve convergent with a network that has
    not been trained (random weights)."""
    from goosefem_gb300 import learned as LR
    from oracle import statics as S

    nx, ny, K, G, iip, xp = small_problem
    lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=3)
    x = lp.initial_guess(xp)
    it, rel = lp.fcg(x, use_nn=True, maxiter=5000)
    A, _ = _direct(nx, ny, K, G, iip, xp)
    assert rel <= 1e-8 and S.residual(A, iip, x.cpu().numpy()) <= 1e-8


def test_trained_network_reduces_iterations(small_problem):
    """What the trained network gains over the same flexible CG without it (Jacobi)."""
    from goosefem_gb300 import learned as LR
    from oracle import statics as S

    nx, ny, K, G, iip, xp = small_problem
    lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=0)
    lp.make_pairs(nloads=16, snaps=16, every=8, inner=8, seed=1)
    losses = lp.train(steps=1200, batch=16, crop=40, margin=8, lr=2e-3, log_every=100)
    assert losses[-1][1] < losses[0][1]
    x_nn = lp.initial_guess(xp)
    it_nn, fb, rel_nn = lp.solve(x_nn, nkeep=8, check_every=16)
    assert fb == 0  # no fallback needed
    x_j = lp.initial_guess(xp)
    it_j, rel_j = lp.fcg(x_j, use_nn=False)
    A, xr = _direct(nx, ny, K, G, iip, xp)
    xg = x_nn.cpu().numpy()
    assert rel_nn <= 1e-8 and S.residual(A, iip, xg) <= 1e-8  # FP64 answer, same tolerance
    assert np.linalg.norm(xg - xr) / np.linalg.norm(xr) <= 1e-6
    assert it_nn < it_j, (it_nn, it_j)


def test_chebyshev_target_matches_restatement(small_problem):
    """The training target of the two-level network, `degree` Jacobi-preconditioned Chebyshev
    steps, against the same recurrence on the scipy stiffness."""
    from goosefem_gb300 import learned as LR

    nx, ny, K, G, iip, xp = small_problem
    lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=0)
    A, _ = _direct(nx, ny, K, G, iip, xp)
    free = np.ones(A.shape[0], dtype=bool)
    free[iip] = False
    Dinv = np.where(free, 1.0 / A.diagonal(), 0.0)
    r = np.random.default_rng(8).standard_normal(A.shape[0]) * free
    got = lp.chebyshev(torch.as_tensor(r, device="cuda"), degree=8).cpu().numpy()
    hi = lp._lambda_max()
    lo = hi / 30.0
    th, de = 0.5 * (hi + lo), 0.5 * (hi - lo)
    sig = th / de
    rho = 1.0 / sig
    x = np.zeros_like(r)
    res = r.copy()
    d = Dinv * res / th
    for _ in range(8):
        x += d
        res -= free * (A @ d)
        rho_n = 1.0 / (2.0 * sig - rho)
        d = rho_n * rho * d + (2.0 * rho_n / de) * (Dinv * res)
        rho = rho_n
    assert rel_err(got, x) <= 1e-10


def test_trained_network_reduces_twolevel_iterations():
    """What the trained network gains in the two-level solve: the same flexible CG with the
    two-level direction, with and without the network's post-smoothing direction."""
    from goosefem_gb300 import learned as LR
    from goosefem_gb300 import mesh as M
    from oracle import statics as S

    nx = ny = 128
    K, G, _ = LR.inclusion_material(nx, ny, 11, rmin=2.0, rmax=6.0)
    iip, xp = LR.static_bc(M.Quad4.Regular(nx, ny))
    lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=0)
    lp.coarse_setup(8)
    x_2l = lp.initial_guess(xp)
    it_2l, _ = lp.fcg(x_2l, use_nn=False, nkeep=1, coarse=True)
    lp.make_pairs_twolevel(nloads=16, snaps=24, every=3, target="cheb", degree=8, post=True)
    losses = lp.train(steps=1500, batch=16, crop=48, margin=8, lr=2e-3, log_every=100)
    assert losses[-1][1] < 0.5 * losses[0][1]
    x_nn = lp.initial_guess(xp)
    it_nn, fb, rel_nn = lp.solve(x_nn, nkeep=4)
    assert fb == 0
    # the same solve with the network's layers launched without dependent launches: same bits
    from goosefem_gb300 import _lib as L

    try:
        L.call("gfgpu_set_nn_pdl", 0)
        x_np = lp.initial_guess(xp)
        it_np, fb_np, _ = lp.solve(x_np, nkeep=4)
    finally:
        L.call("gfgpu_set_nn_pdl", 1)
    assert (it_np, fb_np) == (it_nn, fb) and torch.equal(x_np, x_nn)
    A, xr = _direct(nx, ny, K, G, iip, xp)
    xg = x_nn.cpu().numpy()
    assert rel_nn <= 1e-8 and S.residual(A, iip, xg) <= 1e-8
    assert np.linalg.norm(xg - xr) / np.linalg.norm(xr) <= 1e-6
    assert it_nn < 0.8 * it_2l, (it_nn, it_2l)
