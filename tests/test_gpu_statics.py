"""GPU matrix-free Jacobi-PCG (static linear elasticity with prescribed displacements) against
the oracle's assembled partitioned direct solve (oracle/statics.py)."""

import os

import numpy as np
import pytest
import torch

from _common import RTOL, rel_err, seeded_field, seeded_material, to_np

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    return gf


def _hex8_case(n, seed):
    from oracle import gfref as R

    coor, conn = R.hex8_regular(n, n, n)
    K, G = seeded_material(n ** 3, seed)
    nxy = (n + 1) ** 2
    front = np.arange(nxy)
    back = front + n * nxy
    iip = np.unique(np.concatenate([(front[:, None] * 3 + np.arange(3)).ravel(), back * 3 + 2]))
    xp = np.where(np.isin(iip, back * 3 + 2), -1e-2, 0.0)
    return coor, conn, K, G, iip, xp


def _solve_gpu(gf, coor, conn, K, G, iip, xp, uniform):
    nnode, nd = coor.shape
    dofs = np.arange(nnode * nd).reshape(nnode, nd)
    st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, iip, uniform=uniform)
    x = torch.zeros((nnode, nd), dtype=torch.float64, device="cuda")
    xv = x.view(-1)
    xv[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
    it, rel = st.solve(x, tol=1e-8)
    return st, x, it, rel


@pytest.mark.parametrize("uniform", [True, False])
def test_hex8_uniform_force_matches_oracle(gf, oracle, uniform):
    """Stiffness action: closed-form uniform Hex8 kernel and general kernel vs the reference
    chain (SymGradN_vector -> stress -> Int_gradN_dot_tensor2_dV -> AssembleNode)."""
    R = oracle
    for (nx, ny, nz, sc) in ((5, 4, 3, (1.0, 1.0, 1.0)), (4, 3, 5, (0.6, 1.3, 0.9))):
        coor, conn = R.hex8_regular(nx, ny, nz)
        coor = coor * np.array(sc)
        K, G = seeded_material(conn.shape[0], 40)
        nnode = coor.shape[0]
        dofs = np.arange(nnode * 3).reshape(nnode, 3)
        st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, np.array([0, 1, 2]),
                                      uniform=uniform)
        assert st.uniform == uniform
        u = seeded_field((nnode, 3), 41)
        dNx, vol = R.compute_dN(R.as_element(conn, coor), *R.hex8_gauss())
        eps = R.sym_grad_n_vector(dNx, R.as_element(conn, u))
        f_r = R.assemble_node(conn, dofs, R.int_grad_n_dot_tensor2_dv(dNx, vol, R.elastic_stress(
            eps, K, G)))
        assert rel_err(to_np(st.force(u)), f_r) <= RTOL


@pytest.mark.parametrize("uniform", [True, False])
def test_pcg_vs_direct_solve_small(gf, oracle, uniform):
    from oracle import statics as S

    coor, conn, K, G, iip, xp = _hex8_case(10, 42)
    A = S.stiffness(coor, conn, K, G)
    x_ref = S.solve_partitioned(A, iip, xp)
    st, x, it, rel = _solve_gpu(gf, coor, conn, K, G, iip, xp, uniform)
    xg = to_np(x).ravel()
    assert rel <= 1e-8
    assert S.residual(A, iip, xg) <= 1e-8  # the oracle's own residual of the GPU answer
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) <= 1e-6
    assert np.array_equal(xg[iip], xp)


def test_pcg_vs_direct_solve_32(gf, oracle):
    """The 32^3 case against the committed direct-solve fixture (tests/golden/hex8_32_static.npz,
    made by tests/golden/make_static_golden.py)."""
    from oracle import statics as S

    path = os.path.join(HERE, "golden", "hex8_32_static.npz")
    fx = np.load(path)
    coor, conn, K, G, iip, xp = _hex8_case(32, 3)
    st, x, it, rel = _solve_gpu(gf, coor, conn, K, G, iip, xp, True)
    xg = to_np(x).ravel()
    A = S.stiffness(coor, conn, K, G)
    assert rel <= 1e-8 and S.residual(A, iip, xg) <= 1e-8
    x_ref = fx["x"].ravel()
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) <= 1e-6


def test_pcg_is_deterministic(gf, oracle):
    coor, conn, K, G, iip, xp = _hex8_case(8, 43)
    _, x1, it1, r1 = _solve_gpu(gf, coor, conn, K, G, iip, xp, True)
    _, x2, it2, r2 = _solve_gpu(gf, coor, conn, K, G, iip, xp, True)
    assert it1 == it2 and r1 == r2 and torch.equal(x1, x2)


def test_pcg_quad4(gf, oracle):
    """2-d: bottom edge fixed, top edge uy = -1e-2."""
    from oracle import statics as S

    R = oracle
    coor, conn = R.quad4_regular(24, 16)
    K, G = seeded_material(conn.shape[0], 44)
    bot = np.arange(25)
    top = bot + 16 * 25
    iip = np.unique(np.concatenate([(bot[:, None] * 2 + np.arange(2)).ravel(), top * 2 + 1]))
    xp = np.where(np.isin(iip, top * 2 + 1), -1e-2, 0.0)
    A = S.stiffness(coor, conn, K, G)
    x_ref = S.solve_partitioned(A, iip, xp)
    st, x, it, rel = _solve_gpu(gf, coor, conn, K, G, iip, xp, "auto")
    assert st.uniform
    xg = to_np(x).ravel()
    assert S.residual(A, iip, xg) <= 1e-8
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) <= 1e-6


@pytest.mark.parametrize("n", [6, 7])
def test_flexible_cg_jacobi_hex8(gf, oracle, n):
    """gfgpu_fcg_solve without a network (Jacobi direction, ring of earlier directions) on Hex8:
    an odd dof count (n = 6: 7^3 nodes x 3) and an even one, against the direct solve."""
    import ctypes as C

    from goosefem_gb300 import _dev, _lib
    from oracle import statics as S

    coor, conn, K, G, iip, xp = _hex8_case(n, 45)
    nnode, nd = coor.shape
    dofs = np.arange(nnode * nd).reshape(nnode, nd)
    st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, iip, uniform=True)
    x = torch.zeros(nnode * nd, dtype=torch.float64, device="cuda")
    x[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
    nb = int(_lib.lib().gfgpu_fcg_workspace_bytes(C.addressof(st.desc), 0, 0, 3, 1))
    ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device="cuda")
    it, rel = C.c_int64(0), C.c_double(0.0)
    _lib.call("gfgpu_fcg_solve", C.addressof(st.desc), st.diag.data_ptr(), None, x.data_ptr(), 1e-8,
              100000, 3, 4, ws.data_ptr(), _dev.stream(), C.addressof(it), C.addressof(rel))
    A = S.stiffness(coor, conn, K, G)
    x_ref = S.solve_partitioned(A, iip, xp)
    xg = to_np(x)
    assert rel.value <= 1e-8 and S.residual(A, iip, xg) <= 1e-8
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) <= 1e-6


def test_hex8_cube_coefficients_match_uniform_kernel(gf, oracle):
    """Cube Hex8 with folded per-element coefficients (gfgpu_verlet_precompute) against the
    uniform-box kernel that recombines K, G in every application and against the oracle."""
    R = oracle
    coor, conn = R.hex8_regular(6, 5, 4)
    coor = coor * 0.7
    K, G = seeded_material(conn.shape[0], 46)
    nnode = coor.shape[0]
    dofs = np.arange(nnode * 3).reshape(nnode, 3)
    st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, np.array([0, 1, 2]), uniform=True)
    assert st.coef is not None and tuple(st.coef.shape) == (conn.shape[0], 8)
    u = seeded_field((nnode, 3), 47)
    f_cube = to_np(st.force(u))
    st.desc.coef = None
    f_box = to_np(st.force(u))
    assert rel_err(f_cube, f_box) <= 1e-13
    dNx, vol = R.compute_dN(R.as_element(conn, coor), *R.hex8_gauss())
    eps = R.sym_grad_n_vector(dNx, R.as_element(conn, u))
    f_r = R.assemble_node(conn, dofs, R.int_grad_n_dot_tensor2_dv(dNx, vol, R.elastic_stress(
        eps, K, G)))
    assert rel_err(f_cube, f_r) <= RTOL


@pytest.mark.parametrize("uniform", ["auto", False])
def test_regular_gather_same_bits_as_csr(gf, oracle, uniform):
    """On a Regular Quad4 mesh the static operator gathers element forces by index arithmetic
    (detected on the device); the Jacobi-PCG iterates are bit-identical to the dof-CSR gather's,
    and so are the flexible CG's with the two-level correction."""
    from goosefem_gb300 import learned as LR

    R = oracle
    nx, ny = 37, 22
    coor, conn = R.quad4_regular(nx, ny)
    K, G = seeded_material(conn.shape[0], 45)
    bot = np.arange(nx + 1)
    top = bot + ny * (nx + 1)
    iip = np.unique(np.concatenate([(bot[:, None] * 2 + np.arange(2)).ravel(), top * 2 + 1]))
    xp = np.where(np.isin(iip, top * 2 + 1), -1e-2, 0.0)
    out = []
    for csr in (False, True):
        dofs = np.arange(coor.shape[0] * 2).reshape(-1, 2)
        st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, iip, uniform=uniform)
        assert st.desc.reg_nx == nx
        if csr:
            st.use_csr_gather()
        x = torch.zeros(coor.shape[0] * 2, dtype=torch.float64, device="cuda")
        x[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
        xv = x.view(-1, 2).clone()
        it = st.solve(xv, tol=1e-10)
        out.append((it, to_np(xv)))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    # the flexible CG (two-level) through the learned-preconditioner object
    res = []
    for csr in (False, True):
        lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=0)
        assert lp.static.desc.reg_nx == nx
        if csr:
            lp.static.use_csr_gather()
        lp.coarse_setup(8)
        xx = lp.initial_guess(xp)
        lp.fcg(xx, use_nn=False, nkeep=2, coarse=True)
        res.append(to_np(xx))
    assert np.array_equal(res[0], res[1])


@pytest.mark.parametrize("uniform", [True, False])
def test_hex8_regular_gather_same_bits_as_csr(gf, oracle, uniform):
    """On a Regular Hex8 mesh (nx, ny, nz all different) the operator gathers a node's <= 8
    element forces by index arithmetic in the CSR's order: the Jacobi-PCG iterates are
    bit-identical to the dof-CSR gather's; a renumbered mesh is not taken for a Regular one."""
    R = oracle
    nx, ny, nz = 9, 6, 5
    coor, conn = R.hex8_regular(nx, ny, nz)
    K, G = seeded_material(conn.shape[0], 46)
    nxy = (nx + 1) * (ny + 1)
    front = np.arange(nxy)
    back = front + nz * nxy
    iip = np.unique(np.concatenate([(front[:, None] * 3 + np.arange(3)).ravel(), back * 3 + 2]))
    xp = np.where(np.isin(iip, back * 3 + 2), -1e-2, 0.0)
    nnode = coor.shape[0]
    out = []
    for csr in (False, True):
        dofs = np.arange(nnode * 3).reshape(-1, 3)
        st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, iip, uniform=uniform)
        assert (st.desc.reg_nx, st.desc.reg_ny, st.desc.reg_nz) == (nx, ny, nz)
        if csr:
            st.use_csr_gather()
        x = torch.zeros(nnode * 3, dtype=torch.float64, device="cuda")
        x[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
        it, rel = st.solve(x.view(-1, 3), tol=1e-10)
        out.append((it, rel, to_np(x)))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])
    # the same mesh with its dofs permuted: gathered through the CSR
    perm = np.random.default_rng(3).permutation(nnode * 3)
    st = gf.statics.ElasticStatic(coor, conn, perm.reshape(-1, 3), K, G, iip, uniform=uniform)
    assert st.desc.reg_nz == 0


def _pcg_vec(st, which):
    import ctypes as C

    from goosefem_gb300 import _lib

    p = C.c_void_p(0)
    _lib.call("gfgpu_pcg_vector", C.addressof(st.desc), st.ws.data_ptr(), which, C.addressof(p))
    n = st.nnode * st.ndim
    off = (p.value - st.ws.data_ptr()) // 8
    return st.ws[off: off + n]


def test_pcg_pair_operator_matches_fp64(gf, oracle):
    """The float-float stiffness action of the Jacobi-PCG iterations (Regular cube Hex8, nx, ny,
    nz all different) against the FP64 operator on the same direction: q = A p0 with p0 = M^-1 r0
    after gfgpu_pcg_begin, on the free dofs, within 1e-12 of max |A p0| (pairs carry ~48 bits)."""
    import ctypes as C

    from goosefem_gb300 import _dev, _lib

    R = oracle
    nx, ny, nz = 9, 6, 5
    coor, conn = R.hex8_regular(nx, ny, nz)
    K, G = seeded_material(conn.shape[0], 47)
    nxy = (nx + 1) * (ny + 1)
    front = np.arange(nxy)
    back = front + nz * nxy
    iip = np.unique(np.concatenate([(front[:, None] * 3 + np.arange(3)).ravel(), back * 3 + 2]))
    xp = np.where(np.isin(iip, back * 3 + 2), -1e-2, 0.0)
    nnode = coor.shape[0]
    st = gf.statics.ElasticStatic(coor, conn, np.arange(nnode * 3).reshape(-1, 3), K, G, iip,
                                  arithmetic="pair")
    assert st.arithmetic == "pair"
    x = torch.zeros(nnode * 3, dtype=torch.float64, device="cuda")
    x[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
    _lib.call("gfgpu_pcg_begin", C.addressof(st.desc), st.diag.data_ptr(), None, x.data_ptr(),
              st.ws.data_ptr(), _dev.stream())
    p0 = _pcg_vec(st, 2).clone()
    _lib.call("gfgpu_pcg_iterate", C.addressof(st.desc), 1, x.data_ptr(), st.ws.data_ptr(),
              _dev.stream())
    q = to_np(_pcg_vec(st, 3))
    f = to_np(st.force(p0.view(-1, 3))).ravel()
    free = np.setdiff1d(np.arange(nnode * 3), iip)
    assert np.max(np.abs(q[iip])) == 0.0
    err = np.max(np.abs(q[free] - f[free])) / np.max(np.abs(f[free]))
    assert 0 < err <= 1e-12, err


def test_pcg_pair_solve(gf, oracle):
    """Jacobi-PCG with the pair operator reaches the same 1e-8 true residual (checked with the FP64
    operator and by the oracle), agrees with the FP64 solve and with the direct solve, is
    deterministic, and refuses meshes it does not cover."""
    from oracle import statics as S

    coor, conn, K, G, iip, xp = _hex8_case(10, 42)
    A = S.stiffness(coor, conn, K, G)
    x_ref = S.solve_partitioned(A, iip, xp)
    nnode = coor.shape[0]
    dofs = np.arange(nnode * 3).reshape(-1, 3)
    out = []
    for arith in ("pair", "pair", "fp64"):
        st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, iip, arithmetic=arith)
        x = torch.zeros((nnode, 3), dtype=torch.float64, device="cuda")
        x.view(-1)[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
        it, rel = st.solve(x, tol=1e-8)
        out.append((it, rel, to_np(x).ravel()))
    (it_p, rel_p, xp_), (it_p2, rel_p2, xp2), (it_d, rel_d, xd) = out
    assert rel_p <= 1e-8 and S.residual(A, iip, xp_) <= 1e-8
    assert it_p == it_p2 and rel_p == rel_p2 and np.array_equal(xp_, xp2)
    assert abs(it_p - it_d) <= 2
    assert np.linalg.norm(xp_ - x_ref) / np.linalg.norm(x_ref) <= 1e-6
    assert np.linalg.norm(xp_ - xd) / np.linalg.norm(xd) <= 1e-7
    assert np.array_equal(xp_[iip], xp)
    # not a cube mesh / not Regular: refused
    st = gf.statics.ElasticStatic(coor * np.array([1.0, 1.0, 1.5]), conn, dofs, K, G, iip)
    with pytest.raises(RuntimeError):
        st.use_pair()


def _quad4_case(nx, ny, seed):
    from oracle import gfref as R

    coor, conn = R.quad4_regular(nx, ny)
    K, G = seeded_material(conn.shape[0], seed)
    W = nx + 1
    bot = np.arange(W)
    top = bot + ny * W
    iip = np.unique(np.concatenate([(bot[:, None] * 2 + np.arange(2)).ravel(), top * 2 + 1]))
    xp = np.where(np.isin(iip, top * 2 + 1), -1e-2, 0.0)
    return coor, conn, K, G, iip, xp


def test_pcg_pair_operator_quad4(gf, oracle):
    """Uniform square Quad4: the pair element kernel (FP64 direction split into pairs, square closed
    form on pairs, forces joined to FP64) followed by the FP64 gather, against the FP64 operator on
    the same direction, within 1e-12 of max |A p0|."""
    import ctypes as C

    from goosefem_gb300 import _dev, _lib

    coor, conn, K, G, iip, xp = _quad4_case(24, 16, 48)
    nnode = coor.shape[0]
    st = gf.statics.ElasticStatic(coor, conn, np.arange(nnode * 2).reshape(-1, 2), K, G, iip,
                                  arithmetic="pair")
    assert st.arithmetic == "pair"
    x = torch.zeros(nnode * 2, dtype=torch.float64, device="cuda")
    x[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
    _lib.call("gfgpu_pcg_begin", C.addressof(st.desc), st.diag.data_ptr(), None, x.data_ptr(),
              st.ws.data_ptr(), _dev.stream())
    p0 = _pcg_vec(st, 2).clone()
    _lib.call("gfgpu_pcg_iterate", C.addressof(st.desc), 1, x.data_ptr(), st.ws.data_ptr(),
              _dev.stream())
    q = to_np(_pcg_vec(st, 3))
    f = to_np(st.force(p0.view(-1, 2))).ravel()
    free = np.setdiff1d(np.arange(nnode * 2), iip)
    err = np.max(np.abs(q[free] - f[free])) / np.max(np.abs(f[free]))
    assert 0 < err <= 1e-12, err


def test_pcg_pair_quad4_solve(gf, oracle):
    """Quad4 Jacobi-PCG with the pair operator against the direct solve and the FP64 PCG."""
    from oracle import statics as S

    coor, conn, K, G, iip, xp = _quad4_case(24, 16, 44)
    A = S.stiffness(coor, conn, K, G)
    x_ref = S.solve_partitioned(A, iip, xp)
    nnode = coor.shape[0]
    dofs = np.arange(nnode * 2).reshape(-1, 2)
    out = []
    for arith in ("pair", "fp64"):
        st = gf.statics.ElasticStatic(coor, conn, dofs, K, G, iip, arithmetic=arith)
        x = torch.zeros((nnode, 2), dtype=torch.float64, device="cuda")
        x.view(-1)[torch.as_tensor(iip, device="cuda").long()] = torch.as_tensor(xp, device="cuda")
        it, rel = st.solve(x, tol=1e-8)
        out.append((it, rel, to_np(x).ravel()))
    (it_p, rel_p, xq), (it_d, rel_d, xd) = out
    assert rel_p <= 1e-8 and S.residual(A, iip, xq) <= 1e-8
    assert abs(it_p - it_d) <= 2
    assert np.linalg.norm(xq - x_ref) / np.linalg.norm(x_ref) <= 1e-6
    assert np.linalg.norm(xq - xd) / np.linalg.norm(xd) <= 1e-7


def test_two_level_fcg_pair_operator(gf, oracle):
    """The two-level flexible CG (no network) with the pair operator on its directions reaches the
    FP64 true residual and agrees with the FP64-operator solve."""
    from goosefem_gb300 import learned as LR
    from goosefem_gb300 import mesh as M

    nx = ny = 48
    K, G, _ = LR.inclusion_material(nx, ny, 5, rmin=2.0, rmax=5.0)
    iip, xp = LR.static_bc(M.Quad4.Regular(nx, ny))
    res = []
    for arith in ("pair", "fp64"):
        lp = LR.LearnedPreconditioner(nx, ny, K, G, iip, seed=0, arithmetic=arith)
        assert lp.static.arithmetic == arith
        lp.coarse_setup(8)
        x = lp.initial_guess(xp)
        it, rel = lp.fcg(x, tol=1e-8, use_nn=False, nkeep=4, coarse=True)
        res.append((it, rel, to_np(x)))
    assert res[0][1] <= 1e-8 and res[1][1] <= 1e-8
    assert abs(res[0][0] - res[1][0]) <= 2
    assert np.linalg.norm(res[0][2] - res[1][2]) / np.linalg.norm(res[1][2]) <= 1e-7
