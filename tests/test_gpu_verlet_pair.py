"""The float-float ("pair") explicit increments (gfgpu_verlet_precompute_pair + gfgpu_verlet_step,
one fused tile kernel per increment) against the oracle's loop
(docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157 restated in oracle/gfref.cpp) and
against the FP64 kernels, at the suite's 1e-12 relative tolerance; tile edges (meshes that are
not multiples of the 32 x 8 node tile), external forces, split calls, repeatability, exact
linearity and the refusal of meshes the path does not cover."""

import numpy as np
import pytest
import torch

from _common import RTOL, rel_err, seeded_field, to_np
from test_gpu_verlet import _run_oracle, _setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    gf.set_strict(False)
    yield gf
    gf.set_strict(False)
    _lib().call("gfgpu_set_pair_kernel", DEFAULT_KERNEL)


def _lib():
    from goosefem_gb300 import _lib as L

    return L


DEFAULT_KERNEL = 2


@pytest.fixture(params=[0, 1, 2], ids=["tma31x7", "tile", "tma31x15"])
def kernel(request, gf):
    """The persistent TMA pipeline (2, the default, 31 x 15 tiles; 0 with 31 x 7 tiles) and the
    one-tile-per-CTA kernel (1); every test ends by checking that no bounded wait gave up."""
    _lib().call("gfgpu_set_pair_kernel", request.param)
    yield request.param
    _lib().call("gfgpu_verlet_pair_status")
    _lib().call("gfgpu_set_pair_kernel", DEFAULT_KERNEL)


def _state(v0):
    u = torch.zeros(v0.shape, dtype=torch.float64, device="cuda")
    return [u, torch.tensor(v0, device="cuda"), torch.zeros_like(u)]


@pytest.mark.parametrize("nx,ny", [(64, 48), (45, 19), (1, 1), (2, 3), (33, 9), (31, 7), (96, 200)])
def test_pair_matches_oracle(gf, oracle, kernel, nx, ny):
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, nx, ny, False, True, 41)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, arithmetic="pair")
    assert vv.path == "uniform-square-pair"
    s = _state(v0)
    vv.step(*s, 60)
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, 60)
    for g, r in zip(s, (ur, vr, ar)):
        assert rel_err(to_np(g), r) <= RTOL


def test_pair_with_external_force_and_free_edges(gf, oracle, kernel):
    """No fixed dofs (every node free, corner / edge / interior mass classes) and an external
    force."""
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 50, 37, False, False, 43)
    fext = seeded_field((mesh.nnode(), 2), 44, amp=1e-4)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, fext=fext, arithmetic="pair")
    s = _state(v0)
    vv.step(*s, 80)
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, 80, fext)
    for g, r in zip(s, (ur, vr, ar)):
        assert rel_err(to_np(g), r) <= RTOL


def test_pair_agrees_with_fp64_kernels(gf, oracle, kernel):
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 96, 80, False, True, 45)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip)
    s64 = _state(v0)
    vv.step(*s64, 200)
    vv.use_pair()
    sp = _state(v0)
    vv.step(*sp, 200)
    for g, r in zip(sp, s64):
        assert rel_err(to_np(g), to_np(r)) <= RTOL


@pytest.mark.parametrize("split", [(1, 1), (1, 2), (7, 10), (16, 1)])
def test_pair_split_calls(gf, oracle, kernel, split):
    """Calls convert the state in and out: step(n1) + step(n2) agrees with step(n1 + n2) to the
    pair rounding of the state between the calls, and odd and even counts end in the right
    buffer."""
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 40, 24, False, True, 47)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, arithmetic="pair")
    one, two = _state(v0), _state(v0)
    vv.step(*one, sum(split))
    for n in split:
        vv.step(*two, n)
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, sum(split))
    for x, y, r in zip(one, two, (ur, vr, ar)):
        assert rel_err(to_np(x), to_np(y)) <= 1e-13
        assert rel_err(to_np(x), r) <= RTOL


def test_pair_repeatable_and_exactly_linear(gf, oracle, kernel):
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 70, 66, False, True, 49)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, arithmetic="pair")
    s1, s2, s3 = _state(v0), _state(2.0 * v0), _state(v0)
    for s in (s1, s2, s3):
        vv.step(*s, 300)
    for x, y, z in zip(s1, s2, s3):
        assert torch.equal(y, 2.0 * x)  # every FP32 operation commutes with a power-of-two scale
        assert torch.equal(z, x)


@pytest.mark.parametrize("case", ["periodic", "periodic-per-dof", "distorted", "rectangles"])
def test_pair_csr_paths(gf, oracle, case):
    """Quad4 meshes outside the Regular square-element case: periodic ties (square closed form +
    dof-CSR node kernel, pair path 2), distorted and rectangular elements (stored element
    stiffness, pair path 3), and the node update with per-dof inverse masses (no mass classes)."""
    R = oracle
    periodic = case.startswith("periodic")
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 30, 22, periodic, not periodic, 51)
    if not periodic:
        coor = coor * np.array([0.7, 1.3]) if case == "rectangles" else coor + seeded_field(coor.shape, 52, amp=0.08)
        xr = R.as_element(conn, coor)
        ref["dNx"], ref["vol"] = R.compute_dN(xr, *R.quad4_gauss())
        xin, win = R.quad4_nodal()
        _, voln = R.compute_dN(xr, xin, win)
        Nn, _ = R.shape(xin)
        ref["A"] = R.diag_assemble(conn, dofs, R.int_n_scalar_nt_dv(Nn, voln, np.ones((mesh.nelem(), 4)), 2))
        dt = 0.05 * gf.critical_dt(K, G) * 0.7
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip)
    if case == "periodic-per-dof":
        vv.use_per_dof_mass()
    if periodic:  # uniform density: one mass class, unless the per-dof update is asked for
        assert (vv.desc.ncls > 0) == (case == "periodic")
    vv.use_pair()
    assert vv.path == ("uniform-square-pair-csr" if periodic else "general-pair"), vv.path
    s = _state(v0)
    vv.step(*s, 60)
    ur, vr, ar = _run_oracle(oracle, ref, v0, dt, 0.1, 60)
    for g, r in zip(s, (ur, vr, ar)):
        assert rel_err(to_np(g), r) <= RTOL
    # the same against the FP64 kernels, and repeatable
    vv.use_fp64()
    s64 = _state(v0)
    vv.step(*s64, 60)
    vv.use_pair()
    s2 = _state(v0)
    vv.step(*s2, 60)
    for g, r, h in zip(s, s64, s2):
        assert rel_err(to_np(g), to_np(r)) <= RTOL
        assert torch.equal(g, h)
    if not periodic:
        # a Regular numbering (distorted or not): the node kernel gathers by index arithmetic in
        # the CSR's order; through the CSR tables it gives the same bits
        assert vv.desc.reg_nx == 30
        vv.desc.reg_nx = 0
        s3 = _state(v0)
        vv.step(*s3, 60)
        for g, h in zip(s, s3):
            assert torch.equal(g, h)


def test_pair_refuses_hex8(gf):
    m3 = gf.Mesh.Hex8.Regular(3, 3, 3)
    K = np.ones(27)
    with pytest.raises(gf.GFGPUError) as ei:
        gf.VelocityVerlet(m3.coor(), m3.conn(), m3.dofs(), K, 0.5 * K, dt=0.01, arithmetic="pair")
    assert ei.value.code == -7


def test_pair_ignored_in_strict_mode(gf, oracle):
    """Strict mode runs the FP64 kernels even with coef_pair set: the same bits as without it."""
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 24, 20, False, True, 53)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, arithmetic="pair")
    try:
        gf.set_strict(True)
        sp = _state(v0)
        vv.step(*sp, 20)
        vv.use_fp64()
        s64 = _state(v0)
        vv.step(*s64, 20)
        for x, y in zip(sp, s64):
            assert torch.equal(x, y)
    finally:
        gf.set_strict(False)


def test_pair_kernels_agree(gf, oracle):
    """The TMA pipeline and the one-tile-per-CTA kernel group the four-element sums differently:
    their states agree to a few pair roundings."""
    mesh, coor, conn, dofs, K, G, iip, v0, dt, ref = _setup(gf, oracle, 130, 75, False, True, 55)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip, arithmetic="pair")
    out = []
    try:
        for k in (0, 1, 2):
            _lib().call("gfgpu_set_pair_kernel", k)
            s = _state(v0)
            vv.step(*s, 100)
            out.append(s)
        _lib().call("gfgpu_verlet_pair_status")
    finally:
        _lib().call("gfgpu_set_pair_kernel", DEFAULT_KERNEL)
    for k in (1, 2):
        for x, y in zip(out[0], out[k]):
            assert rel_err(to_np(x), to_np(y)) <= 1e-13
    # the two TMA tile shapes group every sum alike: identical bits
    for x, y in zip(out[0], out[2]):
        assert torch.equal(x, y)
