"""The GooseFEM-compatible C++ interface (include/gfgpu/GooseFEM.hpp) compiled into a host program
(tests/cpp/test_api.cpp) and checked against the oracle: the drop-in path a C++ GooseFEM user
takes, through the C ABI of libgfgpu.so."""

import os
import subprocess

import numpy as np
import pytest

from _common import RTOL, rel_err, seeded_field, seeded_material

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_api_force_chain_and_mass(oracle, tmp_path):
    import __graft_entry__

    __graft_entry__.build()
    lib = os.path.join(ROOT, "goosefem_gb300")
    exe = str(tmp_path / "test_api")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "test_api.cpp"), "-L" + lib,
                           "-lgfgpu", "-Wl,-rpath," + lib, "-o", exe])
    nx = 64
    nelem, nnode = nx * nx, (nx + 1) ** 2
    K, G = seeded_material(nelem, 61)
    u = seeded_field((nnode, 2), 62)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([nx], dtype=np.int64).tofile(f)
        K.tofile(f)
        G.tofile(f)
        u.tofile(f)
    out = tmp_path / "out.bin"
    res = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    data = np.fromfile(out, dtype=np.float64)

    R = oracle
    coor, conn = R.quad4_regular(nx, nx)
    dofs = R.dofs(nnode, 2)
    x = R.as_element(conn, coor)
    dNx, vol = R.compute_dN(x, *R.quad4_gauss())
    ue = R.as_element(conn, u)
    eps = R.sym_grad_n_vector(dNx, ue)
    sig = R.elastic_stress(eps, K, G)
    fe = R.int_grad_n_dot_tensor2_dv(dNx, vol, sig)
    fint = R.assemble_node(conn, dofs, fe)
    xin, win = R.quad4_nodal()
    _, voln = R.compute_dN(x, xin, win)
    Nn, _ = R.shape(xin)
    M = R.diag_assemble(conn, dofs, R.int_n_scalar_nt_dv(Nn, voln, np.ones((nelem, 4)), 2))
    _, vol3 = R.quad4_planar_compute_dN(x, *R.quad4_gauss(), thick=2.0)
    eps3 = R.grad_n_vector_planar(dNx, ue, 2)
    sig3 = R.elastic_stress(eps3, K, G)
    fe3 = R.int_grad_n_dot_tensor2_dv_planar(dNx, vol3, sig3)
    expect = [dNx, vol, ue, eps, sig, fe, fint, M, vol3, eps3, sig3, fe3]
    k = 0
    for ref in expect:
        got = data[k:k + ref.size].reshape(ref.shape)
        k += ref.size
        assert rel_err(got, ref) <= RTOL
    # static solve through MatrixPartitioned + MatrixPartitionedSolver vs the direct solve
    from oracle import statics as S

    bot = np.arange(nx + 1)
    top = bot + nx * (nx + 1)
    iip = np.unique(np.concatenate([(bot[:, None] * 2 + np.arange(2)).ravel(), top * 2 + 1]))
    xp = np.where(np.isin(iip, top * 2 + 1), -0.01, 0.0)
    x_ref = S.solve_partitioned(S.stiffness(coor, conn, K, G), iip, xp)
    xs = data[k:k + nnode * 2]
    k += nnode * 2
    assert np.linalg.norm(xs - x_ref) / np.linalg.norm(x_ref) <= 1e-9
    # VectorPartitioned round trip and copies: both equal u with the right open edge = the left
    left = np.arange(1, nx) * (nx + 1)
    u2 = u.copy()
    u2[left + nx] = u2[left]
    for _ in range(2):
        assert np.array_equal(data[k:k + nnode * 2].reshape(nnode, 2), u2)
        k += nnode * 2
    # MatrixDiagonalPartitioned: dot, solve (unknown dofs only), reaction (prescribed dofs only)
    Mn = M[dofs]
    isp = np.isin(dofs, iip)
    got = [data[k + j * nnode * 2:k + (j + 1) * nnode * 2].reshape(nnode, 2) for j in range(3)]
    k += 3 * nnode * 2
    assert rel_err(got[0], Mn * u) <= RTOL
    assert rel_err(got[1], np.where(isp, 0.0, u / Mn)) <= RTOL
    assert np.all(got[1][isp] == 0.0)
    assert rel_err(got[2], np.where(isp, Mn * u, 0.0)) <= RTOL
    assert np.all(got[2][~isp] == 0.0)
    assert k == data.size
    assert np.array_equal(data[:dNx.size].reshape(dNx.shape), dNx)  # set-up is bit-exact
