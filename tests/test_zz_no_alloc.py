"""The allocation-free explicit increment, gfgpu_verlet_step_noalloc, called through the C ABI.

Some callers cannot call cudaMalloc: host codes that reach the GPU only through this library's
C ABI (no CUDA runtime of their own), or codes whose device memory belongs entirely to another
allocator or pool. For them the element-force scratch of the increment is a fixed-size array
built into the library. This test checks that the entry point gives the same state as the
allocating entry point gfgpu_verlet_step, within the suite's tolerance, on two calls in a row,
and that a mesh larger than the built-in scratch is refused. It lives in a file of its own that
pytest collects last, and passes both alone in a fresh process and after the other tests.
"""

import ctypes as C
import re

import numpy as np
import pytest
import torch

from _common import RTOL, rel_err, seeded_field, seeded_material

pytestmark = pytest.mark.gpu


def _problem(gf, nx, ny, uniform, hex8=False):
    if hex8:
        mesh = gf.Mesh.Hex8.Regular(nx, ny, ny)
        fixed = mesh.nodesFront()
    else:
        mesh = gf.Mesh.Quad4.Regular(nx, ny)
        fixed = mesh.nodesBottomEdge()
    coor, conn, dofs = mesh.coor(), mesh.conn(), mesh.dofs()
    nd = coor.shape[1]
    K, G = seeded_material(mesh.nelem(), 71)
    iip = dofs[fixed, :].ravel()
    v0 = seeded_field((mesh.nnode(), nd), 72)
    v0[fixed, :] = 0.0
    dt = 0.1 * gf.critical_dt(K, G)
    vv = gf.VelocityVerlet(coor, conn, dofs, K, G, dt=dt, eta=0.1, iip=iip,
                           uniform="auto" if uniform else False)
    return mesh, vv, v0


def _state(v0):
    u = torch.zeros(v0.shape, dtype=torch.float64, device="cuda")
    return [u, torch.tensor(v0, device="cuda"), torch.zeros_like(u)]


@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("elem,uniform", [("quad4", True), ("quad4", False), ("hex8", True),
                                          ("hex8", False)])
def test_noalloc_matches_allocating_step(elem, uniform, strict):
    """Both entry points run the same kernels (the node kernel is chosen by one shared helper), so
    the states agree bit for bit; the suite's tolerance is asserted as well."""
    import goosefem_gb300 as gf
    from goosefem_gb300 import _lib

    gf.set_strict(strict)
    try:
        hex8 = elem == "hex8"
        mesh, vv, v0 = _problem(gf, 12 if hex8 else 96, 10 if hex8 else 64, uniform, hex8)
        ref = _state(v0)
        got = _state(v0)
        stream = torch.cuda.current_stream().cuda_stream
        for nsteps in (17, 23):  # two calls in a row, continuing the same state
            _lib.call("gfgpu_verlet_step", C.addressof(vv.desc), ref[0].data_ptr(), ref[1].data_ptr(),
                      ref[2].data_ptr(), nsteps, vv.ws.data_ptr(), stream)
            _lib.call("gfgpu_verlet_step_noalloc", C.addressof(vv.desc), got[0].data_ptr(),
                      got[1].data_ptr(), got[2].data_ptr(), nsteps, stream)
            torch.cuda.synchronize()
            for r, g in zip(ref, got):
                r_np, g_np = r.cpu().numpy(), g.cpu().numpy()
                assert rel_err(g_np, r_np) <= RTOL
                assert np.array_equal(g_np, r_np)
    finally:
        gf.set_strict(False)


def test_noalloc_rejects_meshes_above_its_scratch():
    import goosefem_gb300 as gf
    from goosefem_gb300 import _lib

    mesh, vv, v0 = _problem(gf, 8, 8, True)
    d = _lib.VerletDesc.from_buffer_copy(vv.desc)
    limit = int(re.search(r"#define GFGPU_NOALLOC_FE_DOUBLES (\d+)", open(_lib.HEADER).read())[1])
    d.nelem = limit // (d.nne * d.ndim) + 1  # one element too many; nothing is launched
    s = _state(v0)
    with pytest.raises(gf.GFGPUError) as ei:
        _lib.call("gfgpu_verlet_step_noalloc", C.addressof(d), s[0].data_ptr(), s[1].data_ptr(),
                  s[2].data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
    assert ei.value.code == -1
    assert "scratch" in str(ei.value)
