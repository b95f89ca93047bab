"""The row-block partition's GPU engines (goosefem_gb300/partition.py) on one GPU: three ranks'
local meshes advanced in lock step in one process, the halo rows copied between them after every
increment as the point-to-point exchange would (no kernel waits for another rank). Each rank owns
its node rows and computes the elements around them, so the partitioned run gives the bits of the
single-domain run with the same kernels: the FP64 kernels and the float-float fused kernel."""

import numpy as np
import pytest
import torch

from _common import seeded_field, seeded_material

pytestmark = pytest.mark.gpu

NX, NY, WORLD, NSTEPS = 96, 70, 3, 40


@pytest.fixture(scope="module")
def gf():
    import goosefem_gb300 as gf

    gf.set_strict(False)
    yield gf


def _global(gf):
    mesh = gf.Mesh.Quad4.Regular(NX, NY)
    K, G = seeded_material(mesh.nelem(), 81)
    v0 = seeded_field((mesh.nnode(), 2), 82)
    v0[mesh.nodesBottomEdge(), :] = 0.0
    dt = 0.1 * gf.critical_dt(K, G)
    return mesh, K, G, v0, dt


@pytest.mark.parametrize("arithmetic", ["fp64", "pair"])
def test_partitioned_run_gives_single_domain_bits(gf, arithmetic):
    from goosefem_gb300 import partition as P

    mesh, K, G, v0, dt = _global(gf)
    iip = mesh.dofs()[mesh.nodesBottomEdge(), :].ravel()
    # single domain
    vv = gf.VelocityVerlet(mesh.coor(), mesh.conn(), mesh.dofs(), K, G, dt=dt, eta=0.1, iip=iip,
                           arithmetic=arithmetic)
    ug = torch.zeros((mesh.nnode(), 2), dtype=torch.float64, device="cuda")
    vg, ag = torch.tensor(v0, device="cuda"), torch.zeros_like(ug)
    vv.step(ug, vg, ag, NSTEPS)
    # partitioned, lock step
    runs, states = [], []
    for r in range(WORLD):
        part = P.RowBlockPartition(NX, NY, WORLD, r)
        coor, conn, dofs, Kl, Gl, iipl, vl = P.local_problem(part, K, G, v0)
        lv = gf.VelocityVerlet(coor, conn, dofs, Kl, Gl, dt=dt, eta=0.1, iip=iipl, arithmetic=arithmetic)
        eng = P.PairEngine(lv) if arithmetic == "pair" else P.FP64Engine(lv)
        u = torch.zeros((part.nnode_local, 2), dtype=torch.float64, device="cuda")
        st = [u, torch.tensor(vl, device="cuda"), torch.zeros_like(u)]
        run = P.RankRun(part, eng)
        run.begin(*st)
        runs.append(run)
        states.append(st)
    for it in range(NSTEPS):
        last = it + 1 == NSTEPS
        for run in runs:
            run.increment(it, last)
        if last:
            continue
        outs = [run.halo_out(it) for run in runs]
        for r, run in enumerate(runs):
            lo = outs[r - 1][1].clone() if r > 0 else None
            hi = outs[r + 1][0].clone() if r < WORLD - 1 else None
            run.halo_in(it, lo, hi)
    W = NX + 1
    for r, run in enumerate(runs):
        u, v, a = run.end(NSTEPS - 1)
        lo, hi = run.part.owned()
        r0, r1 = run.part.r0, run.part.r1
        for got, ref in ((u, ug), (v, vg), (a, ag)):
            assert torch.equal(got[lo * W: hi * W], ref[r0 * W: r1 * W]), (r, arithmetic)
    assert float(ug.abs().max()) > 0
