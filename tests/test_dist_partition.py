"""The row-block partition of the explicit dynamics (goosefem_gb300/partition.py) across 2 and 3
ranks on CPU, torch.distributed with the gloo backend: each rank advances its local mesh (owned
node rows + one halo row per neighbour) and exchanges the halo rows after every increment through
the partition's own exchange (exchange_halo, run_partitioned). The per-rank arithmetic is the
oracle's increment loop (docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157 restated
in oracle/gfref.cpp) standing in for the GPU engines, which need a GPU: 50 increments of a 64 x 64
mesh split into row blocks give the single-domain oracle run's bits on every owned node."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NX = NY = 64
NSTEPS = 50


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    rng = np.random.default_rng(64)
    nelem, nnode = NX * NY, (NX + 1) * (NY + 1)
    K = rng.uniform(0.5, 1.5, nelem)
    G = rng.uniform(0.25, 0.75, nelem)
    v0 = rng.uniform(-1e-3, 1e-3, (nnode, 2))
    v0[: NX + 1, :] = 0.0  # bottom row fixed
    dt = 0.1 / np.sqrt(np.max(K + 4.0 * G / 3.0))
    return K, G, v0, dt


class OracleEngine:
    """The oracle's increment on one rank's local mesh (host numpy state)."""

    def __init__(self, R, coor, conn, dofs, K, G, iip, dt, eta):
        self.R, self.conn, self.dofs, self.K, self.G, self.dt, self.eta = R, conn, dofs, K, G, dt, eta
        xr = R.as_element(conn, coor)
        self.dNx, self.vol = R.compute_dN(xr, *R.quad4_gauss())
        xin, win = R.quad4_nodal()
        _, voln = R.compute_dN(xr, xin, win)
        Nn, _ = R.shape(xin)
        self.A = R.diag_assemble(conn, dofs, R.int_n_scalar_nt_dv(Nn, voln, np.ones((conn.shape[0], 4)), 2))
        self.free = np.ones(dofs.size, dtype=np.uint8)
        if iip is not None:
            self.free[np.asarray(iip)] = 0
        self.W = NX + 1

    def begin(self, u, v, a):
        self.u, self.v, self.a = u, v, a

    def increment(self, it, last):
        self.R.verlet_run(self.conn, self.dofs, self.dNx, self.vol, self.K, self.G, self.A, self.free, None,
                          self.dt, self.eta, 1, self.u, self.v, self.a)

    def rows(self, it, row):
        sl = slice(row * self.W, (row + 1) * self.W)
        return torch.from_numpy(np.stack([self.u[sl], self.v[sl], self.a[sl]])).contiguous()

    def set_rows(self, it, row, buf):
        sl = slice(row * self.W, (row + 1) * self.W)
        b = buf.numpy()
        self.u[sl], self.v[sl], self.a[sl] = b[0], b[1], b[2]

    def end(self, last):
        return self.u, self.v, self.a


def _worker(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from goosefem_gb300 import partition as P
    from oracle import gfref as R

    K, G, v0, dt = _problem()
    part = P.RowBlockPartition(NX, NY, world, rank)
    coor, conn, dofs, Kl, Gl, iip, vl = P.local_problem(part, K, G, v0)
    eng = OracleEngine(R, coor, conn, dofs, Kl, Gl, iip, dt, 0.1)
    u = np.zeros_like(vl)
    v = vl.copy()
    a = np.zeros_like(vl)
    P.run_partitioned(part, eng, u, v, a, NSTEPS)
    lo, hi = part.owned()
    W = NX + 1
    out[rank] = (part.r0, part.r1, u[lo * W: hi * W].copy(), v[lo * W: hi * W].copy(),
                 a[lo * W: hi * W].copy())
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_row_block_partition_matches_single_domain(oracle, world):
    R = oracle
    K, G, v0, dt = _problem()
    # single domain
    coor, conn = R.quad4_regular(NX, NY)
    dofs = R.dofs(coor.shape[0], 2)
    iip = dofs[: NX + 1, :].ravel()
    eng = OracleEngine(R, coor, conn, dofs, K, G, iip, dt, 0.1)
    u, v, a = np.zeros_like(v0), v0.copy(), np.zeros_like(v0)
    eng.begin(u, v, a)
    for it in range(NSTEPS):
        eng.increment(it, it + 1 == NSTEPS)
    # partitioned
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
    W = NX + 1
    covered = np.zeros(NY + 1, dtype=int)
    for r in range(world):
        r0, r1, ur, vr, ar = out[r]
        covered[r0:r1] += 1
        for got, ref in ((ur, u), (vr, v), (ar, a)):
            exp = ref[r0 * W: r1 * W]
            assert np.max(np.abs(got - exp)) <= 1e-12 * np.max(np.abs(ref))
            assert np.array_equal(got, exp)  # same element forces, same order: same bits
    assert np.all(covered == 1)
    assert np.max(np.abs(u)) > 0


def test_partition_rows_cover_the_mesh():
    from goosefem_gb300 import partition as P

    for ny, world in ((64, 2), (64, 3), (10, 11), (7, 1)):
        parts = [P.RowBlockPartition(8, ny, world, r) for r in range(world)]
        assert parts[0].r0 == 0 and parts[-1].r1 == ny + 1
        for p, q in zip(parts[:-1], parts[1:]):
            assert p.r1 == q.r0  # contiguous, disjoint
            assert p.g1 - 1 == q.r0 and q.g0 == p.r1 - 1  # each halo row is the neighbour's owned row
        for p in parts:
            assert p.r1 > p.r0 and p.local_ny >= 1 or ny == 0
