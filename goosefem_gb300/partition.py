"""Row-block partition of the explicit dynamics of a Mesh::Quad4::Regular mesh over ranks.

The explicit step (docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157) shards by
element: every element force depends only on its own nodes, and the assembly
(Vector::assembleNode, Vector.h:724-757) sums a node's contributions from at most four elements.
Rank r owns the node rows [r0, r1) of the (ny + 1) rows and computes every element that touches
them, i.e. the element rows [r0 - 1, r1 - 1]. Those elements also read the node rows r0 - 1 and
r1, owned by the neighbours: a one-node-row halo. Each rank therefore holds a local Regular mesh of
node rows [g0, g1) = [max(r0 - 1, 0), min(r1 + 1, ny + 1)) and, after every increment, receives
the halo rows from its neighbours and sends them its own first and last owned rows. The halo
elements are computed by both ranks instead of exchanging partial forces, so each owned node sums
the same element forces in the same (ascending element) order as the single-domain run: the
partitioned run gives the single-domain bits, and the only exchange is one node row per neighbour
and increment.

Engines advance one rank's local mesh and expose its halo rows:
 * PairEngine: the float-float fused kernel (gfgpu_verlet_pair_*): the halo is the predicted
   displacement of the next increment, one pair row (16 bytes per node) per neighbour;
 * FP64Engine: the FP64 kernels (gfgpu_verlet_step with one increment per call): the halo is the
   row's u, v, a (48 bytes per node), from which the next call's predictor recomputes the halo's
   displacement with the owner's arithmetic.
The exchange itself (exchange_halo) runs over torch.distributed point-to-point messages: NCCL for
device tensors, gloo for host tensors.
"""

import ctypes as C

import numpy as np
import torch

from . import _dev, _lib


class RowBlockPartition:
    """Rank `rank` of `world` in a row-block partition of Regular(nx, ny): balanced blocks of the
    ny + 1 node rows (the first (ny + 1) % world ranks take one row more)."""

    def __init__(self, nx, ny, world, rank):
        if not (0 <= rank < world) or world > ny + 1:
            raise ValueError("need 0 <= rank < world <= ny + 1")
        self.nx, self.ny, self.world, self.rank = int(nx), int(ny), int(world), int(rank)
        rows = ny + 1
        base, extra = divmod(rows, world)
        self.r0 = rank * base + min(rank, extra)
        self.r1 = self.r0 + base + (1 if rank < extra else 0)
        self.g0 = max(self.r0 - 1, 0)
        self.g1 = min(self.r1 + 1, rows)
        self.W = nx + 1

    @property
    def local_ny(self):
        """Element rows of the local mesh."""
        return self.g1 - self.g0 - 1

    @property
    def nnode_local(self):
        return (self.g1 - self.g0) * self.W

    def node_rows(self):
        """Global node indices of the local mesh (row-major, as Regular numbers them)."""
        return np.arange(self.g0 * self.W, self.g1 * self.W)

    def element_rows(self):
        """Global element indices of the local mesh."""
        return np.arange(self.g0 * self.nx, (self.g1 - 1) * self.nx)

    def owned(self):
        """Local row range [a, b) of the owned node rows."""
        return self.r0 - self.g0, self.r1 - self.g0

    def neighbours(self):
        """(rank below or None, rank above or None)."""
        return (self.rank - 1 if self.rank > 0 else None,
                self.rank + 1 if self.rank < self.world - 1 else None)

    def send_rows(self):
        """Local rows sent to the rank below and above: the first and the last owned row."""
        a, b = self.owned()
        return a, b - 1

    def recv_rows(self):
        """Local halo rows received from the rank below and above."""
        return 0, self.g1 - self.g0 - 1


def exchange_halo(part, send_lo, send_hi, recv_lo, recv_hi, group=None):
    """Point-to-point halo exchange with the neighbours (torch.distributed isend / irecv): send_lo
    goes to the rank below, whose recv_hi receives it, and so on. Tensors of the lower / upper
    neighbour that does not exist are ignored. Deterministic (plain copies)."""
    import torch.distributed as dist

    lo, hi = part.neighbours()
    reqs = []
    if lo is not None:
        reqs.append(dist.isend(send_lo, lo, group=group))
        reqs.append(dist.irecv(recv_lo, lo, group=group))
    if hi is not None:
        reqs.append(dist.isend(send_hi, hi, group=group))
        reqs.append(dist.irecv(recv_hi, hi, group=group))
    for r in reqs:
        r.wait()


def local_problem(part, K, G, v0=None, fixed_bottom=True):
    """The local mesh of a rank: Regular(nx, local_ny) with the y coordinates of its global rows,
    its elements' moduli, the prescribed dofs of the global bottom edge it holds, and the initial
    velocity of its nodes (global arrays in, local arrays out)."""
    from . import mesh as M

    m = M.Quad4.Regular(part.nx, part.local_ny)
    coor = m.coor()
    coor[:, 1] += part.g0
    conn, dofs = m.conn(), m.dofs()
    e = part.element_rows()
    Kl, Gl = np.asarray(K)[e], np.asarray(G)[e]
    iip = dofs[: part.W, :].ravel() if (fixed_bottom and part.g0 == 0) else None
    vl = None if v0 is None else np.asarray(v0).reshape(-1, 2)[part.node_rows()]
    return coor, conn, dofs, Kl, Gl, iip, vl


class FP64Engine:
    """One rank's local mesh advanced by the FP64 kernels, one increment per call."""

    def __init__(self, vv):
        self.vv = vv
        vv.use_fp64()

    def begin(self, u, v, a):
        self.u, self.v, self.a = u, v, a

    def increment(self, it, last):
        self.vv.step(self.u, self.v, self.a, 1)

    def rows(self, it, row):
        W = self.vv.desc.reg_nx + 1
        sl = slice(row * W, (row + 1) * W)
        return torch.stack([self.u[sl], self.v[sl], self.a[sl]]).contiguous()

    def set_rows(self, it, row, buf):
        W = self.vv.desc.reg_nx + 1
        sl = slice(row * W, (row + 1) * W)
        self.u[sl], self.v[sl], self.a[sl] = buf[0], buf[1], buf[2]

    def end(self, last):
        return self.u, self.v, self.a


class PairEngine:
    """One rank's local mesh advanced by the float-float fused kernel; between increments the
    state stays in pairs, and the halo rows are rows of the predicted pair displacement."""

    def __init__(self, vv):
        self.vv = vv
        vv.use_pair()

    def _ws(self):
        return C.addressof(self.vv.desc), self.vv.ws.data_ptr()

    def begin(self, u, v, a):
        self.u, self.v, self.a = u, v, a
        d, ws = self._ws()
        _lib.call("gfgpu_verlet_pair_begin", d, u.data_ptr(), v.data_ptr(), a.data_ptr(), ws, _dev.stream())

    def increment(self, it, last):
        d, ws = self._ws()
        _lib.call("gfgpu_verlet_pair_increments", d, int(it), 1, 0 if last else 1, ws, _dev.stream())

    def _disp(self, it):
        d, ws = self._ws()
        p = C.c_void_p(0)
        _lib.call("gfgpu_verlet_pair_displacement", d, int(it), ws, C.addressof(p))
        n = self.vv.nnode
        # the pair nodevec [nnode] of float4 inside the workspace, viewed through the workspace
        # tensor (float64 elements, 2 per node)
        off = (p.value - self.vv.ws.data_ptr()) // 8
        return self.vv.ws[off: off + 2 * n].view(n, 2)

    def rows(self, it, row):
        W = self.vv.desc.reg_nx + 1
        return self._disp(it + 1)[row * W:(row + 1) * W].contiguous()

    def set_rows(self, it, row, buf):
        W = self.vv.desc.reg_nx + 1
        self._disp(it + 1)[row * W:(row + 1) * W] = buf

    def end(self, last):
        d, ws = self._ws()
        _lib.call("gfgpu_verlet_pair_end", d, int(last), self.u.data_ptr(), self.v.data_ptr(), self.a.data_ptr(),
                  ws, _dev.stream())
        return self.u, self.v, self.a


class RankRun:
    """One rank's increments in lock-step pieces: begin, then per increment `increment(it)`, and
    between increments `halo_out(it)` (rows for the neighbours below and above) and
    `halo_in(it, lo, hi)` (their rows into this rank's halo), then `end(last)`."""

    def __init__(self, part, engine):
        self.part, self.engine = part, engine

    def begin(self, u, v, a):
        self.engine.begin(u, v, a)

    def increment(self, it, last):
        self.engine.increment(it, last)

    def halo_out(self, it):
        s_lo, s_hi = self.part.send_rows()
        return self.engine.rows(it, s_lo), self.engine.rows(it, s_hi)

    def halo_in(self, it, recv_lo, recv_hi):
        r_lo, r_hi = self.part.recv_rows()
        lo, hi = self.part.neighbours()
        if lo is not None:
            self.engine.set_rows(it, r_lo, recv_lo)
        if hi is not None:
            self.engine.set_rows(it, r_hi, recv_hi)

    def end(self, last):
        return self.engine.end(last)


def run_partitioned(part, engine, u, v, a, nsteps, exchange=None):
    """nsteps increments of one rank's local state (u, v, a: local nodevecs, updated in place by
    the engine), exchanging the halo rows after every increment but the last. `exchange(part,
    send_lo, send_hi, recv_lo, recv_hi)` defaults to exchange_halo (torch.distributed)."""
    exchange = exchange or exchange_halo
    run = RankRun(part, engine)
    run.begin(u, v, a)
    for it in range(nsteps):
        last = it + 1 == nsteps
        run.increment(it, last)
        if last or part.world == 1:
            continue
        send_lo, send_hi = run.halo_out(it)
        recv_lo, recv_hi = torch.empty_like(send_lo), torch.empty_like(send_hi)
        if send_lo.is_cuda:
            torch.cuda.current_stream().synchronize()  # the rows are complete before they are sent
        exchange(part, send_lo, send_hi, recv_lo, recv_hi)
        run.halo_in(it, recv_lo, recv_hi)
    return run.end(nsteps - 1)
