"""Benchmark: explicit velocity-Verlet dynamics of a 2048 x 2048 Quad4 Regular mesh (FP64).

Workload (one bench step = 1000 increments of the explicit scheme of GooseFEM's
docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp): 4,194,304 elements, 4,198,401 nodes,
plane-strain linear elasticity with per-element K ~ U[0.5,1.5], G ~ U[0.25,0.75] (seeded),
density 1 (lumped mass from nodal quadrature), nodal viscous damping 0.1, bottom row fixed,
random initial velocity U[-1e-3, 1e-3], dt = 0.1 x the CFL limit.

Metric: element-Gauss-point updates per second (nelem x 4 Gauss points x increments / s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gfgpu|reference]

--impl reference times the reference algorithm's CPU implementation on the host cores: the
reference (header-only C++ on xtensor/Eigen) cannot be built here, so its restatement in
oracle/ (same loop nests and summation order) is timed with all host threads.
"""

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NIP = 4
SEED = 2048


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gfgpu", choices=["gfgpu", "reference"])
    p.add_argument("--nx", type=int, default=2048)
    p.add_argument("--increments", type=int, default=1000)
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="bounded CPU-baseline sample length")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--path", default="auto", choices=["auto", "general"],
                   help="element kernel: auto (uniform fast path when applicable) or general")
    return p.parse_args()


def workload(nx, mesh_mod=None):
    """Host-side synthetic inputs of the 2048^2 configuration (seeded)."""
    if mesh_mod is None:
        from oracle import gfref as R

        coor, conn = R.quad4_regular(nx, nx)
        dofs = R.dofs(coor.shape[0], 2)
    else:
        m = mesh_mod.Quad4.Regular(nx, nx)
        coor, conn, dofs = m.coor(), m.conn(), m.dofs()
    nelem = nx * nx
    nnode = (nx + 1) * (nx + 1)
    rng = np.random.default_rng(SEED)
    K = rng.uniform(0.5, 1.5, nelem)
    G = rng.uniform(0.25, 0.75, nelem)
    v0 = rng.uniform(-1e-3, 1e-3, (nnode, 2))
    bottom = np.arange(nx + 1)
    v0[bottom, :] = 0.0
    iip = np.asarray(dofs)[bottom, :].ravel()
    dt = 0.1 * 1.0 / math.sqrt(float(np.max(K + 4.0 * G / 3.0)))
    return dict(coor=coor, conn=conn, dofs=dofs, K=K, G=G, v0=v0, iip=iip, dt=dt, eta=0.1,
                nelem=nelem, nnode=nnode, bottom=bottom)


def cpu_info():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        model = [l.split(":", 1)[1].strip() for l in out.splitlines() if "Model name" in l]
        return model[0] if model else "unknown"
    except Exception:
        return "unknown"


def cpu_sample(w, seconds, parallel):
    """Time the oracle's per-operator explicit loop (the reference algorithm) on the host."""
    from oracle import gfref as R

    conn, dofs, coor = w["conn"], w["dofs"], w["coor"]
    xr = R.as_element(conn, coor)
    dNx, vol = R.compute_dN(xr, *R.quad4_gauss(), parallel=True)
    xin, win = R.quad4_nodal()
    _, voln = R.compute_dN(xr, xin, win, parallel=True)
    Nn, _ = R.shape(xin)
    A = R.diag_assemble(conn, dofs, R.int_n_scalar_nt_dv(Nn, voln, np.ones((w["nelem"], 4)), 2))
    del voln
    free = np.ones(w["nnode"] * 2, dtype=np.uint8)
    free.reshape(-1, 2)[w["bottom"], :] = 0
    u = np.zeros_like(w["v0"])
    v = w["v0"].copy()
    a = np.zeros_like(u)

    def run(n):
        t0 = time.perf_counter()
        R.verlet_run(conn, dofs, dNx, vol, w["K"], w["G"], A, free, None, w["dt"], w["eta"], n, u,
                     v, a, parallel=parallel)
        return time.perf_counter() - t0

    # calibrate with 2 increments (first-touch of the work arrays included), then one call of
    # as many increments as fit in the requested sample length
    t2 = run(2)
    n = max(1, min(1000, int(seconds / max(t2 / 2.0, 1e-9))))
    return n, run(n)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    w = workload(args.nx)
    from oracle import gfref as R

    threads = R.num_threads(True)
    # each bench step: a bounded sample of increments with all host threads
    per = max(args.cpu_seconds / max(args.steps + args.warmup, 1), 0.5)
    for _ in range(args.warmup):
        cpu_sample(w, per, True)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, t = cpu_sample(w, per, True)
        tot_n += n
        tot_t += t
    value = w["nelem"] * NIP * tot_n / tot_t
    line = {
        "impl": "reference", "metric": "elem-Gauss-pt updates/s", "value": value,
        "unit": "elem-Gauss-pt/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"Quad4 Regular {args.nx}x{args.nx} explicit velocity-Verlet, "
                               "per-element K,G, damping 0.1, bottom row fixed",
                   "increments_per_step": f"bounded sample (~{per:.1f} s of increments)"},
        "cpu_baseline": {"value": value, "unit": "elem-Gauss-pt/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{tot_n} increments over {args.steps} steps of the oracle's "
                                   f"per-operator loop, {threads} OpenMP threads ({cpu_info()})"},
        "e2e": {"value": value, "unit": "elem-Gauss-pt/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, rank, world):
    import torch

    import goosefem_gb300 as gf
    from goosefem_gb300 import _lib

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    w = workload(args.nx, gf.Mesh)
    nnode, nelem, inc = w["nnode"], w["nelem"], args.increments
    vv = gf.VelocityVerlet(w["coor"], w["conn"], w["dofs"], w["K"], w["G"], rho=1.0, dt=w["dt"],
                           eta=w["eta"], iip=w["iip"], uniform=("auto" if args.path == "auto"
                                                                else False))
    u = torch.zeros((nnode, 2), dtype=torch.float64, device=dev)
    v = torch.tensor(w["v0"], device=dev)
    a = torch.zeros_like(u)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---------------------------------------------------------------- device-resident timing
    for _ in range(args.warmup):
        vv.step(u, v, a, inc)
    barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        vv.step(u, v, a, inc)
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if sampler else None
    ms_t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = world * nelem * NIP * inc * args.steps / (ms * 1e-3)

    # ---------------------------------------------------------------- per-kernel timing
    # element kernel alone (same launch as inside the step), on the launching stream
    fe = vv.ws
    reps = 50
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        _lib.call("gfgpu_verlet_element_forces", C.addressof(vv.desc), u.data_ptr(),
                  fe.data_ptr(), stream.cuda_stream)
    k0.record(stream)
    for _ in range(reps):
        _lib.call("gfgpu_verlet_element_forces", C.addressof(vv.desc), u.data_ptr(),
                  fe.data_ptr(), stream.cuda_stream)
    k1.record(stream)
    torch.cuda.synchronize()
    ms_elem = k0.elapsed_time(k1) / reps
    ms_inc = ms / (args.steps * inc)
    ms_node = max(ms_inc - ms_elem, 0.0)

    # FP64 issue-rate probe (for the FP64 roof)
    probe_out = torch.zeros(2, dtype=torch.float64, device=dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 16, 20000
    _lib.call("gfgpu_probe_fp64", blocks, 2000, probe_out.data_ptr(), stream.cuda_stream)
    k0.record(stream)
    _lib.call("gfgpu_probe_fp64", blocks, iters, probe_out.data_ptr(), stream.cuda_stream)
    k1.record(stream)
    torch.cuda.synchronize()
    fp64_peak = 2.0 * 8 * iters * blocks * 256 / (k0.elapsed_time(k1) * 1e-3)

    # ---------------------------------------------------------------- end-to-end (host buffers)
    hu = torch.zeros((nnode, 2), dtype=torch.float64).pin_memory()
    hv = torch.tensor(w["v0"]).pin_memory()
    ha = torch.zeros((nnode, 2), dtype=torch.float64).pin_memory()
    ou = torch.empty_like(hu).pin_memory()
    ov = torch.empty_like(hu).pin_memory()
    oa = torch.empty_like(hu).pin_memory()
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        u.copy_(hu, non_blocking=True)
        v.copy_(hv, non_blocking=True)
        a.copy_(ha, non_blocking=True)
        vv.step(u, v, a, inc)
        ou.copy_(u, non_blocking=True)
        ov.copy_(v, non_blocking=True)
        oa.copy_(a, non_blocking=True)
    e1.record(stream)
    barrier()
    ms_e2e = e0.elapsed_time(e1)
    t = torch.tensor([ms_e2e], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_e2e = float(t.item())
    e2e_value = world * nelem * NIP * inc * args.steps / (ms_e2e * 1e-3)
    state_bytes = 3 * nnode * 2 * 8

    if rank != 0:
        return 0

    # ---------------------------------------------------------------- roofline
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        hbm_peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    uniform = vv.uniform
    # algorithmic bytes of one element-kernel launch: u (16 B/node), conn (16 B/elem),
    # K and G (16 B/elem), element forces out (64 B/elem); general path adds dNx + vol (72 B/elem)
    b_elem = 16 * nnode + (16 + 16 + 64) * nelem + (0 if uniform else 72 * nelem)
    achieved = b_elem / (ms_elem * 1e-3) / 1e9
    # FP64 operations of the element kernel per element (DFMA counted as 2)
    fl_elem = 55 if uniform else 4 * (8 * 2 + 8 * 2 + 2 + 12 + 16 * 2 + 8)
    fp64_ach = fl_elem * nelem / (ms_elem * 1e-3)
    # fused-step minimum traffic: u, v, a read+write (96 B/node), inverse mass (16 B/node),
    # K, G (16 B/elem)
    b_step = 112 * nnode + 16 * nelem
    line = {
        "metric": "elem-Gauss-pt updates/s", "value": value, "unit": "elem-Gauss-pt/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"Quad4 Regular {args.nx}x{args.nx} explicit velocity-Verlet, "
                               "per-element K,G, density 1, damping 0.1, bottom row fixed",
                   "nelem": nelem, "nnode": nnode, "increments_per_step": inc,
                   "element_path": "uniform" if uniform else "general",
                   "l2": "inputs larger than L2 (working set > 0.6 GB); no flush",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": "k_elem_force_quad4_uniform" if uniform
                     else "k_elem_force_general", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "peak_source": peak_src, "ms_per_launch": ms_elem,
                     "alg_bytes_per_launch": b_elem,
                     "fp64": {"achieved_tflops": fp64_ach / 1e12,
                              "peak_tflops": fp64_peak / 1e12,
                              "frac": fp64_ach / fp64_peak,
                              "flops_per_elem": fl_elem,
                              "peak_source": "measured live (gfgpu_probe_fp64)"},
                     "step": {"ms_per_increment": ms_inc, "ms_node_kernel": ms_node,
                              "alg_bytes": b_step,
                              "achieved_gbs": b_step / (ms_inc * 1e-3) / 1e9}},
        "e2e": {"value": e2e_value, "unit": "elem-Gauss-pt/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes},
        "gpu_launches": args.steps * (1 + 2 * inc),
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu:
        threads = 1
        try:
            from oracle import gfref as R

            threads = R.num_threads(True)
            n, t = cpu_sample(w, args.cpu_seconds, True)
            cpu_val = nelem * NIP * n / t
            line["cpu_baseline"] = {
                "value": cpu_val, "unit": "elem-Gauss-pt/s", "cores": threads, "kind": "port",
                "sample": f"{n} increments of the oracle's per-operator loop ({t:.1f} s, "
                          f"{threads} OpenMP threads, {cpu_info()})"}
        except Exception as ex:  # the baseline never blocks the GPU line
            line["cpu_baseline"] = {"value": None, "unit": "elem-Gauss-pt/s", "cores": threads,
                                    "kind": "port", "sample": f"failed: {ex}"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    try:
        return run_gpu(args, rank, world)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
