"""Benchmark: explicit velocity-Verlet dynamics of a 2048 x 2048 Quad4 Regular mesh (FP64 state),
plus the static, batched and learned-preconditioner workloads.

Headline (one bench step = 1000 increments of the explicit scheme of GooseFEM's
docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp): 4,194,304 elements, 4,198,401 nodes,
plane-strain linear elasticity with per-element K ~ U[0.5,1.5], G ~ U[0.25,0.75] (seeded),
density 1 (lumped mass from nodal quadrature), nodal viscous damping 0.1, bottom row fixed,
random initial velocity U[-1e-3, 1e-3], dt = 0.1 x the CFL limit. By default the increments run
in float-float arithmetic (--arith pair: FP64 state in and out, pairs of FP32 numbers inside one
fused kernel per increment); --arith fp64 runs the FP64 kernels. Metric: element-Gauss-point
updates per second (nelem x 4 Gauss points x increments / s).

The default single-GPU run also measures, under "workloads" in the same JSON line:
  static   Hex8 128^3 matrix-free Jacobi-PCG to 1e-8 (vs the oracle's matvec on the host cores),
           the iterations' stiffness action in float-float pairs and in FP64 (--static-operator),
  batch    256 periodic Quad4 instances x 500 increments in the autotuned schedule (FP64 graph,
           persistent kernel or mixed arithmetic) vs the instances one at a time,
  learned  Quad4 512^2 two-phase static solve to 1e-8: learned two-level FCG and the one-level
           learned FCG (network trained on 4096 Jacobi-PCG pairs) vs Jacobi-PCG on the same GPU,
           every solver with the pair stiffness action (FP64 with --static-operator fp64).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gfgpu|reference]
                  [--workload explicit|static|batch|learned] [--no-workloads]

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
    p.add_argument("--workload", default="explicit",
                   choices=["explicit", "static", "batch", "learned"],
                   help="explicit: 2048^2 Quad4 dynamics (headline); static: Hex8 n3d^3 Jacobi-PCG;"
                        " batch: periodic Quad4 instances; learned: n2d^2 learned two-level FCG vs"
                        " Jacobi-PCG")
    p.add_argument("--n3d", type=int, default=128)
    p.add_argument("--n2d", type=int, default=512)
    p.add_argument("--nloads", type=int, default=64)
    p.add_argument("--train-steps", type=int, default=15000)
    p.add_argument("--hc", type=int, default=12, help="learned workload: coarse-grid spacing (nodes)")
    p.add_argument("--cheb-degree", type=int, default=8,
                   help="learned workload: degree of the Chebyshev smoother the network is trained to "
                        "reproduce (its support radius in nodes; the network's receptive field radius is 8)")
    p.add_argument("--margin", type=int, default=8, help="learned workload: crop margin of the loss")
    p.add_argument("--nn-path", type=int, default=2,
                   help="learned workload: tensor-core form of the network's 32->32 layers "
                        "(gfgpu_set_nn_tensor_path: 0 mma.sync, 1 tcgen05, 2 tcgen05 + TMA pipeline, "
                        "3 the same with halo-row reuse)")
    p.add_argument("--profile-iters", type=int, default=0,
                   help="learned workload, kernel-share probe: skip pair generation and training "
                        "and run each solver for this many iterations (untrained network)")
    p.add_argument("--ninst", type=int, default=256)
    p.add_argument("--batch-steps", type=int, default=500)
    p.add_argument("--kernel-variant", default="0,0",
                   help="element,node kernel variant (gfgpu_set_variant): 0 one element / dof per "
                        "thread, 1 two per thread")
    p.add_argument("--path", default="auto", choices=["auto", "uniform", "general"],
                   help="element kernel: auto (fastest applicable), uniform (closed form with K, G "
                        "read every increment) or general (per Gauss point, stored dNx)")
    p.add_argument("--arith", default="pair", choices=["pair", "fp64"],
                   help="explicit workload: float-float fused kernel (pair) or the FP64 kernels")
    p.add_argument("--no-workloads", action="store_true",
                   help="headline only (skip the static, batch and learned workloads)")
    p.add_argument("--static-operator", choices=["both", "pair", "fp64"], default="both",
                   help="static workload: stiffness action of the PCG iterations in float-float "
                        "pairs, in FP64, or both (pair is the reported value where it applies); "
                        "learned workload: pair unless fp64")
    p.add_argument("--train-steps-1level", type=int, default=6000,
                   help="learned workload: Adam steps of the one-level network")
    p.add_argument("--pairs-1level", type=int, default=64,
                   help="learned workload: Jacobi-PCG loads of the one-level pairs (x 64 snapshots)")
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


def cpu_sample(w, seconds, parallel, serial_seconds=0.0):
    """Time the oracle's per-operator explicit loop (the reference algorithm) on the host.
    With serial_seconds > 0 a second sample runs the same loop on one thread (the reference as
    shipped: its OpenMP pragmas are inert) and (n, t, n1, t1) is returned."""
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
    t = run(n)
    if serial_seconds <= 0.0:
        return n, t
    parallel = False
    t1 = run(1)
    n1 = max(1, min(1000, int(serial_seconds / max(t1, 1e-9))))
    return n, t, n1, run(n1)


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


def job_rate(units_per_rank, ms_local, world, device="cpu"):
    """Whole-job throughput of `world` replicas that each processed `units_per_rank` units: the
    slowest rank's time (MAX over ranks) bounds the job. Returns (units/s, max ms)."""
    import torch

    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms = float(t.item())
    return world * units_per_rank / (ms * 1e-3), ms


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


def _event_ms(fn, stream):
    import torch

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def _profile_value(kernel, nx, key):
    """A figure recorded in the ncu summary profiles/<kernel>_<nx>.txt ("key: value" lines)."""
    prof = os.path.join(ROOT, "profiles", f"{kernel}_{nx}.txt")
    if os.path.exists(prof):
        for ln in open(prof):
            if ln.startswith(key + ":"):
                v = ln.split(":", 1)[1].strip()
                try:
                    return float(v)
                except ValueError:
                    return v
    return None


def run_gpu(args, rank, world):
    import torch

    import goosefem_gb300 as gf
    from goosefem_gb300 import _lib

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    ev, nv = (int(t) for t in args.kernel_variant.split(","))
    _lib.call("gfgpu_set_variant", ev, nv)
    w = workload(args.nx, gf.Mesh)
    nnode, nelem, inc = w["nnode"], w["nelem"], args.increments
    pair = args.arith == "pair" and args.path in ("auto", "general")
    vv = gf.VelocityVerlet(w["coor"], w["conn"], w["dofs"], w["K"], w["G"], rho=1.0, dt=w["dt"],
                           eta=w["eta"], iip=w["iip"], uniform=(False if args.path == "general"
                                                                else "auto"),
                           arithmetic="pair" if pair else "fp64")
    if args.path == "uniform":
        vv.use_uniform_onthefly()
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
    value, ms = job_rate(nelem * NIP * inc * args.steps, ms, world, dev)
    ms_inc = ms / (args.steps * inc)

    # ---------------------------------------------------------------- per-kernel timing
    fe = vv.ws
    if pair:
        # the fused increment kernel alone: two calls of different lengths on the launching
        # stream; the difference cancels the per-call FP64 <-> pair conversions
        n1, n2 = 20, 220
        t1 = min(_event_ms(lambda: vv.step(u, v, a, n1), stream) for _ in range(3))
        t2 = min(_event_ms(lambda: vv.step(u, v, a, n2), stream) for _ in range(3))
        ms_kernel = (t2 - t1) / (n2 - n1)
        ms_elem, ms_node = None, None
        # the FP64 kernels on the same state, for comparison
        vv.use_fp64()
        vv.step(u, v, a, 20)
        ms_fp64 = min(_event_ms(lambda: vv.step(u, v, a, 200), stream) for _ in range(2)) / 200
        vv.use_pair()
    else:
        reps = 50
        for _ in range(3):
            _lib.call("gfgpu_verlet_element_forces", C.addressof(vv.desc), u.data_ptr(),
                      fe.data_ptr(), stream.cuda_stream)
        ms_elem = _event_ms(lambda: [_lib.call("gfgpu_verlet_element_forces", C.addressof(vv.desc),
                                               u.data_ptr(), fe.data_ptr(), stream.cuda_stream)
                                     for _ in range(reps)], stream) / reps
        ms_kernel = ms_elem
        ms_node = max(ms_inc - ms_elem, 0.0)
        ms_fp64 = None

    fp64_peak = fp64_probe()

    # ---------------------------------------------------------------- end-to-end (host buffers)
    # through the public Capital method VelocityVerlet.Step: pinned host state in, the step's
    # host state out, every bench step
    hu = torch.zeros((nnode, 2), dtype=torch.float64).pin_memory()
    hv = torch.tensor(w["v0"]).pin_memory()
    ha = torch.zeros((nnode, 2), dtype=torch.float64).pin_memory()
    out = vv.Step(hu, hv, ha, inc)  # warm-up (allocates the pinned outputs)
    barrier()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        out = vv.Step(hu, hv, ha, inc, out=out)
    e1.record(stream)
    barrier()
    ms_e2e = 1e3 * (time.perf_counter() - t0)
    e2e_value, ms_e2e = job_rate(nelem * NIP * inc * args.steps, ms_e2e, world, dev)
    state_bytes = 3 * nnode * 2 * 8

    if rank != 0:
        return 0

    # ---------------------------------------------------------------- roofline
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        hbm_peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    path = vv.path
    kernel = {"uniform-square-pair": "k_verlet_pair_tma", "general-pair": "k_pair_elem_stiff",
              "uniform-square": "k_elem_force_quad4_square", "uniform": "k_elem_force_quad4_uniform",
              "general": "k_elem_force_general"}[path]
    # fused-step minimum traffic (SURVEY-defined algorithmic bytes of one increment): u, v, a
    # read+write (96 B/node), inverse mass (16 B/node), K, G (16 B/elem)
    b_step = 112 * nnode + 16 * nelem
    if pair:
        # one fused kernel per increment: its algorithmic bytes are the increment's
        b_launch = b_step
    else:
        # element kernel: u (16 B/node), conn (16 B/elem), material (K, G: 16 B/elem, or the 4
        # precomputed coefficients: 32 B/elem), element forces out (64 B/elem); the general path
        # also streams dNx and vol (72 B/elem)
        mat = 32 if path == "uniform-square" else 16
        b_launch = 16 * nnode + (16 + mat + 64) * nelem + (72 * nelem if path == "general" else 0)
    achieved = b_launch / (ms_kernel * 1e-3) / 1e9
    traffic = _profile_value(kernel, args.nx, "dram_bytes_per_launch")
    binding = _profile_value(kernel, args.nx, "binding_resource")
    roof = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm_peak,
            "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
            "peak_source": peak_src, "ms_per_launch": ms_kernel, "alg_bytes_per_launch": b_launch,
            "step": {"ms_per_increment": ms_inc, "alg_bytes": b_step,
                     "achieved_gbs": b_step / (ms_inc * 1e-3) / 1e9,
                     "frac": b_step / (ms_inc * 1e-3) / 1e9 / hbm_peak}}
    if binding is not None:
        roof["binding_resource"] = binding
    if pair:
        roof["fp64_kernels"] = {
            "ms_per_increment": ms_fp64, "value": nelem * NIP / (ms_fp64 * 1e-3),
            "note": "the FP64 element + node kernels on the same state (34 + 2 x 10 FP64 "
                    "instructions per node, at GB300's FP64 issue rate)",
            "fp64_probe_tflops": fp64_peak / 1e12}
    else:
        # FP64 operations of the element kernel per element, DFMA counted as 2
        fl_elem = {"uniform-square": 36, "uniform": 55, "general": 4 * (2 * 25 + 7 + 2 * 16 + 8)}[path]
        in_elem = {"uniform-square": 34, "uniform": 48, "general": 4 * (25 + 7 + 16 + 8)}[path]
        roof["bound"] = "fp64"
        roof["step"]["ms_node_kernel"] = ms_node
        roof["fp64"] = {"achieved_tflops": fl_elem * nelem / (ms_elem * 1e-3) / 1e12,
                        "peak_tflops": fp64_peak / 1e12,
                        "frac": fl_elem * nelem / (ms_elem * 1e-3) / fp64_peak,
                        "instr_per_elem": in_elem,
                        "achieved_ginstr_s": in_elem * nelem / (ms_elem * 1e-3) / 1e9,
                        "peak_ginstr_s": fp64_peak / 2.0 / 1e9,
                        "instr_frac": in_elem * nelem / (ms_elem * 1e-3) / (fp64_peak / 2.0),
                        "peak_source": "measured live (gfgpu_probe_fp64: DFMA chains)"}
    line = {
        "metric": "elem-Gauss-pt updates/s", "value": value, "unit": "elem-Gauss-pt/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32x2 (float-float pairs, 48-bit significands; FP64 state in and out)"
                  if pair else "f64"),
        "data": "synthetic (seeded)",
        "config": {"workload": f"Quad4 Regular {args.nx}x{args.nx} explicit velocity-Verlet, "
                               "per-element K,G, density 1, damping 0.1, bottom row fixed",
                   "nelem": nelem, "nnode": nnode, "increments_per_step": inc,
                   "element_path": path, "arithmetic": vv.arithmetic,
                   "kernel_variant": args.kernel_variant,
                   "l2": "inputs larger than L2 (working set > 0.5 GB); no flush",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": "elem-Gauss-pt/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes,
                "via": "VelocityVerlet.Step (pinned host u, v, a in and out every step)"},
        "gpu_launches": args.steps * ((inc + 2) if pair else (1 + 2 * inc)),
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu:
        threads = 1
        try:
            from oracle import gfref as R

            threads = R.num_threads(True)
            n, t, n1, t1 = cpu_sample(w, args.cpu_seconds, True, serial_seconds=args.cpu_seconds / 2)
            cpu_val = nelem * NIP * n / t
            line["cpu_baseline"] = {
                "value": cpu_val, "unit": "elem-Gauss-pt/s", "cores": threads, "kind": "port",
                "sample": f"{n} increments of the oracle's per-operator loop ({t:.1f} s, "
                          f"{threads} OpenMP threads, {cpu_info()})",
                "serial": {"value": nelem * NIP * n1 / t1, "cores": 1,
                           "sample": f"{n1} increments on one thread ({t1:.1f} s): the reference "
                                     "as shipped runs serially"}}
        except Exception as ex:  # the baseline never blocks the GPU line
            line["cpu_baseline"] = {"value": None, "unit": "elem-Gauss-pt/s", "cores": threads,
                                    "kind": "port", "sample": f"failed: {ex}"}
    del vv, u, v, a, hu, hv, ha, out, fe
    torch.cuda.empty_cache()
    if world == 1 and not args.no_workloads:
        line["workloads"] = {}
        for name, fn in (("static", workload_static), ("batch", workload_batch),
                         ("learned", workload_learned)):
            try:
                line["workloads"][name] = _with_clocks(fn, args)
            except Exception as ex:  # a failing workload is reported, not fatal to the line
                line["workloads"][name] = {"error": f"{type(ex).__name__}: {ex}"}
            torch.cuda.empty_cache()
    print(json.dumps(line), flush=True)
    return 0


def _with_clocks(fn, args):
    import torch

    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    t0 = time.perf_counter()
    try:
        res = fn(args)
    finally:
        clocks = sampler.stop()
    res["clocks"] = clocks
    res["wall_seconds"] = time.perf_counter() - t0
    return res


def static_case(n, seed=3):
    """Hex8 Regular n^3 (h = 1), K ~ U[0.5,1.5], G ~ U[0.25,0.75] per element, z = 0 face fixed,
    z = top face uz = -1e-2 (ux, uy free). The mesh comes from the package's own Mesh.Hex8."""
    import goosefem_gb300 as gf

    mesh = gf.Mesh.Hex8.Regular(n, n, n)
    coor, conn = mesh.coor(), mesh.conn()
    rng = np.random.default_rng(seed)
    K = rng.uniform(0.5, 1.5, n ** 3)
    G = rng.uniform(0.25, 0.75, n ** 3)
    nxy = (n + 1) ** 2
    front = np.arange(nxy)
    back = front + n * nxy
    iip = np.unique(np.concatenate([(front[:, None] * 3 + np.arange(3)).ravel(), back * 3 + 2]))
    xp = np.where(np.isin(iip, back * 3 + 2), -1e-2, 0.0)
    return coor, conn, K, G, iip, xp


def network_ms(lp, n):
    """One network application on the n x n nodal grid (gfgpu_nn_infer: the four layers of the
    preconditioner's correction), CUDA events over 50 applications after 5 warm-ups."""
    import ctypes as C

    import torch

    from goosefem_gb300 import _lib

    X0 = torch.randn((n, n, 4), dtype=torch.float32, device="cuda")
    Y = torch.empty((n, n, 2), dtype=torch.float32, device="cuda")
    wsi = torch.empty(int(_lib_call_bytes(n, n)) // 8 + 1, dtype=torch.float64, device="cuda")
    nnd = lp.nn_desc()
    st = torch.cuda.current_stream()

    def call():
        _lib.call("gfgpu_nn_infer", C.addressof(nnd), X0.data_ptr(), Y.data_ptr(), wsi.data_ptr(),
                  st.cuda_stream)

    for _ in range(5):
        call()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(50):
        call()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 50


def fp64_probe():
    """Measured FP64 FLOP/s of independent DFMA chains on every SM (gfgpu_probe_fp64), the FP64
    roof the element kernels are held against (2 FLOP per DFMA)."""
    import torch

    from goosefem_gb300 import _lib

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 16, 10000
    _lib.call("gfgpu_probe_fp64", blocks, 1000, out.data_ptr(), stream.cuda_stream)
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    _lib.call("gfgpu_probe_fp64", blocks, iters, out.data_ptr(), stream.cuda_stream)
    k1.record(stream)
    torch.cuda.synchronize()
    return 2.0 * 16 * iters * blocks * 256 / (k0.elapsed_time(k1) * 1e-3)


def workload_static(args):
    """3-d static case: Hex8 n3d^3 matrix-free Jacobi-PCG to 1e-8 relative residual (FP64
    solution, residuals and dot products), two timed solves from a zero initial guess (best
    counts), with the stiffness action of the iterations in float-float pairs (the headline of this
    workload) and in FP64, against the oracle's matrix-free operator (one stiffness action) on the
    host cores."""
    import torch

    import goosefem_gb300 as gf

    n = args.n3d
    coor, conn, K, G, iip, xp = static_case(n)
    nnode = coor.shape[0]
    dofs = np.arange(nnode * 3).reshape(nnode, 3)
    iip_d = torch.as_tensor(iip, device="cuda").long()
    xp_d = torch.as_tensor(xp, device="cuda")
    x = torch.zeros((nnode, 3), dtype=torch.float64, device="cuda")

    def timed(st):
        def solve():
            x.zero_()
            x.view(-1)[iip_d] = xp_d
            return st.solve(x, tol=1e-8, check_every=16)

        solve()  # warm-up
        torch.cuda.synchronize()
        secs, its = [], []
        for _ in range(2):
            t0 = time.perf_counter()
            its.append(solve())
            torch.cuda.synchronize()
            secs.append(time.perf_counter() - t0)
        sec = min(secs)
        it, rel = its[-1]
        return {"seconds": sec, "iterations": it, "relres_true": rel,
                "ms_per_iteration": sec * 1e3 / it}

    uni = "auto" if args.path == "auto" else False
    st = gf.ElasticStatic(coor, conn, dofs, K, G, iip, uniform=uni)
    path = ("uniform-cube" if st.coef is not None else "uniform") if st.uniform else "general"
    pair_ok = int(gf._lib.lib().gfgpu_pcg_pair_coef_floats(C.addressof(st.desc))) > 0
    fp64 = timed(st) if args.static_operator in ("both", "fp64") or not pair_ok else None
    if fp64 is not None and st.coef is not None and st.desc.reg_nz > 0:
        # FP64 instructions of one iteration of the cube / Regular path: element kernel ~171 per
        # element, gather 8 adds + 1 FMA, update 5 per free dof, direction 1 per dof
        nfree = nnode * 3 - iip.size
        instr = 171 * n ** 3 + 14 * nfree + nnode * 3
        peak = fp64_probe() / 2.0
        sec_it = fp64["ms_per_iteration"] * 1e-3
        fp64["fp64"] = {"instr_per_iteration": instr, "achieved_ginstr_s": instr / sec_it / 1e9,
                        "peak_ginstr_s": peak / 1e9, "instr_frac": instr / sec_it / peak,
                        "peak_source": "measured live (gfgpu_probe_fp64: DFMA chains)"}
    pair = None
    if pair_ok and args.static_operator in ("both", "pair"):
        st.use_pair()
        pair = timed(st)
    head = pair if pair is not None else fp64
    res = {"metric": "time-to-1e-8 resid (Jacobi-PCG)", "value": head["seconds"], "unit": "s",
           "higher_is_better": False,
           "dtype": ("f64 solve, float-float (f32 pair) stiffness action in the iterations"
                     if pair is not None else "f64"),
           "data": "synthetic (seeded)",
           "config": {"workload": f"Hex8 Regular {n}^3 static, z=0 fixed, top uz=-1e-2, "
                                  "matrix-free Jacobi-PCG", "element_path": path,
                      "operator_arithmetic": "pair" if pair is not None else "fp64",
                      "solves_timed": 2},
           "iterations": head["iterations"], "relres_true": head["relres_true"],
           "ms_per_iteration": head["ms_per_iteration"],
           "elem_updates_per_s": n ** 3 * 8 * head["iterations"] / head["seconds"],
           "fp64_operator": fp64}
    if pair is not None and fp64 is not None:
        res["speedup_vs_fp64_operator"] = fp64["seconds"] / pair["seconds"]
    del st, x
    if not args.no_cpu:
        try:
            res["cpu_baseline"] = static_cpu_matvec(coor, conn, K, G)
            res["cpu_baseline"]["gpu_ms_per_iteration"] = res["ms_per_iteration"]
        except Exception as ex:
            res["cpu_baseline"] = {"error": f"{type(ex).__name__}: {ex}"}
    return res


def static_cpu_matvec(coor, conn, K, G):
    """One stiffness action of the oracle (the reference's per-operator chain: AsElement,
    SymGradN_vector, stress, Int_gradN_dot_tensor2_dV, AssembleNode) on all host threads; the set-up
    (compute_dN) is not timed."""
    from oracle import gfref as R

    threads = R.num_threads(True)
    xr = R.as_element(conn, coor)
    dNx, vol = R.compute_dN(xr, *R.hex8_gauss(), parallel=True)
    del xr
    u = np.random.default_rng(11).uniform(-1e-3, 1e-3, coor.shape)
    t0 = time.perf_counter()
    ue = R.as_element(conn, u)
    eps = R.sym_grad_n_vector(dNx, ue, parallel=True)
    sig = R.elastic_stress(eps, K, G, parallel=True)
    fe = R.int_grad_n_dot_tensor2_dv(dNx, vol, sig, parallel=True)
    R.assemble_node(conn, np.arange(coor.shape[0] * 3).reshape(-1, 3), fe)
    t = time.perf_counter() - t0
    return {"value": t, "unit": "s per stiffness action", "cores": threads, "kind": "port",
            "sample": f"one matrix-free stiffness action of the oracle at {conn.shape[0]} Hex8 "
                      f"elements, {threads} OpenMP threads ({cpu_info()}); the element loops in "
                      "parallel, the assembly serial as in the reference"}


def run_static(args):
    print(json.dumps(workload_static(args)), flush=True)
    return 0


def workload_batch(args):
    """256 periodic Quad4 instances (nx, ny ~ U{32..512}), 500 increments each, one batched
    launch schedule (autotuned) vs the instances one at a time."""
    import torch

    from goosefem_gb300 import batch as B

    inst = B.seeded_instances(args.ninst, 256)
    bv = B.BatchedVerlet(inst)
    table = bv.autotune(nsteps=20, reps=2)
    # the pair schedule beside it (not a candidate: see BatchedVerlet.autotune), with its deviation
    mode0 = (bv.mode, bv.block, bv.bps)
    bv.mode = 2
    up, vp, ap = bv.state()
    bv.run_direct(up, vp, ap, 5)
    torch.cuda.synchronize()
    up, vp, ap = bv.state()
    e0p, e1p = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0p.record()
    bv.run_direct(up, vp, ap, args.batch_steps)
    e1p.record()
    torch.cuda.synchronize()
    pair_ms = e0p.elapsed_time(e1p) / args.batch_steps
    bv.mode, bv.block, bv.bps = mode0
    nsteps = args.batch_steps
    u, v, a = bv.state()
    bv.run_graph(u, v, a, nsteps)  # warm-up (also builds the graph)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    u, v, a = bv.state()
    e0.record()
    bv.run_graph(u, v, a, nsteps)
    e1.record()
    torch.cuda.synchronize()
    if bv.mode == 1:
        bv.check_status()
    sec = e0.elapsed_time(e1) * 1e-3
    pair_dev = {k: float((x - y).abs().max() / y.abs().max()) for k, x, y in (("u", up, u), ("v", vp, v), ("a", ap, a))}
    dev = None
    if bv.mode == 3:
        # the chosen (mixed) schedule against the FP64 graph on the same increments
        mode_c = (bv.mode, bv.block, bv.bps)
        bv.mode, bv.block, bv.bps = 0, 256, 0
        u64, v64, a64 = bv.state()
        bv.run_direct(u64, v64, a64, nsteps)
        torch.cuda.synchronize()
        bv.mode, bv.block, bv.bps = mode_c
        dev = {k: float((x - y).abs().max() / y.abs().max())
               for k, x, y in (("u", u, u64), ("v", v, v64), ("a", a, a64))}
    seq = B.run_sequential(inst, nsteps, bv.dt, arithmetic=bv.arithmetic)
    res = {"metric": "elem-Gauss-pt updates/s (batched)", "value": bv.nelem * 4 * nsteps / sec,
           "unit": "elem-Gauss-pt/s", "higher_is_better": True,
           "dtype": ("f64 state and predictor, float-float (f32 pair) element forces and "
                     "velocity estimates" if bv.mode == 3 else "f64"),
           "data": "synthetic (seeded)",
           "config": {"workload": f"{len(inst)} periodic Quad4 Regular instances, nx,ny~U{{32..512}},"
                                  f" {nsteps} increments, applied shear 1e-3",
                      "nelem_total": bv.nelem,
                      "schedule": {"mode": ["graph of 2 FP64 kernels", "persistent FP64 kernel",
                                            "graph of 2 pair kernels",
                                            "graph of the mixed element kernel (pair closed form on "
                                            "FP64 node differences) + the mixed node kernel"][bv.mode],
                                   "block": bv.block, "blocks_per_sm": bv.bps},
                      "colouring": "none: the node kernels gather through the dof CSR "
                                   "(deterministic, no scatter conflicts to colour)"},
           "seconds": sec, "ms_per_increment": 1e3 * sec / nsteps,
           "max_rel_dev_vs_fp64": dev,
           "accuracy_note": ("mixed: FP64 state and predictor, pair element forces on FP64 node "
                             "differences and pair velocity estimates; over 500 sheared increments it "
                             "is as close to the reference "
                             "algorithm as the FP64 fast path is (both ~1e-12 on 24-40^2 instances; "
                             "tests/test_gpu_batch.py), the deviation above is the two arithmetics' "
                             "shared spread" if bv.mode == 3 else None),
           "pair_schedule": {"ms_per_increment": pair_ms, "max_rel_dev_vs_fp64": pair_dev,
                             "note": "graph of the float-float element + CSR node kernels; not chosen: "
                                     "the applied shear makes the displacement ~600x its fluctuations, "
                                     "and the pair rounding of the displacement then exceeds the 1e-12 "
                                     "agreement"},
           "sequential_seconds": seq,
           "speedup_vs_sequential": seq / sec,
           "autotune": [{"mode": r[0], "block": r[1], "bps": r[2], "ms_per_increment": r[3]}
                        for r in table]}
    bv.release()
    return res


def run_batch(args):
    print(json.dumps(workload_batch(args)), flush=True)
    return 0


def _lib_call_bytes(H, W):
    from goosefem_gb300 import _lib

    return _lib.lib().gfgpu_nn_infer_workspace_bytes(H, W)


def _learned_problem(args):
    from goosefem_gb300 import learned as LR
    from goosefem_gb300 import mesh as M

    nx = args.n2d
    K, G, inside = LR.inclusion_material(nx, nx, 512)
    m = M.Quad4.Regular(nx, nx)
    iip, xp = LR.static_bc(m)
    return LR, nx, K, G, inside, iip, xp


def run_learned(args):
    """Kernel-share probe of the learned workload (--profile-iters > 0), else the workload line."""
    import torch

    from goosefem_gb300 import _lib

    if args.profile_iters <= 0:
        print(json.dumps(workload_learned(args)), flush=True)
        return 0
    _lib.call("gfgpu_set_nn_tensor_path", int(args.nn_path))
    LR, nx, K, G, inside, iip, xp = _learned_problem(args)
    lp = LR.LearnedPreconditioner(nx, nx, K, G, iip, seed=0)
    # the coarse set-up, then each two-level solver for a fixed number of iterations (untrained
    # network)
    lp.coarse_setup(args.hc)
    k = args.profile_iters
    for name, kw in (("twolevel", dict(use_nn=False, nkeep=1)),
                     ("learned_twolevel_keep4", dict(use_nn=True, nkeep=4, post=True))):
        x = lp.initial_guess(xp)
        try:
            lp.fcg(x, maxiter=k, coarse=True, **kw)
        except _lib.GFGPUError as e:
            if e.code != -8:
                raise
    torch.cuda.synchronize()
    print(json.dumps({"workload": "learned kernel-share probe (untrained network)",
                      "config": {"nx": nx, "hc": args.hc, "iterations": k,
                                 "nn_path": args.nn_path},
                      "network_application_ms": network_ms(lp, nx + 1)}), flush=True)
    return 0


def workload_learned(args):
    """Quad4 512^2 two-phase static case, every solve to 1e-8 relative residual in FP64
    (time-to-solution on the same GPU; coarse set-up, pair generation and training reported
    apart): Jacobi-PCG (the baseline; step-by-step session solver and the ring solver with the
    Jacobi direction alone replayed as a CUDA graph, the faster of the two counts), the two-level
    flexible CG without the network (the method without it), the learned two-level solve (the
    network as the post-smoother of the two-level step) and the one-level learned flexible CG
    (the network trained on 4096 (residual, Jacobi-PCG correction) pairs as the second direction
    beside Jacobi)."""
    import torch

    from goosefem_gb300 import _lib as _L

    _L.call("gfgpu_set_nn_tensor_path", int(args.nn_path))
    LR, nx, K, G, inside, iip, xp = _learned_problem(args)
    # the stiffness action of every solver's iterations (Jacobi-PCG, two-level, learned) in
    # float-float pairs, or all in FP64 (--static-operator fp64)
    op = "fp64" if args.static_operator == "fp64" else "pair"
    lp = LR.LearnedPreconditioner(nx, nx, K, G, iip, seed=0, arithmetic=op)
    reps = 2

    def timed(fn, l=lp):
        x = l.initial_guess(xp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn(x)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0,) + tuple(out)

    def best_of(fn, l=lp):
        timed(fn, l)  # warm-up
        return min((timed(fn, l) for _ in range(reps)), key=lambda r: r[0])

    res = {}
    for name, fn in (("jacobi_pcg", lambda x: lp.jacobi_pcg(x)),
                     ("jacobi_pcg_graph", lambda x: lp.fcg(x, use_nn=False, nkeep=1))):
        b = best_of(fn)
        res[name] = {"seconds": b[0], "iterations": b[1], "relres_true": b[2]}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lp.coarse_setup(args.hc)
    torch.cuda.synchronize()
    t_coarse = time.perf_counter() - t0
    for ce in (4, 8, 16):  # residual checked between graph replays of ce iterations
        b = best_of(lambda x: lp.fcg(x, use_nn=False, nkeep=1, coarse=True, check_every=ce))
        res[f"twolevel_check{ce}"] = {"seconds": b[0], "iterations": b[1], "relres_true": b[2]}
    res["twolevel"] = min((v for k, v in res.items() if k.startswith("twolevel_check")),
                          key=lambda v: v["seconds"])
    # the training pairs come from solves with the FP64 stiffness action (the network learns the
    # solver of the reference's arithmetic); the timed solves use `op`
    lp.static.use_fp64()
    t0 = time.perf_counter()
    npairs = lp.make_pairs_twolevel(nloads=args.nloads, snaps=64, every=4, target="cheb",
                                    degree=args.cheb_degree, post=True)
    torch.cuda.synchronize()
    t_pairs = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = lp.train(steps=args.train_steps, batch=32, crop=96, margin=args.margin, lr=2e-3,
                      log_every=max(args.train_steps // 10, 1))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    if op == "pair":
        lp.static.use_pair()
    for nkeep in (1, 2, 4):
        for ce in (2, 4):
            b = best_of(lambda x: lp.solve(x, nkeep=nkeep, check_every=ce))
            res[f"learned_twolevel_keep{nkeep}_check{ce}"] = {
                "seconds": b[0], "iterations": b[1], "fallback_iterations": b[2], "relres_true": b[3]}
    res["learned_twolevel"] = min((v for k, v in res.items() if k.startswith("learned_twolevel_keep")),
                                  key=lambda v: v["seconds"])
    nn_ms = network_ms(lp, nx + 1)
    del lp
    torch.cuda.empty_cache()
    # the one-level design: 4096 (residual, Jacobi-PCG correction) pairs from the plain solver
    # (64 random loads x 64 snapshots every 16 iterations; target PCG_8(r) - D^-1 r), the network
    # as the second direction of the flexible CG beside Jacobi, no coarse grid
    lp1 = LR.LearnedPreconditioner(nx, nx, K, G, iip, seed=0)  # FP64 action for the pairs
    t0 = time.perf_counter()
    np1 = lp1.make_pairs(nloads=args.pairs_1level, snaps=64, every=16, inner=8)
    torch.cuda.synchronize()
    t_pairs1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses1 = lp1.train(steps=args.train_steps_1level, batch=32, crop=96, margin=args.margin,
                        lr=2e-3, log_every=max(args.train_steps_1level // 10, 1))
    torch.cuda.synchronize()
    t_train1 = time.perf_counter() - t0
    lp1.R = lp1.T = None
    if op == "pair":
        lp1.static.use_pair()
    # ring of 8 directions (shorter rings needed up to 20x more iterations in trial runs); the
    # iteration cap bounds the time of a network that does not help
    cap = 4 * res["jacobi_pcg"]["iterations"]
    try:
        b = best_of(lambda x: lp1.fcg(x, use_nn=True, nkeep=8, check_every=16, maxiter=cap), lp1)
        res["learned_onelevel"] = {"seconds": b[0], "iterations": b[1], "relres_true": b[2],
                                   "directions_kept": 8}
    except _L.GFGPUError as e:
        if e.code != -8:
            raise
        res["learned_onelevel"] = {"seconds": float("inf"), "iterations": cap,
                                   "relres_true": None, "directions_kept": 8,
                                   "note": f"not converged within {cap} iterations"}
    del lp1
    for v in res.values():
        v["us_per_iteration"] = 1e6 * v["seconds"] / max(v["iterations"] + v.get("fallback_iterations", 0), 1)
    jac = min(res["jacobi_pcg"]["seconds"], res["jacobi_pcg_graph"]["seconds"])
    learned = res["learned_twolevel"]
    one = res["learned_onelevel"]
    return {"metric": "time-to-1e-8 resid (learned FCG vs Jacobi PCG)",
            "value": learned["seconds"], "unit": "s", "higher_is_better": False,
            "dtype": ("f64 solve, " + ("float-float (f32 pair) stiffness action in the iterations, "
                                       if op == "pair" else "") +
                      "bf16-weight/fp32-accumulate network, fp32 coarse correction"),
            "data": "synthetic (seeded inclusions)",
            "config": {"workload": f"Quad4 Regular {nx}x{nx}, two-phase (inclusions "
                                   f"{100 * inside.mean():.1f}% area, x10 moduli), bottom fixed, "
                                   "top uy=-1e-2", "coarse_spacing": args.hc,
                       "pairs_twolevel": npairs, "pairs_onelevel": np1,
                       "train_steps": args.train_steps, "train_steps_onelevel": args.train_steps_1level,
                       "crop": 96, "margin": args.margin, "chebyshev_degree": args.cheb_degree,
                       "residual_check": "best of every 2, 4 (learned two-level), 4, 8, 16 "
                                         "(two-level) and 16 (one-level) iterations",
                       "target_twolevel": "Chebyshev smoother minus Jacobi step, on the residual "
                                          "after the two-level step",
                       "target_onelevel": "8 Jacobi-PCG iterations minus the Jacobi step",
                       "loss": "energy norm", "nn_tensor_path": args.nn_path,
                       "operator_arithmetic": op},
            "solvers": res,
            "speedup_vs_jacobi_pcg": jac / learned["seconds"],
            "speedup_vs_twolevel_without_network": res["twolevel"]["seconds"] / learned["seconds"],
            "network_gain_iterations": res["twolevel"]["iterations"] / max(learned["iterations"], 1),
            "onelevel_speedup_vs_jacobi_pcg": (jac / one["seconds"]) if one["seconds"] > 0 else None,
            "iteration_ratio_vs_jacobi_pcg": res["jacobi_pcg"]["iterations"] / max(learned["iterations"], 1),
            "coarse_setup_seconds": t_coarse, "pair_generation_seconds": t_pairs,
            "training_seconds": t_train, "pair_generation_seconds_onelevel": t_pairs1,
            "training_seconds_onelevel": t_train1, "network_application_ms": nn_ms,
            "loss_first_last": [losses[0], losses[-1]],
            "loss_first_last_onelevel": [losses1[0], losses1[-1]]}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "static":
        return run_static(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "learned":
        return run_learned(args)
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
