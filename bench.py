#!/usr/bin/env python
"""Benchmark of the VoxelFEM solve path on GB300.

Workload: the 3D cantilever at 256x128x128 trilinear voxels (12.83M DOF),
densities uniform[0.01, 1] (seed 0), E0 = 1, Emin = 1e-9, nu = 0.3, SIMP p = 3,
6-level geometric multigrid (5 coarsenings), mgIterations = 1, 2 pre- and 2
post-sweeps of the coloured block Gauss-Seidel, plain V-cycles, x0 = 0,
relative residual 1e-8.

A step is one MG-PCG solve from PCG entry to ||r||/||b|| <= 1e-8, including the
density upload and the Galerkin rebuild of the hierarchy it triggers. ``value``
is the mixed-precision (FP32 V-cycle, FP64 outer CG) time per solve with all
inputs resident in HBM; the FP64 solve (the reference's method) is timed beside
it. ``e2e`` is the same step through the public API with pinned host buffers.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--config c1|c2]

With N > 1 (torchrun), every rank solves its own replica; the line reports the
aggregate time per solve (max-over-ranks duration / (N * K)).
"""
import argparse
import concurrent.futures
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "MG-PCG time-to-1e-8 residual (mixed vs FP64, 12.7M DOF); applyK HBM GB/s"
CONFIGS = {
    # name: (elements, rho_lo, coarsenings)
    "c2": ((256, 128, 128), 0.01, 5),
    "c1": ((64, 32, 32), 0.3, 3),
}
TOL = 1e-8
KERNEL_NAMES = {0: "applyk_fine_fp64", 1: "applyk_fine_fp32", 2: "applyk_fine_df", 3: "gs_fine_sweep_fp32",
                4: "gs_fine_sweep_fp64", 5: "residual_fine_fp32", 6: "gs_level1_sweep_fp32",
                7: "residual_level1_fp32", 8: "gs_level2_sweep_fp32", 9: "residual_level2_fp32",
                10: "applyk_fine_tc"}


def tc_mma_flops(ne):
    """bf16 MMA flops one launch of the tensor-core matvec issues: per CTA step (one element layer
    of an 8 x 16 element tile) 16 MMAs of 128 x 32 x 16; a CTA walks its x segment plus one layer."""
    nn = [v + 1 for v in ne]
    cols = -(-nn[1] // 7) * -(-nn[2] // 15)
    seg = max(1, min(int(round(8.0 * 152 / cols)), nn[0]))
    seg_len = -(-nn[0] // seg)
    n_seg = -(-nn[0] // seg_len)
    steps = cols * (nn[0] + n_seg)
    return steps * 16 * 2.0 * 128 * 32 * 16


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f).get("bf16_tflops", 1900.0))
    return 1900.0


def fp64_peak_tflops(n=4096, reps=5):
    """FP64 throughput of this GPU, measured with a cuBLAS DGEMM (best of two timed batches)."""
    import torch

    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(2):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3 / reps
        best = t if best is None else min(best, t)
    return 2.0 * n ** 3 / best / 1e12


def fp32_peak_tflops(n=8192, reps=5):
    """FP32 FMA throughput of this GPU, measured with a cuBLAS SGEMM with TF32 off (FFMA on the
    CUDA cores; best of two timed batches), the denominator of the FP32-pipe rooflines."""
    import torch

    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, dtype=torch.float32, device="cuda")
        b = torch.randn(n, n, dtype=torch.float32, device="cuda")
        torch.matmul(a, b)
        best = None
        for _ in range(2):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1) * 1e-3 / reps
            best = t if best is None else min(best, t)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return 2.0 * n ** 3 / best / 1e12


def level1_contraction_tc_probe(nc_elems, reps=20):
    """The level-1 operator as the reference applies it, Sum_f E_f Kc_f u_c over the coarse
    elements (MultigridSolver.hh:475-499), cast as one tensor-core GEMM [Kc_0 ... Kc_7] (192 x 24)
    times U_c (24 x coarse elements) through cuBLAS: device time in bf16 (one product; FP32-class
    accuracy would need a three-way split of both operands, six products) and in TF32, with the
    192-row output written in the operands' precision. The E-weighted combine and the gather of
    U_c are not included, so this is a lower bound on a tensor-core level-1 residual."""
    import torch

    out = {"shape": [192, 24, int(nc_elems)], "flops": 2.0 * 192 * 24 * nc_elems}
    prev = torch.backends.cuda.matmul.allow_tf32
    try:
        for name, dt, tf32 in (("bf16", torch.bfloat16, False), ("tf32", torch.float32, True)):
            torch.backends.cuda.matmul.allow_tf32 = tf32
            a = torch.randn(192, 24, dtype=dt, device="cuda")
            b = torch.randn(24, int(nc_elems), dtype=dt, device="cuda")
            torch.matmul(a, b)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out[name + "_ms"] = ms
            out[name + "_tflops"] = out["flops"] / (ms * 1e-3) / 1e12
            out[name + "_output_bytes"] = 192 * int(nc_elems) * (2 if dt == torch.bfloat16 else 4)
            del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    out["bf16_split3_ms_estimate"] = 6 * out["bf16_ms"]
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value, ws, device="cuda"):
    """The largest of every rank's value: replicas finish when their slowest rank does."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_per_solve(t_max, ws, steps):
    """Whole-job time per solve of ws replicas that each ran `steps` solves in t_max seconds
    (the slowest rank's time): ws * steps solves in t_max."""
    return t_max / (ws * steps)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def phase_breakdown(lib, capi, mg_h, reps=3):
    import ctypes as C
    names = C.create_string_buffer(16384)
    ms = (C.c_double * 256)()
    n = C.c_int()
    capi.check(lib.vfem_mg_profile(mg_h, 1, 2, reps, names, 16384, ms, 256, C.byref(n)))
    keys = names.value.decode().strip().split("\n")
    return {k: round(ms[i], 4) for i, k in enumerate(keys[: n.value])}


def cpu_baseline_solve(cfg_name, threads=None):
    """One complete FP64 MG-PCG solve of the workload by the CPU oracle (a restatement of the
    reference's solver), timed like the GPU step: from the density upload (which invalidates the
    hierarchy) through the Galerkin rebuild (the oracle's PCG rebuilds the hierarchy's operators on
    entry, as the reference's does) and the PCG iterations to relative residual 1e-8."""
    from oracle import pyoracle as po
    from voxelfem_gb300 import workloads as wl
    ne, rho_lo, levels = CONFIGS[cfg_name]
    threads = threads or os.cpu_count()
    po.set_num_threads(threads)
    sim = po.Sim(ne)
    rho, _ = wl.setup_cantilever(sim, ne, rho_lo, 0)
    mg = po.MG(sim, levels)
    b = sim.buildLoadVector()
    x0 = np.zeros_like(b)
    t0 = time.perf_counter()
    sim.setDensities(rho)
    x = mg.preconditionedConjugateGradient(x0, b, 500, TOL, None, 1, 2, False)
    t1 = time.perf_counter()
    return {"value": t1 - t0, "unit": "s", "cores": threads, "kind": "port",
            "sample": "complete CPU-oracle FP64 MG-PCG solve of the %s cantilever %dx%dx%d (density upload, Galerkin "
                      "rebuild, %d PCG iterations to relres %.2e), OpenMP over %d host threads"
                      % (cfg_name, ne[0], ne[1], ne[2], mg.lastIterations, mg.lastRelativeResidual, threads),
            "iterations": int(mg.lastIterations), "relres": float(mg.lastRelativeResidual),
            "compliance": float(0.5 * np.sum(b * x))}


def run_reference(args):
    """The reference arm: the CPU oracle's complete FP64 solves of the same workload on the host
    cores, one solve per step (no extrapolation)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cfg = args.config
    vals, last = [], None
    for _ in range(args.warmup):  # untimed: page-in of the oracle library, thread pool, first-touch
        cpu_baseline_solve(cfg)
    t_all = time.perf_counter()
    for _ in range(args.steps):
        last = cpu_baseline_solve(cfg)
        vals.append(last["value"])
    t_all = time.perf_counter() - t_all
    v = float(np.mean(vals))
    ne = CONFIGS[cfg][0]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1000, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "cantilever %dx%dx%d Q1, rho U[%g,1] seed 0, %d coarsenings, FP64 MG-PCG to 1e-8"
                       % (ne[0], ne[1], ne[2], CONFIGS[cfg][1], CONFIGS[cfg][2])},
            "cpu_baseline": {"value": v, "unit": "s", "cores": last["cores"], "kind": last["kind"],
                             "sample": last["sample"]},
            "iterations": last["iterations"], "compliance": last["compliance"],
            "timed_region_s": t_all, "min_s": float(min(vals)), "max_s": float(max(vals)),
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes as C

    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()

    from voxelfem_gb300 import _capi
    from voxelfem_gb300 import pyVoxelFEM as pv
    from voxelfem_gb300 import workloads as wl

    lib = _capi.load()
    ne, rho_lo, levels = CONFIGS[args.config]
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    sim = pv.TensorProductSimulator([1, 1, 1], bbox, ne)
    rho, f = wl.setup_cantilever(sim, ne, rho_lo, 0)
    mg = sim.multigridSolver(levels)
    if args.host_loop:
        mg.setDeviceLoop(False)  # one graph per iteration: profilers see every kernel launch
    nn, nel = sim.numNodes(), sim.numElements()
    b_host = sim.buildLoadVector()
    # device-resident inputs: SoA (3, nn) is the (nn, 3) column-major VField layout
    b_d = torch.from_numpy(np.ascontiguousarray(b_host.T)).to("cuda")
    rho_d = torch.from_numpy(rho).to("cuda")
    x_d = torch.zeros(3, nn, dtype=torch.float64, device="cuda")
    sptr = C.c_void_p()
    _capi.check(lib.vfem_mg_get_stream(mg._h, C.byref(sptr)))
    stream = torch.cuda.ExternalStream(sptr.value)
    stats = _capi.PcgStats()
    cb = _capi.PCG_CALLBACK()

    def step_device():
        with torch.cuda.stream(stream):
            x_d.zero_()
        _capi.check(lib.vfem_grid_set_densities(sim._h, C.c_void_p(rho_d.data_ptr())))
        _capi.check(lib.vfem_mg_pcg(mg._h, C.c_void_p(x_d.data_ptr()), C.c_void_p(b_d.data_ptr()), 500, TOL, 1, 2,
                                    0, 0, cb, None, C.byref(stats)))
        return stats.iterations, stats.relres

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(fn, k):
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        out = None
        for _ in range(k):
            out = fn()
        e1.record(stream)
        e1.synchronize()
        t1 = time.perf_counter()
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1), ws)
        return ms / 1000.0, (t1 - t0), out

    # ---------------- FP64 (the reference's method) ----------------
    mg.setPrecision("fp64")
    step_device()  # warm-up: hierarchy, graphs
    k64 = max(1, min(args.steps, 2 if args.config == "c2" else args.steps))
    t64, _, (it64, rr64) = timed(step_device, k64)
    t64 /= k64
    x64 = x_d.clone()
    comp64 = 0.5 * float(torch.dot(b_d.flatten(), x64.flatten()))

    # ---------------- mixed precision (headline) ----------------
    mg.setPrecision("mixed", "df")
    for _ in range(args.warmup):
        step_device()
    clocks = ClockSampler(dev)
    clocks.start()
    cnt0 = C.c_uint64()
    _capi.check(lib.vfem_kernel_launch_count(C.byref(cnt0)))
    # NVTX range: lets a profiler restrict its launch list to the timed mixed solves
    torch.cuda.nvtx.range_push("vfem_mixed_solve")
    tmix, wall, (itmix, rrmix) = timed(step_device, args.steps)
    torch.cuda.nvtx.range_pop()
    cnt1 = C.c_uint64()
    _capi.check(lib.vfem_kernel_launch_count(C.byref(cnt1)))
    clk = clocks.stop()
    tmix_step = tmix / args.steps
    xm = x_d.clone()
    compm = 0.5 * float(torch.dot(b_d.flatten(), xm.flatten()))
    # true residual of the mixed solution in FP64
    xm_host = xm.cpu().numpy().T.copy(order="F")
    r = b_host - sim.applyK(xm_host)
    r[sim.getDirichletMask()] = 0
    true_rel = float(np.linalg.norm(r) / np.linalg.norm(b_host))

    # ---------------- the same mixed solve with bf16 smoothing-level stencils ----------------
    _capi.check(lib.vfem_mg_set_stencil_bf16(mg._h, 1))
    for _ in range(2):
        step_device()
    tbf, _, (itbf, rrbf) = timed(step_device, args.steps)
    compbf = 0.5 * float(torch.dot(b_d.flatten(), x_d.flatten()))
    _capi.check(lib.vfem_mg_set_stencil_bf16(mg._h, 0))
    bf16_stencils = {"s_per_solve": tbf / args.steps, "iterations": int(itbf), "relres": rrbf,
                     "compliance_rel_err_vs_fp64": abs(compbf - comp64) / abs(comp64)}
    step_device()  # back to the FP32 stencils before the end-to-end leg

    # ---------------- end to end through the public API, pinned host buffers ----------------
    rho_p = torch.from_numpy(rho).pin_memory()
    b_p = torch.from_numpy(np.ascontiguousarray(b_host.T)).pin_memory()
    # Two pinned iterates: step i solves in x_bufs[i % 2] from its zero initial guess, and once
    # its result has been read the buffer is zeroed again on a host thread during the next step's
    # solve (the library call releases the interpreter lock), ready for step i + 2. The thread
    # waits until that solve's uploads are done (they take about 1 ms of the ~44 ms call) and
    # zeroes with one core, so that it does not compete with them for host memory bandwidth.
    x_bufs = [torch.zeros(3, nn, dtype=torch.float64).pin_memory() for _ in range(2)]
    zeroing = [None, None]
    host_pool = concurrent.futures.ThreadPoolExecutor(max_workers=1)
    step_no = [0]

    e2e_parts = {"wait_zero_x0": 0.0, "set_densities": 0.0, "pcg_call": 0.0, "compliance_dot": 0.0}

    def step_host():
        i = step_no[0]
        x_p = x_bufs[i % 2]
        t = [time.perf_counter()]
        if zeroing[i % 2] is not None:
            zeroing[i % 2].result()
        t.append(time.perf_counter())
        _capi.check(lib.vfem_grid_set_densities(sim._h, C.c_void_p(rho_p.data_ptr())))
        t.append(time.perf_counter())
        _capi.check(lib.vfem_mg_pcg(mg._h, C.c_void_p(x_p.data_ptr()), C.c_void_p(b_p.data_ptr()), 500, TOL, 1, 2,
                                    0, 0, cb, None, C.byref(stats)))
        t.append(time.perf_counter())
        c = 0.5 * float(np.dot(b_p.numpy().ravel(), x_p.numpy().ravel()))
        t.append(time.perf_counter())
        def rezero(buf=x_p.numpy()):
            time.sleep(0.005)
            buf.fill(0.0)

        zeroing[i % 2] = host_pool.submit(rezero)
        step_no[0] = i + 1
        for key, a, b in zip(e2e_parts, t, t[1:]):
            e2e_parts[key] += b - a
        return c

    step_host()
    for key in e2e_parts:
        e2e_parts[key] = 0.0
    _, e2e_wall, _ = timed(step_host, args.steps)
    e2e = e2e_wall / args.steps
    for f in zeroing:
        if f is not None:
            f.result()
    host_pool.shutdown()
    e2e_parts_ms = {k: v / args.steps * 1e3 for k, v in e2e_parts.items()}
    h2d = rho.nbytes + 2 * 3 * nn * 8  # densities, b, x0
    d2h = 3 * nn * 8

    breakdown_mixed = phase_breakdown(lib, _capi, mg._h)
    mg.setPrecision("fp64")
    breakdown_fp64 = phase_breakdown(lib, _capi, mg._h, reps=1)
    mg.setPrecision("mixed", "df")

    # ---------------- hot kernels: device time per launch (CUDA events on the solver stream) ----------------
    hbm, peak_kind = peaks()
    kernels = {}
    outer_kind = mg.outerMatvecKind()
    kids = (1, 2, 0, 3, 5, 6, 7, 8, 9) + ((10,) if outer_kind == "tensor" else ())
    for kid in kids:
        ms = C.c_double()
        nbytes = C.c_double()
        reps = 3 if kid == 0 else 20
        _capi.check(lib.vfem_mg_time_kernel(mg._h, kid, reps, C.byref(ms), C.byref(nbytes)))
        kernels[KERNEL_NAMES[kid]] = {"ms": ms.value, "bytes": nbytes.value,
                                      "gbs": nbytes.value / (ms.value * 1e-3) / 1e9}
    # the other forms of the fine sweep (the solve uses the default one): eight colour launches
    # (one per colour of the reference's order), two plane-pair launches (one cluster per x-plane)
    for mode in ("colours", "planes", "lines", "staged"):
        os.environ["VFEM_GS_MODE"] = mode
        ms, nbytes = C.c_double(), C.c_double()
        _capi.check(lib.vfem_mg_time_kernel(mg._h, 3, 20, C.byref(ms), C.byref(nbytes)))
        kernels["gs_fine_sweep_fp32_" + mode] = {"ms": ms.value, "bytes": nbytes.value,
                                                  "gbs": nbytes.value / (ms.value * 1e-3) / 1e9}
    del os.environ["VFEM_GS_MODE"]
    # the level-1 and level-2 passes with bf16 stencils
    _capi.check(lib.vfem_mg_set_stencil_bf16(mg._h, 1))
    for kid in (6, 7, 8):
        ms, nbytes = C.c_double(), C.c_double()
        _capi.check(lib.vfem_mg_time_kernel(mg._h, kid, 20, C.byref(ms), C.byref(nbytes)))
        kernels[KERNEL_NAMES[kid] + "_bf16_stencil"] = {"ms": ms.value}
    _capi.check(lib.vfem_mg_set_stencil_bf16(mg._h, 0))
    # register budgets of the FP32 fine kernels: fitted to 3 or 4 resident 256-thread blocks per SM
    for occ in ("2", "3", "4"):
        os.environ["VFEM_FINE_OCC"] = occ
        for kid, name in ((3, "gs_fine_sweep_fp32"), (5, "residual_fine_fp32")):
            ms, nbytes = C.c_double(), C.c_double()
            _capi.check(lib.vfem_mg_time_kernel(mg._h, kid, 20, C.byref(ms), C.byref(nbytes)))
            kernels[name + "_occ" + occ] = {"ms": ms.value, "bytes": nbytes.value,
                                            "gbs": nbytes.value / (ms.value * 1e-3) / 1e9}
    del os.environ["VFEM_FINE_OCC"]
    # launches per PCG iteration of the hot kernels of the mixed solve (2 pre + 2 post sweeps per level)
    outer_name = "applyk_fine_tc" if outer_kind == "tensor" else "applyk_fine_df"
    per_iter_launches = {outer_name: 1, "gs_fine_sweep_fp32": 4, "residual_fine_fp32": 1,
                         "gs_level1_sweep_fp32": 4, "residual_level1_fp32": 1, "gs_level2_sweep_fp32": 4,
                         "residual_level2_fp32": 1}
    share = {k: n * kernels[k]["ms"] for k, n in per_iter_launches.items()}
    dom = max(share, key=share.get)
    traffic_tab = {}
    tpath = os.path.join(ROOT, "profiles", "kernel_traffic_%s.json" % args.config)
    if os.path.exists(tpath):
        with open(tpath) as fh:
            traffic_tab = json.load(fh)
    rooflines = {}
    for k in per_iter_launches:
        kd = kernels[k]
        rooflines[k] = {"bound": "hbm", "achieved": kd["gbs"], "peak": hbm, "unit": "GB/s", "frac": kd["gbs"] / hbm,
                        "traffic": traffic_tab.get(k), "algorithmic_bytes": kd["bytes"], "ms_per_launch": kd["ms"],
                        "ms_per_iteration": share[k]}
    p64 = fp64_peak_tflops()
    peaks_measured = {"fp64_tflops": p64, "fp64_how": "cuBLAS DGEMM 4096^3 in this run"}
    for k in ("applyk_fine_df", "applyk_fine_tc"):
        if k not in rooflines:
            continue
        # FP64-class matvecs: their FP64-equivalent arithmetic (2 * 24^2 flops per element)
        # against the measured FP64 rate of this GPU
        flops = 2.0 * 24 * 24 * nel
        achieved = flops / (kernels[k]["ms"] * 1e-3) / 1e12
        rooflines[k]["fp64_equivalent"] = {"flops": flops, "achieved": achieved, "unit": "TFLOP/s", "peak": p64,
                                           "peak_kind": "measured (cuBLAS DGEMM 4096^3 in this run)",
                                           "frac": achieved / p64 if p64 else None}
    if "applyk_fine_tc" in rooflines:
        tflops = tc_mma_flops(ne) / (kernels["applyk_fine_tc"]["ms"] * 1e-3) / 1e12
        bf16 = bf16_peak()
        rooflines["applyk_fine_tc"]["tensor"] = {"mma_flops": tc_mma_flops(ne), "achieved": tflops,
                                                 "unit": "TFLOP/s", "peak": bf16,
                                                 "peak_kind": "measured (MEASURED_PEAKS.json bf16 burst)",
                                                 "frac": tflops / bf16 if bf16 else None}
    # the matrix-free FP32 fine-level kernels are bound by the FP32 pipe: 2 * 24^2 flops per node
    # (the 8 incident element rows of K0 times u) against the FFMA rate of this GPU
    p32 = fp32_peak_tflops()
    peaks_measured.update(fp32_tflops=p32, fp32_how="cuBLAS SGEMM 8192^3 with TF32 off, in this run")
    for k in ("gs_fine_sweep_fp32", "residual_fine_fp32"):
        if k in rooflines:
            flops = 2.0 * 24 * 24 * nn
            achieved = flops / (kernels[k]["ms"] * 1e-3) / 1e12
            rooflines[k]["fp32_compute"] = {"flops": flops, "achieved": achieved, "unit": "TFLOP/s",
                                            "peak": p32,
                                            "peak_kind": "measured (cuBLAS SGEMM 8192^3, TF32 off, in this run)",
                                            "frac": achieved / p32}
    roofline = dict(rooflines[dom], kernel=dom, peak_kind=peak_kind)
    # the tensor-core alternative for the level-1 operator, beside the stored FP32 stencil
    tc_probe = level1_contraction_tc_probe(ne[0] * ne[1] * ne[2] // 8)
    tc_probe["stored_stencil_residual_ms"] = kernels.get("residual_level1_fp32", {}).get("ms")
    tc_probe["stored_stencil_sweep_ms"] = kernels.get("gs_level1_sweep_fp32", {}).get("ms")

    line = {"metric": METRIC, "value": aggregate_per_solve(tmix, ws, args.steps), "unit": "s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmix_step * 1000,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "cantilever %dx%dx%d Q1 (%d DOF), rho U[%g,1] seed 0, %d coarsenings, mixed FP32 "
                                   "V-cycle (2+2 block-GS sweeps) in FP64 CG, %s outer matvec, tol 1e-8"
                                   % (ne[0], ne[1], ne[2], 3 * nn, rho_lo, levels,
                                      "tensor-core (integer-slice bf16)" if outer_kind == "tensor"
                                      else "double-float"),
                       "l2": "no flush: working set of every step (> 2 GB) exceeds the 129 MB L2"},
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "parts_ms": e2e_parts_ms},
            "roofline": roofline,
            "rooflines": rooflines,
            "clocks": clk,
            "peaks_measured": peaks_measured,
            "gpu_launches": int(cnt1.value - cnt0.value),
            "mixed": {"s_per_solve": tmix_step, "iterations": int(itmix), "relres": rrmix, "true_relres": true_rel,
                      "compliance": compm},
            "fp64": {"s_per_solve": t64, "iterations": int(it64), "relres": rr64, "compliance": comp64,
                     "steps": k64},
            "speedup_mixed_vs_fp64": t64 / tmix_step,
            "mixed_bf16_stencils": bf16_stencils,
            "compliance_rel_err_mixed_vs_fp64": abs(compm - comp64) / abs(comp64),
            "applyk_gbs": {"fp32": kernels["applyk_fine_fp32"]["gbs"], "fp64": kernels["applyk_fine_fp64"]["gbs"],
                           "df": kernels["applyk_fine_df"]["gbs"],
                           "tc": kernels.get("applyk_fine_tc", {}).get("gbs")},
            "kernels": kernels,
            "level1_tc_probe": tc_probe,
            "breakdown_ms": {"mixed_per_iteration": breakdown_mixed, "fp64_per_iteration": breakdown_fp64}}
    if rank == 0 and ws == 1 and not args.no_lbl:
        line["lbl"] = run_lbl()
    if rank == 0 and ws == 1 and not args.no_q2:
        line["q2"] = run_q2(hbm)
    if rank == 0 and ws == 1 and not args.no_mma:
        line["mma"] = run_mma(args.no_cpu)
        line["filters"] = run_filters()
    if rank == 0 and ws == 1 and not args.no_2d:
        line["2d"] = run_2d(hbm, args.no_cpu)
    if rank == 0 and ws == 1 and not args.no_cpu:
        cb_line = cpu_baseline_solve(args.config)
        line["cpu_baseline"] = cb_line
        # the CPU solve against both GPU forms: the plain method (FP64) and the headline (mixed)
        line["vs_cpu_baseline"] = {"fp64_gpu_speedup": cb_line["value"] / t64,
                                   "mixed_gpu_speedup": cb_line["value"] / tmix_step,
                                   "mixed_e2e_speedup": cb_line["value"] / e2e,
                                   "cpu_iterations": cb_line["iterations"], "gpu_fp64_iterations": int(it64),
                                   "gpu_mixed_iterations": int(itmix),
                                   "compliance_rel_diff_fp64_gpu_vs_cpu":
                                       abs(comp64 - cb_line["compliance"]) / abs(cb_line["compliance"])}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


LBL_NE = (128, 128, 128)
# 5 coarsenings (coarsest 4^3 elements): every height rebuilds the hierarchy, whose FP64 dense
# inverse of the coarsest level costs 7.0 ms at 4 coarsenings (8^3, ~1,944 free DOFs) and 1.2 ms
# here; the PCG iteration counts are identical (1456 / 1477 / 1776 for N=3 x 1, N=3 x 8, zero).
LBL_COARSENINGS = 5


def run_lbl(slots_list=(1, 8, 16)):
    """Layer-by-layer workload: 128^3 Q1, rho U[0.1, 1] seed 0, base fixed, gravity (0, -1, 0),
    heights 1..128 each solved from a zero guess (mixed precision, tol 1e-8, 2+2 sweeps, 5
    coarsenings). Wall time of the 128 solves one height at a time (1 slot) and spread over
    concurrent solver slots; each evaluator warmed up once (graph capture) before its timed run."""
    import torch

    from voxelfem_gb300 import pyVoxelFEM as pv
    from voxelfem_gb300 import workloads as wl

    ne = LBL_NE
    sim = pv.TensorProductSimulator([1, 1, 1], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    wl.setup_layer_by_layer(sim, ne, 0.1, 0)
    mg = sim.multigridSolver(LBL_COARSENINGS)
    mg.setPrecision("mixed")
    out = {"workload": "layer-by-layer 128^3 Q1, rho U[0.1,1] seed 0, base fixed, gravity -y, heights 1..128, "
                       "zero initial guesses, mixed precision, tol 1e-8, 2+2 sweeps, 5 coarsenings",
           "heights": ne[1]}
    ref = None
    for slots in slots_list:
        ev = pv.LayerByLayerEvaluator(sim)
        ev.selectInitMethod("zero")
        ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=slots)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=slots)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        key = "one_at_a_time_s" if slots == 1 else "slots_%d_s" % slots
        out[key] = dt
        if ref is None:
            ref = ev.compliances.copy()
            out["iterations_total"] = int(ev.iterations.sum())
            out["objective"] = ev.objective()
        else:
            out["max_rel_diff_vs_one_at_a_time_%d" % slots] = float(np.max(np.abs(ev.compliances - ref) / np.abs(ref)))
        ev._release()
    best = min((k for k in out if k.startswith("slots_")), key=lambda k: out[k], default=None)
    if best is not None:
        out["batched_speedup"] = out["one_at_a_time_s"] / out[best]
        out["best"] = best
    # warm starts (the reference's default "N=3" generator): one chain (the reference's
    # sequential algorithm) and 8 concurrent chains of contiguous heights
    for chains in (1, 8):
        ev = pv.LayerByLayerEvaluator(sim)
        ev.selectInitMethod("N=3")
        ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=chains)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=chains)
        torch.cuda.synchronize()
        key = "warm_N3_chains_%d" % chains
        out[key + "_s"] = time.perf_counter() - t0
        out[key + "_iterations_total"] = int(ev.iterations.sum())
        out[key + "_max_rel_diff_vs_zero"] = float(np.max(np.abs(ev.compliances - ref) / np.abs(ref)))
        ev._release()
    # the same warm-started chains at 4 coarsenings (the reference's optMGLevel choice for 128^3)
    mg4 = sim.multigridSolver(4)
    mg4.setPrecision("mixed")
    ev = pv.LayerByLayerEvaluator(sim)
    ev.selectInitMethod("N=3")
    ev.run(mg4, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=8)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev.run(mg4, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=8)
    torch.cuda.synchronize()
    out["warm_N3_chains_8_4_coarsenings_s"] = time.perf_counter() - t0
    out["warm_N3_chains_8_4_coarsenings_iterations_total"] = int(ev.iterations.sum())
    ev._release()
    del mg4
    # where one height's solve spends its time: a mixed solve from zero at a few heights (CUDA
    # events around the library call) and the warm-cache per-phase breakdown of one iteration
    import ctypes as C

    from voxelfem_gb300 import _capi
    lib = _capi.load()
    per_height = {}
    for h in (8, 32, 64, 128):
        mg.setFabricationMaskHeightByLayer(h)
        f = sim.buildLoadVector()
        x0 = np.zeros_like(f)
        mg.preconditionedConjugateGradient(x0, f, 500, TOL, None, 1, 2, False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mg.preconditionedConjugateGradient(x0, f, 500, TOL, None, 1, 2, False)
        dt = time.perf_counter() - t0
        bd = phase_breakdown(lib, _capi, mg._h, reps=2)
        iter_ms = sum(v for k, v in bd.items() if not k.startswith(("galerkin", "coarsest:")) or k == "coarsest:solve")
        top = sorted(((v, k) for k, v in bd.items() if not k.startswith("galerkin")), reverse=True)[:8]
        per_height[str(h)] = {"solve_s_host_buffers": dt, "iterations": int(mg.lastStats.iterations),
                              "iteration_ms": iter_ms, "rebuild_ms": bd.get("galerkin+coarse_inverse"),
                              "top_phases_ms": {k: v for v, k in top}}
    mg.setFabricationMaskHeightByLayer(ne[1])
    out["per_height_mixed"] = per_height
    # the autotuner (slots x fine-sweep form x smoothing sweeps, on every 8th height), then all
    # 128 heights with its choice
    import tempfile

    from voxelfem_gb300 import autotune
    with tempfile.TemporaryDirectory() as tdir:
        entry = autotune.tune_layer_by_layer(sim, mg, "zero", tol=TOL, path=os.path.join(tdir, "cache.json"))
    out["autotune"] = {"key": autotune.key(sim, mg, "zero"), "entry": entry}
    ev = pv.LayerByLayerEvaluator(sim)
    ev.selectInitMethod("zero")
    kw = dict(maxIter=500, tol=TOL, mgIterations=1, mgSmoothingIterations=entry["mgSmoothingIterations"],
              slots=entry["slots"], sweepForm=entry["sweepForm"])
    ev.run(mg, True, 1, **kw)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev.run(mg, True, 1, **kw)
    torch.cuda.synchronize()
    out["tuned_zero_s"] = time.perf_counter() - t0
    out["tuned_zero_iterations_total"] = int(ev.iterations.sum())
    out["tuned_zero_max_rel_diff_vs_2_sweeps"] = float(np.max(np.abs(ev.compliances - ref) / np.abs(ref)))
    ev._release()
    # the plain method: 128 sequential FP64 solves on the same GPU
    mg.setPrecision("fp64")
    ev = pv.LayerByLayerEvaluator(sim)
    ev.selectInitMethod("zero")
    ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=1)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev.run(mg, True, 1, 500, TOL, mgIterations=1, mgSmoothingIterations=2, slots=1)
    torch.cuda.synchronize()
    out["sequential_fp64_s"] = time.perf_counter() - t0
    out["sequential_fp64_iterations_total"] = int(ev.iterations.sum())
    out["max_rel_diff_fp64_vs_mixed"] = float(np.max(np.abs(ev.compliances - ref) / np.abs(ref)))
    ev._release()
    fastest = min((k for k in out if k.endswith("_s") and (k.startswith("slots_") or k.startswith("warm_"))
                   and "4_coarsenings" not in k),
                  key=lambda k: out[k], default=None)
    if fastest is not None:
        out["fastest"] = fastest
        out["speedup_vs_sequential_fp64"] = out["sequential_fp64_s"] / out[fastest]
    return out


Q2_COARSENINGS = 5   # 128^3 -> 4^3 Q2 elements at the coarsest level (1,944 free DOFs)
Q2_SWEEPS = 1
Q2_NE = (128, 128, 128)


MMA_N = 192 * 96 * 96  # the 192x96x96 MBB design's element count


def run_filters():
    """The density filter at the MBB size (192x96x96 elements, radius 2, linear weights) on device
    arrays: the allocating entry point and the allocation-free one (which rebuilds its tap table
    every call), CUDA events over 20 calls each."""
    import ctypes as C

    import torch

    from voxelfem_gb300 import _capi
    lib = _capi.load()
    dims = (192, 96, 96)
    dims_c = (C.c_int64 * 3)(*dims)
    n = dims[0] * dims[1] * dims[2]
    x = torch.rand(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    out = {"workload": "smoothing filter 192x96x96, radius 2, linear (93 taps)", "bytes": 2 * 8 * n}

    def time_calls(fn, reps=20):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    out["allocating_ms"] = time_calls(lambda: _capi.check(lib.vfem_smoothing_filter(
        dims_c, 2, 1, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))))
    out["noalloc_ms"] = time_calls(lambda: _capi.check(lib.vfem_smoothing_filter_noalloc(
        dims_c, 2, 1, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(stream.cuda_stream))))
    return out


def run_mma(no_cpu):
    """One MMA step (and one GCMMA step) on 1,769,472 variables with one volume-type constraint:
    a box-constrained quadratic objective, x0 = 0.5, callbacks evaluated in numpy on the host
    (the reference's interface). Wall time per step from the second step on; the CPU leg runs
    the oracle's numpy restatement of the same algorithm on one step."""
    from voxelfem_gb300 import pyOptimizer

    n = MMA_N
    t = np.random.default_rng(0).uniform(0.1, 0.9, n)
    calls = {"f": 0, "df": 0}

    def f(x):
        calls["f"] += 1
        return np.array([np.sum((x - t) ** 2), np.mean(x) / 0.3 - 1.0])

    def df(x):
        calls["df"] += 1
        return np.vstack([2 * (x - t), np.full(n, 1.0 / (0.3 * n))])

    out = {"workload": "MMA, n = %d, m = 1, quadratic objective, host callbacks" % n}
    for name, gc in (("mma", False), ("gcmma", True)):
        g = pyOptimizer.MMA(n, 1, np.zeros(n), np.ones(n), f, df)
        g.enableGCMMA(gc)
        g.setInitialVar(np.full(n, 0.5))
        g.step()
        t0 = time.perf_counter()
        steps = 3
        for _ in range(steps):
            g.step()
        out[name + "_s_per_step"] = (time.perf_counter() - t0) / steps
        out[name + "_objective"] = float(f(g.getOptimalVar())[0])
    if not no_cpu:
        from oracle import mma as omma
        o = omma.MMA(n, 1, np.zeros(n), np.ones(n), f, df)
        o.setInitialVar(np.full(n, 0.5))
        o.step()
        t0 = time.perf_counter()
        o.step()
        out["cpu_oracle_numpy_s_per_step"] = time.perf_counter() - t0
    return out


def run_q2(hbm, solve=True):
    """Triquadratic applyK at 128^3 Q2 elements (16.97M nodes, 50.9M DOF), rho U[0.01, 1] seed 0:
    device time per launch on resident data (FP64 and FP32), algorithmic bytes s (6 nn + ne) and
    FLOPs 2 * 81^2 * ne."""
    import ctypes as C

    from voxelfem_gb300 import _capi
    from voxelfem_gb300 import pyVoxelFEM as pv

    lib = _capi.load()
    ne = Q2_NE
    g = pv.TensorProductSimulator([2, 2, 2], [[0.0, 0.0, 0.0], [float(v) for v in ne]], ne)
    g.ETensor = (1.0, 0.3)
    g.E_0, g.E_min, g.gamma = 1.0, 1e-9, 3.0
    rho = np.random.default_rng(0).uniform(0.01, 1.0, int(np.prod(ne)))
    g.setDensities(rho)
    flops = 2.0 * 81 * 81 * g.numElements()
    out = {"workload": "128^3 Q2 applyK (%d nodes), rho U[0.01,1] seed 0" % g.numNodes()}
    for name, prec, reps in (("fp64", 0, 2), ("df", 2, 3), ("fp32", 1, 10)):
        ms, nbytes = C.c_double(), C.c_double()
        _capi.check(lib.vfem_q2_time_apply_k(g._h, prec, reps, C.byref(ms), C.byref(nbytes)))
        gbs = nbytes.value / (ms.value * 1e-3) / 1e9
        out[name] = {"ms": ms.value, "bytes": nbytes.value, "gbs": gbs, "hbm_frac": gbs / hbm,
                     "tflops": flops / (ms.value * 1e-3) / 1e12}
    for name, prec, reps in (("smoother_fp32", 1, 3), ("smoother_fp64", 0, 1)):
        ms, nbytes = C.c_double(), C.c_double()
        _capi.check(lib.vfem_q2_time_smooth(g._h, prec, reps, C.byref(ms), C.byref(nbytes)))
        gbs = nbytes.value / (ms.value * 1e-3) / 1e9
        out[name] = {"ms": ms.value, "bytes": nbytes.value, "gbs": gbs, "hbm_frac": gbs / hbm}
    if solve:
        out["solve"] = run_q2_solve(g, ne, rho)
    return out


def run_q2_solve(g, ne, rho):
    """Time to relative residual 1e-8 of the 128^3 Q2 cantilever (x = 0 face fixed, unit total -y
    load spread over the nodes of the x = max, z = mid edge), FP64 CG, 5 coarsenings:
    - mixed (the headline): Q2 sweeps around an FP32 trilinear V-cycle on the same mesh
      (p-multigrid), double-float CG matvec;
    - reference_hierarchy_mixed: the reference's hierarchy of halved Q2 meshes (the library's
      default preconditioner) with an FP32 V-cycle, double-float CG matvec;
    - fp64_plain: the reference's method, FP64 V-cycle and FP64 matvec on that hierarchy.
    Accuracy against FP64:
    - the true FP64 residual |f - K u| / |f| of the mixed u, with K applied by the library's FP64
      kernel and, independently, by the CPU oracle's triquadratic applyK (the reference's generic
      stencil restated, with its own K0 quadrature);
    - the error of u and of the compliance against an FP64 solve of the same system (FP64 matvec)
      to relative residual 1e-11."""
    import time

    import torch

    nx, ny, nz = ne
    g.addDirichletCondition([0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, float(ny), float(nz)], "xyz")
    nnd = [2 * v + 1 for v in ne]
    nn = g.numNodes()
    f = np.zeros((nn, 3), order="F")
    idx = np.arange(nn).reshape(nnd)
    line = idx[nnd[0] - 1, :, nz].ravel()
    f[line, 1] = -1.0 / line.size
    mg = g.multigridSolver(Q2_COARSENINGS)
    x0 = np.zeros((nn, 3), order="F")

    def solve(hierarchy, precision, sweeps, tol=1e-8, maxIter=500):
        mg.setHierarchy(hierarchy)
        mg.setPrecision(precision)
        mg.preconditionedConjugateGradient(x0, f, 1, tol, None, 1, sweeps, False)  # hierarchy, buffers
        torch.cuda.nvtx.range_push("vfem_q2_solve_%s_%s" % (hierarchy, precision))
        t0 = time.perf_counter()
        u = mg.preconditionedConjugateGradient(x0, f, maxIter, tol, None, 1, sweeps, False)
        seconds = time.perf_counter() - t0
        torch.cuda.nvtx.range_pop()
        st = mg.lastStats
        return u, {"seconds": seconds, "iterations": int(st.iterations), "relres": float(st.relres),
                   "hierarchy": hierarchy, "precision": precision, "sweeps": sweeps,
                   "compliance": float(np.sum(f * u))}

    # headline: the faster preconditioner for this workload (p-multigrid onto the trilinear mesh);
    # the reference's hierarchy of halved Q2 meshes (the library's default) is timed beside it
    u, out = solve("p", "mixed", Q2_SWEEPS)
    out["seconds_to_1e-8"] = out.pop("seconds")
    out["dofs"] = 3 * nn
    out["note"] = ("host buffers in and out; includes the h2d of f and x0 and the d2h of u; the hierarchy "
                   "is built in the untimed warm-up call")
    dmask = g.getDirichletMask()
    r = f - g.applyK(u, zeroDirichlet=True)
    r[dmask] = 0.0
    out["true_relres_fp64"] = float(np.linalg.norm(r) / np.linalg.norm(f))
    _, out["reference_hierarchy_mixed"] = solve("q2", "mixed", Q2_SWEEPS)
    _, out["fp64_plain"] = solve("q2", "fp64", Q2_SWEEPS)
    # the FP64 reference solve of the same system: FP64 CG matvec to 1e-11
    mg.setHierarchy("q2")
    mg.setPrecision("mixed")
    mg.setOuterMatvec("fp64")
    t0 = time.perf_counter()
    u64 = mg.preconditionedConjugateGradient(x0, f, 1000, 1e-11, None, 1, Q2_SWEEPS, False)
    out["fp64_reference"] = {"tol": 1e-11, "iterations": int(mg.lastStats.iterations),
                             "relres": float(mg.lastStats.relres), "seconds": time.perf_counter() - t0,
                             "u_rel_err_mixed": float(np.linalg.norm(u - u64) / np.linalg.norm(u64)),
                             "u_max_rel_err_mixed": float(np.max(np.abs(u - u64)) / np.max(np.abs(u64))),
                             "compliance_rel_err_mixed": float(abs(np.sum(f * u) - np.sum(f * u64))
                                                               / abs(np.sum(f * u64)))}
    mg.setOuterMatvec("df")
    try:
        from oracle import pyoracle as po
        K0 = po.q2_k0(1.0, 0.3, (1.0, 1.0, 1.0), 3)
        Y = 1e-9 + rho ** 3 * (1.0 - 1e-9)
        t0 = time.perf_counter()
        ro = f - po.q2_apply_k(ne, K0, Y, u)
        ro[dmask] = 0.0
        out["oracle_relres_fp64"] = float(np.linalg.norm(ro) / np.linalg.norm(f))
        out["oracle_apply_seconds"] = time.perf_counter() - t0
    except Exception as e:  # the oracle library is not built: report why
        out["oracle_relres_fp64"] = None
        out["oracle_error"] = str(e)[:200]
    return out


D2_DEMO = (384, 192)      # the reference's 2D topology-optimisation demo resolution
D2_DEMO_LEVELS = 4        # its optMGLevel([384, 192], 2)
D2_LARGE = (4096, 2048)   # 8.4M nodes: operator traffic well above L2
D2_LARGE_LEVELS = 7       # optMGLevel([4096, 2048], 2): coarsest 32 x 16


def setup_2d(ne, rho=None):
    """2D cantilever on [0, 2] x [0, 1] (B9Creator material: E 1, nu 0.3): x = 0 edge fixed, unit
    -y load at the (x = 2, y = 0) corner (the reference's cantilever_flexion_SE regions)."""
    from voxelfem_gb300 import pyVoxelFEM as pv

    tps = pv.TensorProductSimulator([1, 1], [[0.0, 0.0], [2.0, 1.0]], list(ne))
    tps.ETensor = (1.0, 0.3)
    tps.addDirichletCondition([0.0, 0.0], [-2e-4, -1e-4], [2e-4, 1.0001], "xy")
    f = np.zeros((tps.numNodes(), 2), order="F")
    f[ne[0] * (ne[1] + 1), 1] = -1.0
    tps.setNodalForces(f)
    if rho is not None:
        tps.setDensities(rho)
    return tps, f


def run_2d(hbm, no_cpu):
    """The bilinear-quadrilateral path. Demo case (384 x 192, 4 coarsenings, the demo's filters
    SmoothingFilter(3, Linear) + ProjectionFilter(1), volume 0.33): wall time of setVars (filters +
    MG-PCG to 1e-5 with the objective's defaults: FMG, 2 sweeps) and of one OC step, host arrays
    in and out; a FP64 PCG solve to 1e-8 with the numpy oracle timed beside it on the same problem.
    Large case (4096 x 2048, 7 coarsenings): device time per launch of the fine operator, the
    4-colour Gauss-Seidel sweep, one V-cycle and one PCG iteration on resident data, and a solve
    to 1e-8."""
    import time

    from voxelfem_gb300 import pyVoxelFEM as pv

    out = {}
    tps, f = setup_2d(D2_DEMO)
    sf = pv.SmoothingFilter(3, pv.SmoothingFilter.Type.Linear)
    pf = pv.ProjectionFilter(1.0)
    obj = pv.MultigridComplianceObjective(tps.multigridSolver(D2_DEMO_LEVELS))
    top = pv.TopologyOptimizationProblem(tps, obj, [pv.TotalVolumeConstraint(0.33)], [sf, pf])
    x0 = np.full(top.numVars(), pf.invert(0.33))
    top.setVars(x0)  # graph capture, stiffness
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        top.setVars(x0)
        ts.append(time.perf_counter() - t0)
    oc = pv.OCOptimizer(top)
    oc.step()
    to = []
    for _ in range(3):
        t0 = time.perf_counter()
        oc.step()
        to.append(time.perf_counter() - t0)
    demo = {"workload": "2D cantilever 384x192, 4 coarsenings, filters Smoothing(3, Linear) + Projection(1), "
                        "volume 0.33 (the reference's 2D topology-optimisation demo setup)",
            "set_vars_s": float(np.median(ts)), "oc_step_s": float(np.median(to)),
            "pcg_iterations": int(top.lastSolveStats().iterations), "compliance": top.evaluateObjective()}
    # plain FP64 PCG to 1e-8 (1 V-cycle, 1 sweep) on uniform rho 0.5, and the oracle on the same problem
    tps2, f2 = setup_2d(D2_DEMO, np.full(D2_DEMO[0] * D2_DEMO[1], 0.5))
    mg = tps2.multigridSolver(D2_DEMO_LEVELS)
    x = np.zeros_like(f2)
    mg.preconditionedConjugateGradient(x, f2, 2, 1e-8, None, 1, 1, False)
    t0 = time.perf_counter()
    u = mg.preconditionedConjugateGradient(x, f2, 200, 1e-8, None, 1, 1, False)
    demo["pcg_1e-8_s"] = time.perf_counter() - t0
    demo["pcg_1e-8_iterations"] = int(mg.lastStats.iterations)
    if not no_cpu:
        sys.path.insert(0, ROOT)
        from oracle import oracle2d as o2
        sim = o2.Sim2(D2_DEMO, (0.0, 0.0), (2.0, 1.0))
        sim.setMaterial(1.0, 0.3)
        sim.setDensities(np.full(sim.NE, 0.5))
        sim.addDirichletCondition([0.0, 0.0], [-2e-4, -1e-4], [2e-4, 1.0001])
        sim.force = np.asarray(f2).T.ravel().copy()
        omg = o2.MG2(sim, D2_DEMO_LEVELS)
        t0 = time.perf_counter()
        uo = omg.pcg(np.zeros(2 * sim.NN), sim.buildLoadVector(), 200, 1e-8, 1, 1, False)
        cpu_s = time.perf_counter() - t0
        demo["cpu_baseline"] = {"value": cpu_s, "unit": "s", "cores": 1, "kind": "port",
                                "sample": "numpy restatement (oracle/oracle2d.py), same solve",
                                "iterations": int(omg.lastIterations),
                                "solution_rel_diff": float(np.max(np.abs(np.asarray(u).T.ravel() - uo)) /
                                                           np.max(np.abs(uo)))}
    out["demo"] = demo
    # large case: kernels on resident data and a solve
    ne = D2_LARGE
    rho = np.random.default_rng(0).uniform(0.1, 1.0, ne[0] * ne[1])
    tpsL, fL = setup_2d(ne, rho)
    mgL = tpsL.multigridSolver(D2_LARGE_LEVELS)
    nn, nel = tpsL.numNodes(), tpsL.numElements()
    xL = np.zeros_like(fL)
    mgL.preconditionedConjugateGradient(xL, fL, 2, 1e-8, None, 1, 1, False)
    t0 = time.perf_counter()
    uL = mgL.preconditionedConjugateGradient(xL, fL, 500, 1e-8, None, 1, 1, False)
    large = {"workload": "2D cantilever 4096x2048 (%d nodes), rho U[0.1,1] seed 0, 7 coarsenings" % nn,
             "pcg_1e-8_s": time.perf_counter() - t0, "pcg_1e-8_iterations": int(mgL.lastStats.iterations),
             "relres": float(mgL.lastStats.relres)}
    # algorithmic bytes: operator u (16 B/node) in, K u (16 B/node) out, moduli (8 B/element); a
    # sweep's minimum adds b in and u out once (16 + 16 B/node) and the 1 B/node Dirichlet mask
    alg = {"applyk_fine": 32.0 * nn + 8.0 * nel, "gs_sweep_fine": 49.0 * nn + 8.0 * nel}
    # FP64 work per node: 4 incident elements x 2 rows x (8 FMA + scale + add) = 144 flop; the
    # sweep adds the 2 x 2 diagonal block (8 flop) and the block solve (about 10 flop)
    flops = {"applyk_fine": 144.0 * nn, "gs_sweep_fine": 162.0 * nn}
    fp64_peak = fp64_peak_tflops()
    for name, which, reps in (("applyk_fine", 0, 20), ("gs_sweep_fine", 1, 10), ("vcycle", 2, 5), ("pcg_iteration", 3, 5)):
        ms = mgL.timeKernel(which, reps)
        ent = {"ms": ms}
        if name in alg:
            gbs = alg[name] / (ms * 1e-3) / 1e9
            tf = flops[name] / (ms * 1e-3) / 1e12
            ent.update({"bytes": alg[name], "gbs": gbs, "hbm_frac": gbs / hbm,
                        "fp64_compute": {"flops": flops[name], "achieved": tf, "unit": "TFLOP/s",
                                         "peak": fp64_peak, "frac": tf / fp64_peak,
                                         "peak_kind": "measured (cuBLAS DGEMM 4096^3 in this run)"},
                        "bound": "fp64"})
        large[name] = ent
    # the same solve and the preconditioner's kernels with the V-cycle in FP32 (mixed)
    mgL.setPrecision("mixed")
    mgL.preconditionedConjugateGradient(xL, fL, 2, 1e-8, None, 1, 1, False)
    t0 = time.perf_counter()
    uM = mgL.preconditionedConjugateGradient(xL, fL, 500, 1e-8, None, 1, 1, False)
    mixed = {"pcg_1e-8_s": time.perf_counter() - t0, "pcg_1e-8_iterations": int(mgL.lastStats.iterations),
             "relres": float(mgL.lastStats.relres),
             "compliance_rel_diff_vs_fp64": float(abs(np.sum(fL * uM) - np.sum(fL * uL)) / abs(np.sum(fL * uL)))}
    for name, which, reps in (("gs_sweep_fine_fp32", 1, 20), ("vcycle_fp32", 2, 10), ("pcg_iteration", 3, 10),
                              ("applyk_fine_df", 4, 20)):
        mixed[name] = {"ms": mgL.timeKernel(which, reps)}
    ms = mixed["applyk_fine_df"]["ms"]
    mixed["applyk_fine_df"].update({"bytes": alg["applyk_fine"], "gbs": alg["applyk_fine"] / (ms * 1e-3) / 1e9,
                                    "hbm_frac": alg["applyk_fine"] / (ms * 1e-3) / 1e9 / hbm,
                                    "fp64_equivalent_tflops": flops["applyk_fine"] / (ms * 1e-3) / 1e12})
    gbs = 0.5 * alg["gs_sweep_fine"] / (mixed["gs_sweep_fine_fp32"]["ms"] * 1e-3) / 1e9
    mixed["gs_sweep_fine_fp32"].update({"bytes": 0.5 * alg["gs_sweep_fine"], "gbs": gbs, "hbm_frac": gbs / hbm})
    large["mixed"] = mixed
    out["large"] = large
    return out


def run_kernel_case(args):
    """One hot kernel of the workload, launched a handful of times (profiler captures)."""
    import ctypes as C

    import torch

    torch.cuda.set_device(0)
    from voxelfem_gb300 import _capi
    from voxelfem_gb300 import pyVoxelFEM as pv
    from voxelfem_gb300 import workloads as wl

    lib = _capi.load()
    ne, rho_lo, levels = CONFIGS[args.config]
    bbox = [[0.0, 0.0, 0.0], [float(v) for v in ne]]
    sim = pv.TensorProductSimulator([1, 1, 1], bbox, ne)
    wl.setup_cantilever(sim, ne, rho_lo, 0)
    mg = sim.multigridSolver(levels)
    mg.setPrecision("mixed", "df")
    ms, nbytes = C.c_double(), C.c_double()
    _capi.check(lib.vfem_mg_time_kernel(mg._h, args.kernel_case, 1, C.byref(ms), C.byref(nbytes)))
    print(json.dumps({"kernel": KERNEL_NAMES[args.kernel_case], "ms": ms.value, "bytes": nbytes.value}))


def run_kernel_2d(args):
    """The 2D large case's hot kernel `args.kernel_2d` (0 applyK, 1 GS sweep), launched a few times
    (profiler captures)."""
    import torch

    torch.cuda.set_device(0)
    ne = D2_LARGE
    tps, _ = setup_2d(ne, np.random.default_rng(0).uniform(0.1, 1.0, ne[0] * ne[1]))
    mg = tps.multigridSolver(D2_LARGE_LEVELS)
    ms = mg.timeKernel(args.kernel_2d, 1)
    print(json.dumps({"kernel_2d": args.kernel_2d, "ms": ms}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-lbl", action="store_true", help="skip the layer-by-layer batching measurement")
    ap.add_argument("--no-q2", action="store_true", help="skip the triquadratic applyK measurement")
    ap.add_argument("--no-mma", action="store_true", help="skip the MMA optimiser measurement")
    ap.add_argument("--no-2d", action="store_true", help="skip the bilinear-quadrilateral (2D) measurement")
    ap.add_argument("--host-loop", action="store_true",
                    help="iterate PCG from the host (one graph per iteration) instead of the device-resident loop")
    ap.add_argument("--kernel-2d", type=int, default=None,
                    help="only set up the 2D large case and launch one of its kernels (0 applyK, 1 GS sweep)")
    ap.add_argument("--kernel-case", type=int, default=None,
                    help="only set up the workload and launch one hot kernel (id of vfem_mg_time_kernel) twice")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.kernel_case is not None:
        run_kernel_case(args)
    elif args.kernel_2d is not None:
        run_kernel_2d(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
