"""Benchmark: DOF-stage updates/s of the RKDG hot path on one GB300.

Workload (one GPU): the 3D periodic acoustic pulse on a 64^3 hexahedral mesh,
DG Q2 (27 nodes x 5 variables per element, N = 35,389,440 unknowns), Rusanov
flux, no limiter, SSP-RK3 with dt fixed from CFL 0.2 at t = 0.  One bench
"step" is one Runge-Kutta step (3 stages) over the whole mesh; the metric is
N x stages / second.  Inputs are larger than L2 (the FP64 state alone is
283 MB), so no L2 flush is needed between steps.

Arms:
  default            this implementation: FP32-bulk path (value) next to the
                     plain FP64 path, error of the former against the latter,
                     roofline of the stage kernel, end-to-end number through
                     the C ABI with host buffers, and the CPU oracle timed on
                     the host cores (cpu_baseline).
  --impl reference   the reference's CPU algorithm (the FP64 oracle, all
                     host threads) on the same workload, bounded sample.

Multi-GPU (torchrun, N > 1): replicas only — every rank solves its own copy,
no collective on the data path; value = total units / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-stage updates/s, mixed vs plain FP64 on 1 GB300 at <=1e-6 rel L1 err"
UNIT = "DOF-stage updates/s"
STAGES = 3


def workload_config(case, n_elem_side):
    return {
        "workload": f"periodic acoustic pulse {n_elem_side}^3 hex Q2 (27 nodes x 5 vars), Rusanov, "
                    "no limiter, SSP-RK3, dt fixed from CFL 0.2",
        "elements": case.mesh.num_elements,
        "unknowns": None,
        "stages_per_step": STAGES,
        "l2_policy": "inputs larger than L2 (FP64 state 283 MB > 129 MB L2); no flush",
    }


# DRAM bytes (read + write) per element and stage launch of the C2 stage
# kernel k_rhs_hex_tile<2,float>: mean of the three stage launches of one RK
# step captured with ncu on the 64^3 pulse itself (840.2 MB / 262,144
# elements); traffic scales with the element count.
TRAFFIC_BYTES_PER_ELEMENT_LAUNCH = 3205.0


def algorithmic_bytes_per_step(N, ne, precision):
    """Bytes one SSP-RK3 step must move at stored widths:
    FP32-bulk: stage 0 reads x_hi, x_lo, writes k0, y1 (16N); stage 1 reads
    y1, x_hi, x_lo, k0, writes k1, y2 (24N); stage 2 reads y2, k0, k1, x_hi,
    x_lo, writes x_hi, x_lo (28N).  FP64: stage 0 reads x, writes k0, y1
    (24N); stage 1 reads y1, x, k0, writes k1, y2 (40N); stage 2 reads y2, x,
    k0, k1, writes x (40N).  Plus per stage the element and face tables."""
    if precision == "fp32":
        state = 68 * N
        tables = ne * (10 * 4 + 6 * (4 * 4 + 4 + 4))
    else:
        state = 104 * N
        tables = ne * (10 * 8 + 6 * (4 * 8 + 4 + 4))
    return state + STAGES * tables


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        # the per-sample log goes to RKDG_CLOCKS_DIR (default: the system temp folder)
        self.path = os.path.join(os.environ.get("RKDG_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax.append(float(parts[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl != "reference" else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier_max(val, world):
    if world == 1:
        return val
    import torch
    import torch.distributed as dist
    t = torch.tensor([val], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _peak_hbm():
    """Measured HBM bandwidth of the GB300s (MEASURED_PEAKS.json),
    else the fallback figure; (GB/s, source)."""
    try:
        v = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
        if v:
            return float(v), "measured"
    except Exception:
        pass
    return 6800.0, "fallback"


def oracle_rate(case, x0, dt, steps, threads):
    """Reference CPU algorithm (FP64 oracle) on the full mesh for `steps`
    Runge-Kutta steps; returns (rate, seconds)."""
    from oracle import refcpu
    refcpu.set_threads(threads)
    orc = refcpu.Oracle(case.mesh, case.order)
    from rkdg3d_gb300 import cases
    cases.configure_oracle(case, orc)
    x = x0.copy()
    t0 = time.perf_counter()
    x, _ = orc.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=steps)
    sec = time.perf_counter() - t0
    return orc.n * STAGES * steps / sec, sec


def run_reference(args, rank, world):
    if rank != 0:
        return
    from rkdg3d_gb300 import cases
    case = cases.pulse3d(n=args.n, order=2, steps=args.steps, cfl=0.2)
    from oracle import refcpu
    orc = refcpu.Oracle(case.mesh, case.order)
    cases.configure_oracle(case, orc)
    x0 = cases.project(case, orc.node_coords())
    dt = 0.2 * orc.hmin() / orc.face_speed(x0) / 5.0
    threads = os.cpu_count() or 1
    # bounded sample: a one-step probe sizes the timed sample to ~60 s
    _, probe = oracle_rate(case, x0, dt, 1, threads)
    for _ in range(max(0, min(args.warmup, 1) - 1)):
        oracle_rate(case, x0, dt, 1, threads)
    ksteps = int(max(1, min(args.steps, 60.0 // max(probe, 1e-3))))
    rate, sec = oracle_rate(case, x0, dt, ksteps, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / ksteps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": dict(workload_config(case, args.n), unknowns=orc.n),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{ksteps} full RK steps of the {args.n}^3 mesh (FP64 oracle, "
                                   f"restatement of the reference CPU path; reference not buildable)"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import torch
    from rkdg3d_gb300 import cases
    from rkdg3d_gb300.solver import FP32_BULK, FP64, Context

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    case = cases.pulse3d(n=args.n, order=2, steps=args.steps, cfl=0.2)
    stream = torch.cuda.current_stream(dev)

    def make(prec):
        ctx = Context(case.mesh, case.order, device=local, precision=prec)
        cases.configure_context(case, ctx)
        ctx.set_stream(stream.cuda_stream)
        if args.hex_kernel and prec == FP32_BULK:
            from rkdg3d_gb300.solver import TUNE_HEX_KERNEL
            ctx.set_tuning(TUNE_HEX_KERNEL, args.hex_kernel)
        return ctx

    ctx32 = make(FP32_BULK)
    X = ctx32.node_coords()
    x0 = cases.project(case, X)
    N = ctx32.n
    x0d = torch.tensor(x0, dtype=torch.float64, device=dev)
    mcs = ctx32.face_speed(x0d)
    dt = case.cfl * ctx32.hmin() / mcs / (2 * case.order + 1)

    def timed_run(ctx, steps, warm):
        assert steps > 0
        x = x0d.clone()
        if warm > 0:
            ctx.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=warm)
        torch.cuda.synchronize(dev)
        x = x0d.clone()
        l0 = ctx.launches()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=steps)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return x, e0.elapsed_time(e1) / 1e3, ctx.launches() - l0

    # FP32-bulk (the headline) with clocks sampled during the timed region
    with ClockSampler(local) as clk:
        x32, sec32, launches = timed_run(ctx32, args.steps, args.warmup)
    clocks = clk.summary()
    sec32 = barrier_max(sec32, world)
    value = world * N * STAGES * args.steps / sec32

    # plain FP64 path on a shorter window (it runs at the FP64 issue rate)
    ctx64 = make(FP64)
    k64 = max(1, min(args.steps, args.fp64_steps))
    x64, sec64, _ = timed_run(ctx64, k64, min(args.warmup, 3))
    value64 = world * N * STAGES * k64 / barrier_max(sec64, world)
    # error of the FP32-bulk path against the FP64 path after the same steps
    x32b, _, _ = timed_run(ctx32, k64, 0)
    a = x32b.cpu().numpy()
    b = x64.cpu().numpy()
    nd = ctx32.ndofs
    rho_a, rho_b = a[:nd], b[:nd]
    E_a, E_b = a[-nd:], b[-nd:]
    err = {
        "steps_compared": k64,
        "rho_rel_l1": float(np.abs(rho_a - rho_b).sum() / np.abs(rho_b).sum()),
        "rho_linf": float(np.abs(rho_a - rho_b).max()),
        "E_rel_l1": float(np.abs(E_a - E_b).sum() / np.abs(E_b).sum()),
        "E_linf": float(np.abs(E_a - E_b).max()),
    }
    del ctx64

    # end to end through the C ABI with host buffers: every step uploads the
    # state from pinned host memory, runs one rkdg_step (ExplicitRKLimitedSolver
    # ::Step) and reads the state back, as a drop-in Step() on host vectors does
    xh = torch.tensor(x0, dtype=torch.float64).pin_memory()
    xd = torch.empty(N, dtype=torch.float64, device=dev)
    for _ in range(min(args.warmup, 3)):
        xd.copy_(xh, non_blocking=True)
        ctx32.step(xd, dt)
        xh.copy_(xd, non_blocking=True)
    xh.copy_(torch.from_numpy(x0))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        xd.copy_(xh, non_blocking=True)
        ctx32.step(xd, dt)
        xh.copy_(xd, non_blocking=True)
    torch.cuda.synchronize(dev)
    sec_e2e = barrier_max(time.perf_counter() - t0, world)
    e2e = {"value": world * N * STAGES * args.steps / sec_e2e, "unit": UNIT,
           "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N,
           "note": "per step: pinned host -> device copy of the FP64 state, rkdg_step through "
                   "the ctypes C ABI, device -> pinned host copy of the state"}

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    bps = algorithmic_bytes_per_step(N, ctx32.ne, "fp32")
    ms_step = 1e3 * sec32 / args.steps
    achieved = bps / (ms_step / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": args.traffic_per_launch or TRAFFIC_BYTES_PER_ELEMENT_LAUNCH * ctx32.ne,
            "traffic_source": "ncu dram bytes per launch, 64^3 capture (per element, scaled by elements)"
                              if not args.traffic_per_launch else "command line",
            "peak_source": peak_src,
            "kernel": ("k_rhs_hex_tile<2,float> (face-once tiled stage kernel, 3 launches per step)"
                       if args.hex_kernel in (0, 5) else f"hexahedral kernel variant {args.hex_kernel}"),
            "algorithmic_bytes_per_launch": bps / STAGES}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        try:
            _, probe = oracle_rate(case, x0, dt, 1, threads)
            ks = int(max(1, min(5, 20.0 // max(probe, 1e-3))))
            rate, sec = oracle_rate(case, x0, dt, ks, threads)
            cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"{ks} RK steps of the full {args.n}^3 mesh, FP64 oracle "
                             f"({sec:.1f} s)"}
            # one thread, the reference's one-rank behaviour: one RK step of the
            # same pulse on a 32^3 mesh (the rate per unknown does not depend
            # on the mesh size for this element-local work)
            small = cases.pulse3d(n=min(32, args.n), order=2, steps=1, cfl=0.2)
            from oracle import refcpu
            o1 = refcpu.Oracle(small.mesh, small.order)
            cases.configure_oracle(small, o1)
            xs = cases.project(small, o1.node_coords())
            dts = 0.2 * o1.hmin() / o1.face_speed(xs) / 5.0
            r1, s1 = oracle_rate(small, xs, dts, 1, 1)
            cpu["one_thread"] = {"value": r1, "cores": 1,
                                 "sample": f"1 RK step of the {min(32, args.n)}^3 pulse ({s1:.1f} s)"}
        except Exception as exc:  # pragma: no cover
            cpu = {"value": None, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"failed: {exc}"}

    if rank == 0:
        cfg = workload_config(case, args.n)
        cfg["unknowns"] = N
        cfg["precision"] = "fp32-bulk (float-pair conserved state)"
        cfg["parallelism"] = f"replicas x{world}"
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "fp64": {"value": value64, "unit": UNIT, "steps": k64,
                     "ms_per_step": 1e3 * sec64 / k64, "speedup_mixed_vs_fp64": value / value64},
            "error_vs_fp64": err,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


def one_thread_rate(fn, units, sample, threads):
    """The oracle on one host thread (the reference's one-rank behaviour):
    units / seconds of fn(), then the thread count is restored."""
    from oracle import refcpu
    refcpu.set_threads(1)
    try:
        t0 = time.perf_counter()
        fn()
        sec = time.perf_counter() - t0
    finally:
        refcpu.set_threads(threads)
    return {"value": units / sec, "cores": 1, "sample": f"{sample} ({sec:.1f} s)"}


def run_config(args, local):
    """The other configurations of the workload set, one JSON line each (the
    headline line is the C2 pulse of run_ours):
      c1  Sod 200x4 Q1, HLLC + Einfeldt, BJ limiter, SSP-RK3 CFL 0.3 to t = 0.2
      c3  double Mach reflection, 524,288 jittered P1 triangles, HLL + TRRS,
          Venkatakrishnan, SSP-RK3 CFL 0.25 (the first --config-steps steps);
          as in the reference, each run limits the projected state once
          before its first step (its nodal projection of the Mach-10 jump is
          non-physical on faces of the shock cells until then)
      c4  256 batched Riemann problems on N x 4 strips, one graph launch, to t = 0.15
      c5  adjoint: 32^3 Q1 Gaussian pulses, HLLC + Venkatakrishnan, 200 fixed-dt
          steps forward, then the checkpointed adjoint run (every 20 steps)
      c6  adapted mesh: the C2 pulse on a 48^3 Q2 mesh whose elements within
          0.15 of the pulse centre are refined once (hanging faces), against
          the same pulse on the conforming 48^3 mesh, 100 fixed-dt steps
    FP64 and FP32-bulk runs of the same workload with the density / energy error
    of the latter against the former, and the FP64 oracle on a bounded sample."""
    import torch
    from oracle import refcpu
    from rkdg3d_gb300 import cases
    from rkdg3d_gb300.solver import FP32_BULK, FP64, Context

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    threads = os.cpu_count() or 1
    w = args.config

    def timed(fn):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize(dev)
        return r, time.perf_counter() - t0

    def context(case, prec):
        ctx = Context(case.mesh, case.order, device=local, precision=prec)
        cases.configure_context(case, ctx)
        ctx.set_stream(stream.cuda_stream)
        return ctx

    def errors(a, b, nd):
        ra, rb, Ea, Eb = a[:nd], b[:nd], a[-nd:], b[-nd:]
        return {"rho_rel_l1": float(np.abs(ra - rb).sum() / np.abs(rb).sum()),
                "rho_linf": float(np.abs(ra - rb).max()),
                "E_rel_l1": float(np.abs(Ea - Eb).sum() / np.abs(Eb).sum()),
                "E_linf": float(np.abs(Ea - Eb).max())}

    line = {"config": w, "unit": UNIT, "data": "synthetic", "n_gpus": 1}
    if w in ("c1", "c3"):
        case = cases.sod() if w == "c1" else cases.double_mach()
        kw = {} if w == "c1" else {"max_steps": args.config_steps}
        out = {}
        for name, prec in (("fp64", FP64), ("fp32_bulk", FP32_BULK)):
            ctx = context(case, prec)
            x0 = torch.tensor(cases.project(case, ctx.node_coords()), dtype=torch.float64, device=dev)
            x = x0.clone()
            ctx.run(x, case.t_end, case.cfl, max_steps=2)  # warm-up
            x = x0.clone()
            info, sec = timed(lambda: ctx.run(x, case.t_end, case.cfl, **kw))
            out[name] = (x.cpu().numpy(), info, sec)
            line[name] = {"value": ctx.n * STAGES * info["steps"] / sec, "steps": info["steps"],
                          "ms_per_step": 1e3 * sec / info["steps"], "t": info["t"]}
            n, nd = ctx.n, ctx.ndofs
        line["unknowns"] = n
        line["error_fp32_bulk_vs_fp64"] = errors(out["fp32_bulk"][0], out["fp64"][0], nd)
        if w == "c1":
            # the same run as a batch of one problem: the whole time loop in one
            # CUDA-graph launch (device-side dt and stopping test), without the
            # host round trip per step of rkdg_run
            ctx = context(case, FP32_BULK)
            ctx.batch_setup(np.array([0, case.mesh.num_elements], np.int32),
                            np.array([case.gamma]), np.array([case.covolume]))
            x0 = torch.tensor(cases.project(case, ctx.node_coords()), dtype=torch.float64, device=dev)
            x = x0.clone()
            ctx.batch_run(x, case.t_end, case.cfl, max_steps=2)  # warm-up (graph build)
            x = x0.clone()
            binfo, sec = timed(lambda: ctx.batch_run(x, case.t_end, case.cfl))
            bsteps = int(np.asarray(binfo["steps"])[0])
            line["fp32_bulk_one_graph_launch"] = {
                "value": ctx.n * STAGES * bsteps / sec, "steps": bsteps,
                "ms_per_step": 1e3 * sec / max(bsteps, 1),
                "rho_rel_l1_vs_fp32_bulk_host_loop": float(
                    np.abs(x.cpu().numpy()[:nd] - out["fp32_bulk"][0][:nd]).sum()
                    / np.abs(out["fp32_bulk"][0][:nd]).sum())}
        # at matched step counts: dt fixed from the FP64 CFL evaluation of the
        # initial state, the same in both arms; and the FP64 path's own spread
        # when its initial state is perturbed by 1e-7 (FP32 rounding) relative
        matched = {}
        for name, prec, pert in (("fp64", FP64, 0.0), ("fp32_bulk", FP32_BULK, 0.0),
                                 ("fp64_perturbed_1e-7", FP64, 1e-7)):
            ctx = context(case, prec)
            xh = cases.project(case, ctx.node_coords())
            if pert:
                xh = xh * (1.0 + pert * np.random.default_rng(1).uniform(-1, 1, xh.size))
            x = torch.tensor(xh, dtype=torch.float64, device=dev)
            inf = ctx.run(x, case.t_end, case.cfl, dt_mode=1, **kw)
            matched[name] = (x.cpu().numpy(), inf["steps"])
        line["matched_steps"] = {
            "steps": matched["fp64"][1], "dt": "fixed from the FP64 CFL of the initial state",
            "fp32_bulk_vs_fp64": errors(matched["fp32_bulk"][0], matched["fp64"][0], nd),
            "fp64_perturbed_1e-7_vs_fp64": errors(matched["fp64_perturbed_1e-7"][0],
                                                  matched["fp64"][0], nd)}
        orc = refcpu.Oracle(case.mesh, case.order)
        cases.configure_oracle(case, orc)
        xo = cases.project(case, orc.node_coords())
        ksteps = out["fp64"][1]["steps"] if w == "c1" else 2
        refcpu.set_threads(threads)
        t0 = time.perf_counter()
        orc.run(xo, case.t_end, case.cfl, max_steps=ksteps)
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": orc.n * STAGES * ksteps / sec, "cores": threads,
                                "kind": "port", "sample": f"{ksteps} RK steps, FP64 oracle"}
        k1 = 100 if w == "c1" else 1
        line["cpu_baseline"]["one_thread"] = one_thread_rate(
            lambda: orc.run(xo, case.t_end, case.cfl, max_steps=k1), orc.n * STAGES * k1,
            f"{k1} RK step(s), FP64 oracle", threads)
    elif w == "c4":
        bc = cases.batched_riemann()
        for name, prec in (("fp64", FP64), ("fp32_bulk", FP32_BULK)):
            ctx = Context(bc.mesh, bc.order, device=local, precision=prec)
            cases.configure_batch(bc, ctx)
            ctx.set_stream(stream.cuda_stream)
            x0 = torch.tensor(bc.project(ctx.node_coords()), dtype=torch.float64, device=dev)
            x = x0.clone()
            ctx.batch_run(x, bc.t_end, bc.cfl, max_steps=2)  # warm-up (graph build)
            x = x0.clone()
            info, sec = timed(lambda: ctx.batch_run(x, bc.t_end, bc.cfl))
            steps = np.abs(np.asarray(info["steps"]))
            per_problem = np.diff(bc.offsets) * 4 * 4  # Q1 quads: 4 nodes x 4 variables
            units = float((per_problem * steps).sum()) * STAGES
            line[name] = {"value": units / sec, "seconds": sec, "problems": len(steps),
                          "failed": int((np.asarray(info["steps"]) < 0).sum()),
                          "max_steps": int(steps.max()),
                          "active_fraction": float((np.diff(bc.offsets).astype(np.float64) * steps).sum()
                                                   / (float(bc.mesh.num_elements) * float(steps.max())))}
            if prec == FP32_BULK:
                # algorithmic bytes of the problems' own steps (stored widths):
                # the stage kernel's state streams (68 N per RK step, as the
                # C2 accounting), the limiter's read and write of each stage
                # output (8 N + 8 N + 16 N), and the cell means (8 B written,
                # read by the element and its 4 neighbours, per variable, stage
                # and element)
                ne_p = np.diff(bc.offsets)
                bytes_p = 100.0 * per_problem + 3 * 48.0 * 4 * ne_p
                achieved = float((bytes_p * steps).sum()) / sec / 1e9
                peak = _peak_hbm()
                line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak[0],
                                    "unit": "GB/s", "frac": achieved / peak[0], "peak_source": peak[1],
                                    "note": "whole batched run: algorithmic bytes of the active "
                                            "problems' steps / run time"}
            if name == "fp64":
                a64 = x.cpu().numpy()
                ok64 = np.asarray(info["steps"]) > 0
                nd = ctx.ndofs
            else:
                # problems that ran to t_end in both arms (the others stopped
                # on a non-physical state, where the reference would exit)
                ok = ok64 & (np.asarray(info["steps"]) > 0)
                keep = np.repeat(ok, np.diff(bc.offsets) * 4)  # 4 nodes per Q1 quad
                sel = np.concatenate([keep] * 4)
                line["error_fp32_bulk_vs_fp64"] = errors(x.cpu().numpy()[sel], a64[sel], int(keep.sum()))
                line["error_fp32_bulk_vs_fp64"]["problems_compared"] = int(ok.sum())
        line["unknowns"] = int(ctx.n)
        # matched step counts: dt fixed per problem from the FP64 CFL of its
        # initial state (the same in both arms), and the FP64 path's spread
        # under a 1e-7 relative perturbation of the initial state
        matched = {}
        for name, prec, pert in (("fp64", FP64, 0.0), ("fp32_bulk", FP32_BULK, 0.0),
                                 ("fp64_perturbed_1e-7", FP64, 1e-7)):
            ctx = Context(bc.mesh, bc.order, device=local, precision=prec)
            cases.configure_batch(bc, ctx)
            ctx.set_stream(stream.cuda_stream)
            xh = bc.project(ctx.node_coords())
            if pert:
                xh = xh * (1.0 + pert * np.random.default_rng(1).uniform(-1, 1, xh.size))
            x = torch.tensor(xh, dtype=torch.float64, device=dev)
            inf = ctx.batch_run(x, bc.t_end, bc.cfl, dt_mode=1)
            matched[name] = (x.cpu().numpy(), np.asarray(inf["steps"]))
        okm = np.all([m[1] > 0 for m in matched.values()], axis=0)
        keep = np.repeat(okm, np.diff(bc.offsets) * 4)
        sel = np.concatenate([keep] * 4)
        nk = int(keep.sum())
        line["matched_steps"] = {
            "dt": "fixed per problem from the FP64 CFL of its initial state",
            "problems_compared": int(okm.sum()),
            "steps_equal": bool(np.array_equal(matched["fp64"][1], matched["fp32_bulk"][1])),
            "fp32_bulk_vs_fp64": errors(matched["fp32_bulk"][0][sel], matched["fp64"][0][sel], nk),
            "fp64_perturbed_1e-7_vs_fp64": errors(matched["fp64_perturbed_1e-7"][0][sel],
                                                  matched["fp64"][0][sel], nk)}

        # the same differences problem by problem (density rows: 4 nodes per
        # Q1 quad), as quantiles over the problems
        def per_problem(a, b):
            out = []
            for p_ in range(len(bc.offsets) - 1):
                if not okm[p_]:
                    continue
                lo, hi = 4 * bc.offsets[p_], 4 * bc.offsets[p_ + 1]
                ref = np.abs(b[lo:hi]).sum()
                out.append(float(np.abs(a[lo:hi] - b[lo:hi]).sum() / max(ref, 1e-300)))
            q = np.asarray(out)
            return {"median": float(np.median(q)), "p90": float(np.quantile(q, 0.9)),
                    "max": float(q.max()), "problems_le_1e-6": int((q <= 1e-6).sum()),
                    "problems_le_1e-4": int((q <= 1e-4).sum()), "problems": int(q.size)}
        line["matched_steps"]["rho_rel_l1_per_problem"] = {
            "fp32_bulk_vs_fp64": per_problem(matched["fp32_bulk"][0], matched["fp64"][0]),
            "fp64_perturbed_1e-7_vs_fp64": per_problem(matched["fp64_perturbed_1e-7"][0],
                                                       matched["fp64"][0])}
        small = int(np.argmin(np.diff(bc.offsets)))
        c = bc.cases[small]
        orc = refcpu.Oracle(c.mesh, c.order)
        cases.configure_oracle(c, orc)
        refcpu.set_threads(threads)
        t0 = time.perf_counter()
        try:
            _, ir = orc.run(cases.project(c, orc.node_coords()), c.t_end, c.cfl)
            sec = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": orc.n * STAGES * ir["steps"] / sec, "cores": threads,
                                    "kind": "port",
                                    "sample": f"the smallest problem ({np.diff(bc.offsets)[small]} "
                                              "elements) run alone, FP64 oracle"}
            x_small = cases.project(c, orc.node_coords())
            line["cpu_baseline"]["one_thread"] = one_thread_rate(
                lambda: orc.run(x_small, c.t_end, c.cfl, max_steps=200), orc.n * STAGES * 200,
                "200 RK steps of the smallest problem, FP64 oracle", threads)
        except refcpu.OracleError as ex:
            line["cpu_baseline"] = {"unavailable": str(ex)[:80]}
    elif w == "c6":
        from rkdg3d_gb300 import mesh as M
        base = cases.pulse3d(n=48)
        cen = base.mesh.elem_coords.mean(1)
        ref = np.flatnonzero(np.linalg.norm(cen - 0.5, axis=1) < 0.15)
        nc = cases.pulse3d(n=48)
        nc.mesh = M.refine_nc(base.mesh, ref)
        steps = args.config_steps // 2
        out = {}
        for label, case in (("conforming", base), ("adapted", nc)):
            for name, prec in (("fp64", FP64), ("fp32_bulk", FP32_BULK)):
                ctx = context(case, prec)
                x0 = torch.tensor(cases.project(case, ctx.node_coords()), dtype=torch.float64,
                                  device=dev)
                dt = case.cfl * ctx.hmin() / ctx.face_speed(x0) / (2 * case.order + 1)
                x = x0.clone()
                ctx.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=2)  # warm-up
                x = x0.clone()
                info, sec = timed(lambda: ctx.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=steps))
                out[(label, name)] = x.cpu().numpy()
                line.setdefault(label, {})[name] = {"value": ctx.n * STAGES * steps / sec,
                                                    "ms_per_step": 1e3 * sec / steps}
                line[label]["unknowns"] = ctx.n
                line[label]["elements"] = ctx.ne
            line[label]["error_fp32_bulk_vs_fp64"] = errors(out[(label, "fp32_bulk")],
                                                           out[(label, "fp64")], ctx.ndofs)
        line["adapted"]["refined_elements"] = int(len(ref))
        orc = refcpu.Oracle(nc.mesh, nc.order)
        cases.configure_oracle(nc, orc)
        refcpu.set_threads(threads)
        xo = cases.project(nc, orc.node_coords())
        t0 = time.perf_counter()
        orc.run(xo, 1e30, dt0=dt, dt_mode=2, max_steps=2)
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": orc.n * STAGES * 2 / sec, "cores": threads,
                                "kind": "port", "sample": "2 RK steps on the adapted mesh, FP64 oracle"}
    elif w == "c5":
        case = cases.gaussian_pulses(n=32, seed=0)
        ctx = context(case, FP64)
        x0 = torch.tensor(cases.project(case, ctx.node_coords()), dtype=torch.float64, device=dev)
        dt = case.cfl * ctx.hmin() / ctx.face_speed(x0) / (2 * case.order + 1)
        x = x0.clone()
        ctx.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=2, limit_initial=False)
        x = x0.clone()
        # the adjoint's forward map: 200 steps from x0 as given
        _, sec_f = timed(lambda: ctx.run(x, 1e30, dt0=dt, dt_mode=2, max_steps=200,
                                         limit_initial=False))
        xbar = torch.zeros_like(x)
        xbar[:ctx.ndofs] = x[:ctx.ndofs] - x0[:ctx.ndofs]
        xT = torch.empty_like(x)
        _, sec_a = timed(lambda: ctx.adjoint_run(x0, 200, dt, 20, xbar, xT))
        line["fp64"] = {"value": ctx.n * STAGES * 200 / sec_f, "forward_seconds": sec_f,
                        "adjoint_seconds": sec_a, "adjoint_over_forward": sec_a / sec_f}
        line["unknowns"] = ctx.n
        orc = refcpu.Oracle(case.mesh, case.order)
        cases.configure_oracle(case, orc)
        refcpu.set_threads(threads)
        xo = cases.project(case, orc.node_coords())
        t0 = time.perf_counter()
        orc.run(xo, 1e30, dt0=dt, dt_mode=2, max_steps=2, limit_initial=False)
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": orc.n * STAGES * 2 / sec, "cores": threads,
                                "kind": "port", "sample": "2 RK steps, FP64 oracle"}
        line["cpu_baseline"]["one_thread"] = one_thread_rate(
            lambda: orc.run(xo, 1e30, dt0=dt, dt_mode=2, max_steps=1, limit_initial=False),
            orc.n * STAGES, "1 RK step, FP64 oracle", threads)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--elements-per-side", dest="n", type=int, default=64,
                    help="elements per side (the long form passes through torchrun)")
    ap.add_argument("--fp64-steps", type=int, default=500,
                    help="steps of the plain FP64 run (timed, and the accuracy reference)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--hex-kernel", type=int, default=0,
                    help="RKDG_TUNE_HEX_KERNEL of the FP32-bulk context (0: library default)")
    ap.add_argument("--config", default="c2", choices=["c2", "c1", "c3", "c4", "c5", "c6"],
                    help="c2: the headline pulse (default); c1/c3/c4/c5/c6: the other "
                         "configurations, one JSON line each")
    ap.add_argument("--config-steps", type=int, default=200,
                    help="RK steps of the c3 runs (first steps of the t = 0.2 run)")
    ap.add_argument("--traffic-per-launch", type=float, default=None,
                    help="DRAM bytes per stage launch from an ncu capture (profiles/)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config != "c2":
        if rank == 0:
            run_config(args, local)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
