"""OC iterations/s on the 240x80x80 hex cantilever (1,536,000 elements).

The GB300 arm runs the density-method loop of scikit-topt (Gaussian filter
r = 1.5, Heaviside projection, SIMP p = 3, E0 = 1, Emin = 1e-9, nu = 0.3,
OC with move limit 0.2, volume fraction 0.3) twice from the same start: with
the mixed-precision solver (FP32 multigrid inner solve, FP64 residual,
update and dots; outer tolerance 1e-8) -- the headline ``value`` -- and with
the plain FP64 solver, whose rate is reported beside it together with the
per-iteration compliance difference.  One step = one OC iteration on device-
resident data; ``e2e`` repeats the mixed run through the host-buffer call
(density copied in from pinned host memory and copied back with the
compliance every step).

``--impl reference`` times the CPU restatement of the reference algorithm
(oracle/, NumPy/SciPy: Gaussian filter rebuilt on every call as in
sktopt/filters/spacial.py:139-149, CG with Jacobi preconditioner capped at
1000 iterations by the reference's maxiter rule) on a bounded sample and
scales it to the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "scikit-topt_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = ("OC iters/s at 1.5M hex, mixed-prec vs FP64 GPU "
          "(compliance rel err ≤1e-6)")
SIZE = (240, 80, 80)
# DRAM bytes per node of one k_mf_tile launch (ncu, 120x40x40, caches flushed)
MF_TRAFFIC_PER_NODE = 19.95


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, nargs=3, default=list(SIZE))
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c1", action="store_true",
                    help="skip the 60x20x20 same-configuration run against the reference")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 256 batched designs (sharded over the ranks when N > 1)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the multi-load tetrahedral and autograd configurations")
    ap.add_argument("--phases", action="store_true", help="print a per-phase breakdown")
    ap.add_argument("--nvtx-steps", action="store_true",
                    help="one NVTX range mixed_<k> per timed iteration (profiler filtering)")
    ap.add_argument("--probe", choices=["spmv", "solve", "batch", "autograd", "heat_robin", "amg",
                                        "multiload"],
                    default=None,
                    help="profiling target instead of the benchmark")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def measured_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.out = open(os.path.join("/tmp", f"topt_clocks_{os.getpid()}.csv"), "w+")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.seek(0)
        rows = [r.split(",") for r in self.out.read().strip().splitlines() if r.strip()]
        self.out.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_optimizer(size, precision, max_iters, device, solver="cg_pyamg"):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    cfg = OC_Config(max_iters=max_iters, filter_type="spacial",
                    filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                    p=tools.SchedulerConfig.constant(target_value=3.0),
                    vol_frac=tools.SchedulerConfig.constant(target_value=0.3),
                    move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                    E_min_coeff=1e-9, solver_option=solver, solver_rtol=1e-8,
                    precision=precision, autotune=True)
    opt = OC_Optimizer(cfg, toy_problem.cantilever(*size), device=device)
    opt.parameterize()
    return opt


def replica_barrier():
    """Barrier across the replicas (no-op for one process)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def replica_max(t):
    """Maximum of a per-replica time over all replicas (the job's time)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
        return float(t)
    dev = torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend() == "nccl" else torch.device("cpu")
    tt = torch.tensor([float(t)], dtype=torch.float64, device=dev)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def timed_run(opt, warmup, steps, sampler=None, label="steps", step_ranges=False):
    """Warm-up, then `steps` OC iterations timed with CUDA events, bracketed
    by a replica barrier and a device synchronisation on both sides.  NVTX,
    for profiler filtering: one range `label` around the window, or with
    `step_ranges` one range `label_<k>` around each timed iteration k = 1..K
    instead.  Also returns the launch count of each timed iteration."""
    import torch
    for _ in range(warmup):
        opt.optimize_steps(1)
    torch.cuda.synchronize()
    replica_barrier()
    from sktopt_gb300 import _native
    l0 = _native.launch_count()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if sampler:
        sampler.start()
    torch.cuda.synchronize()
    if not step_ranges:
        torch.cuda.nvtx.range_push(label)
    e0.record(s)
    t0 = time.perf_counter()
    per_step = []
    for k in range(steps):
        lk = _native.launch_count()
        if step_ranges:
            torch.cuda.nvtx.range_push(f"{label}_{k + 1}")
        opt.optimize_steps(1)
        if step_ranges:
            torch.cuda.nvtx.range_pop()
        per_step.append(_native.launch_count() - lk)
    e1.record(s)
    torch.cuda.synchronize()
    if not step_ranges:
        torch.cuda.nvtx.range_pop()
    replica_barrier()
    wall = time.perf_counter() - t0
    clocks = sampler.stop() if sampler else None
    l1 = _native.launch_count()
    ms = e0.elapsed_time(e1)
    return ms, wall, l1 - l0, clocks, per_step


def _event_time(fn, n=20):
    import torch
    for _ in range(3):
        fn()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(n):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / n * 1e-3


def roofline(opt, peak_gbs):
    """Roofline of the kernel family with the largest share of the mixed OC
    iteration: the FP32 matrix-free fine-level operator (four launches per
    V-cycle plus the search-direction product), timed through the FP32
    operator call with CUDA events on the launching stream, for both of its
    kernels: k_mf_tile (FP32 FMA, the solver's default) and k_mf_tc (tensor
    cores: tcgen05 TF32 MMAs with the 3xTF32 split).  Algorithmic bytes per
    launch: x and y (2 * 12 B per node), the fixed-DOF flags (4 B per node)
    and the cell coefficients (4 B per cell).  The FP64 SpMV of the residual
    replacements is reported as well."""
    import torch
    eng = opt.fem.engine
    nodes, cells = eng.mesh.nnodes, eng.mesh.nelements
    x64 = torch.rand((eng.n_dof, 1), dtype=torch.float64, device=eng.device)
    x32 = x64.float()
    times = {}
    for kind in (1, 0):                    # the default (0) is left selected
        eng.set_mf_kernel(kind)
        times[kind] = _event_time(lambda: eng.spmv(x32, torch.float32))
    t64 = _event_time(lambda: eng.spmv(x64))
    bytes_mf = 28 * nodes + 4 * cells
    # DRAM traffic per launch: an ncu capture of the operator on the 120x40x40
    # cantilever (caches flushed), in bytes per node, scaled by node count
    traffic = MF_TRAFFIC_PER_NODE * nodes
    nb = eng.nnzb
    bytes64 = nb * (9 * 8 + 4) + 4 * (nodes + 1) + 2 * 8 * eng.n_dof
    t32 = times[0]
    achieved = bytes_mf / t32 / 1e9
    return {"kernel": "k_mf_tile (FP32 matrix-free operator, fine level)", "bound": "hbm",
            "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
            "frac": round(achieved / peak_gbs, 3), "bytes_per_launch": int(bytes_mf),
            "launch_us": round(t32 * 1e6, 1), "traffic": int(traffic),
            "limiter": "FP32 FMA issue",
            "fp32_tflops": round(2 * 576 * nodes / t32 / 1e12, 2),
            "tensor_core_kernel": {
                "kernel": "k_mf_tc (tcgen05, 3xTF32)", "launch_us": round(times[1] * 1e6, 1),
                "achieved_gbs": round(bytes_mf / times[1] / 1e9, 1)},
            "fp64_spmv": {"kernel": "k_sell_spmv<double,3,1> (residual replacement)",
                          "launch_us": round(t64 * 1e6, 1),
                          "achieved_gbs": round(bytes64 / t64 / 1e9, 1),
                          "bytes_per_launch": int(bytes64)}}


FULL_ITERS = 50     # the 240x80x80 configuration's iteration count


def per_iteration_run(opt, n_iter, check=None):
    """Iterations 1..n_iter of `opt`, each bracketed by CUDA events on the
    launching stream (the events see only the iteration); `check(opt)` runs
    after each iteration, outside the events.  Returns (per-iteration ms,
    check results)."""
    import torch
    s = torch.cuda.current_stream()
    evs = []
    out = []
    for _ in range(n_iter):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        opt.optimize_steps(1)
        e1.record(s)
        evs.append((e0, e1))
        if check is not None:
            out.append(check(opt))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs], out


def same_density_checker(opt, dev):
    """After a mixed iteration: the FP64 solve (to 1e-10) at the iteration's
    projected density and its sensitivity chain (dC_drho_simp x dH, filter
    transpose), against the mixed iteration's compliance and filtered
    sensitivity (relative error and relative L2)."""
    import torch
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    f64 = FEM_SimpLinearElasticity(opt.tsk, 1e-9, solver_config=LinearSolverConfig(
        solver="cg_pyamg", rtol=1e-10, precision="fp64"), device=dev)
    U64 = torch.zeros_like(opt._state.u_dofs) if opt._state is not None else None

    def check(o):
        nonlocal U64
        st = o._state
        if U64 is None:
            U64 = torch.zeros_like(st.u_dofs)
        c64 = float(f64.solve_device(st.rho_projected, 3.0, U64)[0])
        _, dcp = f64.sensitivity_multi_load(st.rho_projected, 3.0, U64, dh=st.dH_drho,
                                            want_energy=False)
        g64 = o.filter.gradient_device(dcp[:, 0].contiguous())
        c32 = float(o.recorder.histories["compliance"][-1])
        serr = float(torch.linalg.norm(st.dC_drho_full - g64) / torch.linalg.norm(g64))
        return abs(c32 - c64) / abs(c64), serr
    return check


def run_gpu(args):
    import numpy as np
    import torch
    rank, local, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    size = tuple(args.size)
    peak, peak_kind = measured_peak_gbs()
    total = args.warmup + args.steps
    n_full = max(FULL_ITERS, total)
    # mixed precision (headline): W warm-up iterations, K timed
    opt = make_optimizer(size, "mixed", n_full, dev)
    ms, wall, launches, clocks, per_step = timed_run(
        opt, args.warmup, args.steps, ClockSampler(local), label="mixed",
        step_ranges=args.nvtx_steps)
    phases = None
    if args.phases:
        opt.timer.enabled = True
        opt.optimize_steps(2)
        opt.timer.enabled = False
        phases = opt.timer.report()
    mixed_stats = [(s.iters, s.outer, s.relres) for s in opt.fem.solve_history]
    roof = roofline(opt, peak)
    n = opt.tsk.mesh.nelements
    del opt
    torch.cuda.empty_cache()
    # all iterations of the configuration, mixed, each against the FP64 solve
    # and sensitivity chain at the same density
    full = None
    comp_mixed = None
    if not args.no_fp64:
        om = make_optimizer(size, "mixed", n_full, dev)
        om._ensure_state_initialized()
        om.fem.engine                     # set-up outside the timed iterations
        t_mixed, errs = per_iteration_run(om, n_full, same_density_checker(om, dev))
        comp_mixed = list(om.recorder.histories["compliance"])
        full = {"iterations": n_full, "mixed_it_per_s": round(n_full / (sum(t_mixed) * 1e-3), 4),
                "mixed_ms_per_iter": [round(t, 2) for t in t_mixed],
                "compliance_rel_err_same_density": [float(f"{e[0]:.3e}") for e in errs],
                "sensitivity_rel_l2_err_same_density": [float(f"{e[1]:.3e}") for e in errs],
                "compliance_rel_err_same_density_max": max(e[0] for e in errs),
                "sensitivity_rel_l2_err_same_density_max": max(e[1] for e in errs),
                "mixed_solver_iters": [(s.iters, s.outer) for s in om.fem.solve_history],
                "_t_mixed": t_mixed}
        del om
        torch.cuda.empty_cache()
    # e2e: the same iterations (same start, same warm-up) through the
    # host-buffer call path: density from pinned host memory in, density and
    # compliance back out, every step
    e2e = None
    if not args.no_e2e:
        oe = make_optimizer(size, "mixed", n_full, dev)
        rho_h = torch.empty(n, dtype=torch.float64).pin_memory()
        oe.optimize_steps(1)                  # state initialised
        rho_h.copy_(oe._state.rho)
        for _ in range(args.warmup - 1):
            oe.step_host(rho_h)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            oe.step_host(rho_h)
        e2e_wall = time.perf_counter() - t0
        e2e = {"value": round(args.steps / e2e_wall * world, 4), "unit": "OC iters/s",
               "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n + 8}
        del oe
        torch.cuda.empty_cache()
    # plain FP64 path from the same start: the K-step window and all iterations
    fp64 = None
    if not args.no_fp64:
        o64 = make_optimizer(size, "fp64", n_full, dev)
        o64._ensure_state_initialized()
        o64.fem.engine
        t64, _ = per_iteration_run(o64, n_full)
        ms64 = sum(t64[args.warmup:total])          # the same K-step window
        comp64 = list(o64.recorder.histories["compliance"])
        errs = [abs(a - b) / abs(b) for a, b in zip(comp_mixed, comp64)]
        fp64 = {"value": round(args.steps / (ms64 * 1e-3), 4),
                "ms_per_step": round(ms64 / args.steps, 2),
                "compliance_rel_err_max": max(errs), "compliance_rel_err_per_iter": errs,
                "speedup_mixed_vs_fp64": round(ms64 / ms, 3),
                "solver_iters": [(s.iters, s.relres) for s in o64.fem.solve_history][-args.steps:]}
        full["fp64_it_per_s"] = round(n_full / (sum(t64) * 1e-3), 4)
        full["fp64_ms_per_iter"] = [round(t, 2) for t in t64]
        full["speedup_mixed_vs_fp64"] = round(sum(t64) / sum(full["_t_mixed"]), 3)
        del o64
    if full is not None:
        full.pop("_t_mixed", None)
    # max over ranks
    t_step = replica_max(ms * 1e-3)
    value = args.steps / t_step * world
    if args.phases and rank == 0:
        print(json.dumps({"phases_ms_mixed": phases}), file=sys.stderr)
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "OC iters/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_step * 1e3 / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (cantilever generated in-process)",
        "config": {"workload": f"OC loop, {size[0]}x{size[1]}x{size[2]} hex cantilever "
                               f"({size[0]*size[1]*size[2]} elements), Gaussian filter r=1.5, "
                               "SIMP p=3, vf=0.3, move 0.2, FP64 flexible CG with FP32 "
                               "multigrid and FP32 operator, FP64 residual replacement, "
                               "to 1e-8; launch shapes from the autotuner",
                   "parallelism": f"replicas x{world}",
                   "l2": "working set (>4 GB per step) exceeds the 129 MB L2"},
        "e2e": e2e, "gpu_launches": int(launches), "gpu_launches_per_step": per_step,
        "roofline": dict(roof, peak_kind=peak_kind),
        "fp64_path": fp64,
        "all_iterations": full,
        "mixed_solver_iters": mixed_stats[-args.steps:],
        "clocks": clocks,
    }
    if rank == 0 and not args.no_c1:
        line["c1_same_config"] = c1_same_config(dev)
    if not args.no_batch:
        line["batched_designs"] = batch_result(world)
    if rank == 0 and not args.no_extra:
        # the other configurations at full size, on this rank's GPU
        line["multi_load_tet"] = probe_multiload()
        line["autograd"] = probe_autograd()
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(size, quick=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if rank == 0:
        print(json.dumps(line))


def cpu_sample(sample, steps_cap=None):
    """One oracle OC iteration on a cantilever of `sample` cells; returns seconds."""
    import numpy as np
    from oracle import optim as oopt
    from oracle import problems
    from oracle.filters import SpacialFilter

    class RebuildingFilter(SpacialFilter):
        """spacial.py:135-157 rebuilds W on every forward call."""

        def forward(self, rho):
            r = self.radius
            self.radius = None
            self.update_radius(r)
            return super().forward(rho)

    m, pb, design, fixed, vol = problems.cantilever(*sample)
    mask = np.zeros(m.nelements, bool)
    mask[design] = True
    filt = RebuildingFilter(m, 1.5, mask)
    cfg = oopt.OracleConfig(max_iters=50, p=oopt.Sched("Constant", 3.0, 3.0),
                            vol_frac=oopt.Sched("Constant", 0.3, 0.3),
                            move_limit=oopt.Sched("Constant", 0.2, 0.2),
                            filter_radius=oopt.Sched("Constant", 1.5, 1.5), E_min_coeff=1e-9,
                            solver="cg_pyamg", rtol=1e-8)
    opt = oopt.OracleOptimizer(cfg, pb, filt, design, fixed, vol)
    t0 = time.perf_counter()
    opt.step()
    return time.perf_counter() - t0, m.nelements


CPU_SAMPLE = (48, 16, 16)


def _sample_text(sample, ne, sec, scale, cores):
    return (f"one OC iteration of the oracle (NumPy/SciPy restatement of the reference "
            f"loop, its cg_pyamg solver option: SciPy CG to 1e-8 preconditioned by the "
            f"restated smoothed-aggregation V-cycle, converged; W of the Gaussian filter "
            f"rebuilt per call as the reference does) on the {sample[0]}x{sample[1]}x"
            f"{sample[2]} cantilever ({ne} elements, {sec:.2f} s), scaled x{scale:.1f} by "
            f"element count (a lower bound on the full-size time: the AMG-CG iteration "
            f"count grows with size); host has {cores} cores, the SciPy sparse kernels "
            f"and the C smoother run on one")


def cpu_baseline(size, quick=True):
    """Oracle iteration on a bounded sample of the workload, scaled linearly in
    the element count."""
    cores = len(os.sched_getaffinity(0))
    sec, ne = cpu_sample(CPU_SAMPLE)
    scale = (size[0] * size[1] * size[2]) / ne
    return {"value": round(1.0 / (sec * scale), 6), "unit": "OC iters/s", "cores": 1,
            "kind": "port", "extrapolated": True,
            "sample": _sample_text(CPU_SAMPLE, ne, sec, scale, cores)}


C1_SIZE, C1_ITERS = (60, 20, 20), 30
C1_FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                          "ref_loop_oc_60x20x20.npz")


def c1_same_config(dev):
    """The 60x20x20 cantilever (24,000 elements, FP64, 30 OC iterations) on
    the GPU, against the committed run of the reference's own driver loop on
    the same configuration (tests/golden/ref_loop_oc_60x20x20.npz, written by
    tests/golden/make_ref_fixtures.py --c1 with the oracle's FEM plugin and
    SuperLU solves): the compliance of every iteration, and the measured wall
    time of that CPU run (one x86 core of the machine that wrote it)."""
    import numpy as np
    import torch
    R = np.load(C1_FIXTURE)
    opt = make_optimizer(C1_SIZE, "fp64", C1_ITERS, dev, solver="spsolve")
    opt._ensure_state_initialized()
    opt.fem.engine
    t, _ = per_iteration_run(opt, C1_ITERS)
    comp = np.array(opt.recorder.histories["compliance"])
    err = np.abs(comp - R["compliance"]) / np.abs(R["compliance"])
    cpu_wall = float(R["wall_s"])
    gpu_s = sum(t) * 1e-3
    return {"workload": "60x20x20 hex cantilever, 30 OC iterations, FP64, Gaussian "
                        "filter r=1.5, p=3, vf=0.3, move 0.2 (the reference's CPU-runnable "
                        "configuration)",
            "gpu_it_per_s": round(C1_ITERS / gpu_s, 3),
            "gpu_ms_per_iter": round(gpu_s * 1e3 / C1_ITERS, 2),
            "reference_driver_it_per_s": round(C1_ITERS / cpu_wall, 5),
            "reference_driver_wall_s": round(cpu_wall, 1),
            "reference_driver_measured": "unmodified reference driver loop (scikit-topt "
                                         "0.3.9 DensityMethod) with the oracle FEM plugin "
                                         "and SuperLU (minimum-degree ordering), one x86 "
                                         "core, when the fixture was written",
            "speedup_same_config": round(cpu_wall / gpu_s, 1),
            "compliance_rel_err_vs_reference_max": float(err.max())}


def run_reference(args):
    rank, local, world = dist_env()
    if rank != 0:
        return
    size = tuple(args.size)
    sample = CPU_SAMPLE
    cores = len(os.sched_getaffinity(0))
    for _ in range(args.warmup):
        cpu_sample(sample)
    secs = []
    ne = None
    for _ in range(args.steps):
        s, ne = cpu_sample(sample)
        secs.append(s)
    scale = (size[0] * size[1] * size[2]) / ne
    t = sum(secs) / len(secs) * scale
    v = round(1.0 / t, 6)
    line = {"metric": METRIC, "value": v, "unit": "OC iters/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (cantilever generated in-process)",
            "impl": "reference",
            "config": {"workload": f"OC loop, {size[0]}x{size[1]}x{size[2]} hex cantilever",
                       "parallelism": "host CPU"},
            "cpu_baseline": {"value": v, "unit": "OC iters/s", "cores": 1, "kind": "port",
                             "extrapolated": True,
                             "sample": _sample_text(sample, ne, sum(secs) / len(secs),
                                                    scale, cores)},
            "e2e": {"value": v, "unit": "OC iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def probe_spmv(size):
    """Profiling target: assemble the mixed engine for a cantilever of `size`
    and run the level-0 operator twice in FP32 on the tensor cores (k_mf_tc,
    NVTX range "spmv32"), twice with the FP32-FMA kernel (k_mf_tile, range
    "spmv32fma") and twice in FP64 (assembled SELL, range "spmv64"), then the
    FP32 assembled SELL product of an engine without the matrix-free operator
    twice (range "spmv32sell", the kernel of the coarse levels)."""
    import numpy as np
    import torch
    from sktopt_gb300.fea import composer
    from sktopt_gb300.fea.engine import FemEngine
    from sktopt_gb300.mesh import toy_problem
    dev = torch.device("cuda", 0)
    tsk = toy_problem.cantilever(*size)
    Ke, _, _ = composer.element_matrices(tsk.mesh, 0.3)
    eng = FemEngine(tsk.mesh, 3, Ke, tsk.dirichlet_mask, mixed=True, multigrid=True)
    eng.update(torch.full((tsk.mesh.nelements,), 0.5, dtype=torch.float64, device=dev),
               1.0, 1e-9, 3.0)
    x32 = torch.rand((eng.n_dof, 1), dtype=torch.float32, device=dev)
    x64 = x32.double()
    torch.cuda.synchronize()
    for name, x, dt, kind in (("spmv32", x32, torch.float32, 1),
                              ("spmv32fma", x32, torch.float32, 0),
                              ("spmv64", x64, torch.float64, 1)):
        eng.set_mf_kernel(kind)
        torch.cuda.nvtx.range_push(name)
        for _ in range(2):
            eng.spmv(x, dt)
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    del eng
    sell = FemEngine(tsk.mesh, 3, Ke, tsk.dirichlet_mask, mixed=True, multigrid=True,
                     matrix_free=False)
    sell.update(torch.full((tsk.mesh.nelements,), 0.5, dtype=torch.float64, device=dev),
                1.0, 1e-9, 3.0)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("spmv32sell")
    for _ in range(2):
        sell.spmv(x32, torch.float32)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    eng = sell
    print(json.dumps({"probe": "spmv", "size": list(size), "nnzb": eng.nnzb,
                      "n_dof": eng.n_dof}))


def probe_solve(size):
    """Profiling target: one mixed state solve (default scheme, from a zero
    guess) of the cantilever of `size` at a seeded random density, after a
    warm-up solve of the same system, inside the NVTX range "solve"."""
    import numpy as np
    import torch
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.mesh import toy_problem
    dev = torch.device("cuda", 0)
    tsk = toy_problem.cantilever(*size)
    fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=LinearSolverConfig(
        solver="cg_pyamg", rtol=1e-8, precision="mixed"), device=dev)
    g = np.random.default_rng(0)
    rho = torch.from_numpy(0.01 + 0.99 * g.random(tsk.mesh.nelements)).to(dev)
    U = torch.zeros((3 * tsk.mesh.nnodes, 1), dtype=torch.float64, device=dev)
    fem.solve_device(rho, 3.0, U)
    U.zero_()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("solve")
    c = fem.solve_device(rho, 3.0, U)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    st = fem.last_stats
    print(json.dumps({"probe": "solve", "size": list(size), "compliance": float(c[0]),
                      "iters": st.iters, "replacements": st.outer, "relres": st.relres}))


def _batch_maker(spec, iters, dev, autotune_on):
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    nx, ny, nz, vf, lf = spec

    def make():
        cfg = OC_Config(max_iters=iters, filter_type="spacial",
                        filter_radius=tools.SchedulerConfig.constant(target_value=1.5),
                        p=tools.SchedulerConfig.constant(target_value=3.0),
                        vol_frac=tools.SchedulerConfig.constant(target_value=vf),
                        move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                        E_min_coeff=1e-9, solver_option="cg_pyamg", precision="mixed",
                        solver_rtol=1e-8, autotune=autotune_on)
        return OC_Optimizer(cfg, toy_problem.cantilever(nx, ny, nz, load_frac=lf), device=dev)
    return make


def batch_run(n_designs=256, iters=40, workers=16, check=4, autotune_on=True):
    """The batched-designs configuration: the first `n_designs` cantilevers of
    the seeded 256-design set (nx ~ U{16..64}, ny, nz ~ U{8..32}, vf ~
    U(0.2, 0.5), load position ~ U(0, 1)), `iters` mixed OC iterations each,
    stepped concurrently (one stream per design, `workers` host threads,
    launch shapes from the autotuner); then `check` designs (spread over the
    set) re-run alone and compared bit for bit."""
    import numpy as np
    import torch
    from sktopt_gb300.core import BatchedDesigns, autotune
    from sktopt_gb300.mesh import toy_problem
    dev = torch.device("cuda", torch.cuda.current_device())
    specs = toy_problem.batched_cantilever_specs(256, seed=0)[:n_designs]
    makers = [_batch_maker(s, iters, dev, autotune_on) for s in specs]
    t0 = time.perf_counter()
    batch = BatchedDesigns(makers, n_workers=workers, device=dev)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch.step(iters)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    idx = sorted(set(int(i) for i in np.linspace(0, n_designs - 1, check)))
    same = []
    for i in idx:
        solo = makers[i]()
        solo.parameterize()
        solo.optimize_steps(iters)
        bo = batch.opts[i]
        same.append(bool(np.array_equal(bo._state.rho.cpu().numpy(),
                                        solo._state.rho.cpu().numpy()) and
                         list(bo.recorder.histories["compliance"]) ==
                         list(solo.recorder.histories["compliance"])))
        del solo
    out = {"workload": f"{n_designs} cantilevers of the seeded set, {iters} mixed OC "
                       f"iterations each, one stream per design, {workers} host threads",
           "design_iters_per_s": round(n_designs * iters / dt, 2), "seconds": round(dt, 2),
           "setup_s": round(t_setup, 2),
           "elements": int(sum(s[0] * s[1] * s[2] for s in specs)),
           "solo_bitwise_equal": {str(i): v for i, v in zip(idx, same)},
           "autotune": autotune.cache() if autotune_on else None}
    del batch
    torch.cuda.empty_cache()
    return out


def batch_result(world):
    """The batched-designs key of the bench line.  One rank: `batch_run` on
    all 256 designs.  N ranks: the designs sharded by cost over the ranks
    (`run_sharded`, one gather), each rank stepping its share concurrently;
    the job's design-iterations per second from the slowest rank."""
    if world <= 1:
        return batch_run()
    import torch
    import torch.distributed as dist
    from sktopt_gb300.core import run_sharded
    from sktopt_gb300.mesh import toy_problem
    rank = dist.get_rank()
    dev = torch.device("cuda", torch.cuda.current_device())
    specs = toy_problem.batched_cantilever_specs(256, seed=0)
    iters = 40
    makers = [_batch_maker(s, iters, dev, True) for s in specs]
    costs = [float(s[0] * s[1] * s[2]) for s in specs]
    replica_barrier()
    t0 = time.perf_counter()
    res = run_sharded(makers, costs, iters, rank=rank, world_size=world, n_workers=16)
    torch.cuda.synchronize()
    t = replica_max(time.perf_counter() - t0)
    out = {"workload": f"256 cantilevers of the seeded set, {iters} mixed OC iterations "
                       f"each, sharded by cost over {world} ranks",
           "design_iters_per_s": round(256 * iters / t, 2), "seconds": round(t, 2)}
    if rank == 0:
        out["designs_gathered"] = len(res)
    return out


def probe_batch(n_designs, iters, workers):
    """Batched uneven designs: `n_designs` of the set, `iters` mixed OC
    iterations each, concurrent (with the autotuner) against sequential."""
    import torch
    out = {"probe": "batch", "concurrent": batch_run(n_designs, iters, workers, check=2)}
    out["sequential"] = batch_run(n_designs, iters, 1, check=0, autotune_on=True)
    torch.cuda.empty_cache()
    print(json.dumps(out))


def probe_autograd(size=(100, 50, 50)):
    """Differentiation workload: compliance(rho) and thermal compliance(rho)
    as autograd Functions on a 100x50x50 hex grid, rho ~ U(0.1, 1) (seed 0),
    p = 3; elasticity with the cantilever supports, heat with k0 = 1,
    kmin = 1e-3, unit source and T = 0 on a centred 10x10 patch of z = 0.
    Times forward + backward (FP64 and mixed solves) and checks the gradient
    against central differences (step 1e-6) along two random directions."""
    import numpy as np
    import torch
    from sktopt_gb300.core.autograd import compliance
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.fea.solver_heat import FEM_SimpLinearHeatConduction
    from sktopt_gb300.mesh import toy_problem
    dev = torch.device("cuda", 0)
    out = {"probe": "autograd", "size": list(size)}
    for phys in ("elasticity", "heat"):
        tsk = toy_problem.cantilever(*size) if phys == "elasticity" else \
            toy_problem.heat_box(*size, patch=10)
        g = np.random.default_rng(0)
        rho = torch.from_numpy(0.1 + 0.9 * g.random(tsk.mesh.nelements)).to(dev)
        for prec in ("fp64", "mixed"):
            cfg = LinearSolverConfig(solver="cg_pyamg", rtol=1e-10, precision=prec)
            fem = FEM_SimpLinearElasticity(tsk, 1e-9, solver_config=cfg, device=dev) \
                if phys == "elasticity" else \
                FEM_SimpLinearHeatConduction(tsk, 1e-3, solver_config=cfg, device=dev)
            x = rho.clone().requires_grad_(True)
            compliance(x, fem, 3.0).backward()          # warm-up (engine, hierarchy)
            x = rho.clone().requires_grad_(True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            C = compliance(x, fem, 3.0)
            C.backward()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            rec = {"forward_backward_ms": round(dt * 1e3, 1), "compliance": float(C.detach())}
            if prec == "fp64":
                h = 1e-6
                errs = []
                for k in range(2):
                    d = torch.from_numpy(np.random.default_rng(10 + k).standard_normal(
                        rho.numel())).to(dev)
                    with torch.no_grad():
                        cp = float(compliance(rho + h * d, fem, 3.0))
                        cm = float(compliance(rho - h * d, fem, 3.0))
                    fd = (cp - cm) / (2 * h)
                    ad = float(torch.dot(x.grad, d))
                    errs.append(abs(fd - ad) / abs(fd))
                rec["grad_vs_central_difference_rel"] = [float(f"{e:.2e}") for e in errs]
            out[f"{phys}_{prec}"] = rec
            del fem
            torch.cuda.empty_cache()
    return out


def probe_heat_robin(size=(200, 200, 25), small=(40, 40, 5), iters=5, warmup=3):
    """Heat objectives with Robin terms: the plate of sktopt's heat flow test
    (8 x 8 x 1, Robin h = 4e-5, T_env = 300 on two sides, T = 600 on a
    corner patch, k = 10) on a size[0] x size[1] x size[2] grid; OC, Gaussian
    filter of 1.5 cells, p = 3, volume fraction 0.4.  Times whole OC
    iterations (after warm-up) for the compliance, heat-exchange (with
    avg_temp_weight 0.5: three right-hand sides per solve) and averaged-
    temperature objectives, FP64 and mixed solves; and, as the CPU baseline,
    one oracle iteration (NumPy/SciPy, direct solves) against one GPU
    iteration at the reference test's own 40 x 40 x 5 size."""
    import dataclasses
    import numpy as np
    import torch
    from sktopt_gb300 import tools
    from sktopt_gb300.core import OC_Config, OC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    dev = torch.device("cuda", 0)
    out = {"probe": "heat_robin", "size": list(size)}

    def cfg_for(n, prec, n_it):
        r = 1.5 * 8.0 / n[0]
        return OC_Config(max_iters=n_it, filter_type="spacial",
                         filter_radius=tools.SchedulerConfig.constant(target_value=r),
                         p=tools.SchedulerConfig.constant(target_value=3.0),
                         vol_frac=tools.SchedulerConfig.constant(target_value=0.4),
                         move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                         E_min_coeff=1e-3, solver_option="cg_pyamg", precision=prec)

    for obj, w in (("compliance", 0.0), ("heat_exchange", 0.5), ("averaged_temp", 0.0)):
        # compliance with Robin data: the explicit Robin term turns dC positive
        # in low-density elements after a few steps at this size, and the OC
        # power law then gives NaN, as in the reference: time its first steps
        wu, it_n = (1, 2) if obj == "compliance" else (warmup, iters)
        for prec in ("fp64", "mixed"):
            tsk = toy_problem.heat_plate(*size, objective=obj, avg_temp_weight=w)
            opt = OC_Optimizer(cfg_for(size, prec, wu + it_n), tsk, device=dev)
            opt.parameterize()
            opt.optimize_steps(wu)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            opt.optimize_steps(it_n)
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / it_n
            st = opt.fem.last_stats
            out[f"{obj}_{prec}"] = {"ms_per_iter": round(dt * 1e3, 2),
                                    "objective": float(opt.recorder.histories[obj][-1]),
                                    "solve_iters": st.iters, "relres": st.relres}
            del opt
            torch.cuda.empty_cache()
    # reference-size comparison: oracle (CPU) vs GPU, one iteration each
    from oracle import optim as oopt
    from oracle import problems
    for obj in ("compliance", "heat_exchange"):
        m, pb, design, fixed, vol = problems.heat_plate(*small, objective=obj)
        r = 1.5 * 8.0 / small[0]
        filt = problems.gaussian_filter_for(m, design, r)
        ocfg = oopt.OracleConfig(max_iters=2, p=oopt.Sched("Constant", 3.0, 3.0),
                                 vol_frac=oopt.Sched("Constant", 0.4, 0.4),
                                 move_limit=oopt.Sched("Constant", 0.2, 0.2),
                                 filter_radius=oopt.Sched("Constant", r, r), E_min_coeff=1e-3)
        ref = oopt.OracleOptimizer(ocfg, pb, filt, design, fixed, vol)
        t0 = time.perf_counter()
        ref.step()
        t_cpu = time.perf_counter() - t0
        opt = OC_Optimizer(dataclasses.replace(cfg_for(small, "fp64", 5), max_iters=5),
                           toy_problem.heat_plate(*small, objective=obj), device=dev)
        opt.parameterize()
        opt.optimize_steps(2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        opt.optimize_steps(1)
        torch.cuda.synchronize()
        t_gpu = time.perf_counter() - t0
        out[f"{obj}_{'x'.join(map(str, small))}"] = {
            "gpu_fp64_ms": round(t_gpu * 1e3, 2),
            "cpu_baseline": {"ms": round(t_cpu * 1e3, 1), "kind": "port", "cores": 1,
                             "sample": "one oracle OC iteration"}}
    print(json.dumps(out))


def probe_multiload(size=(160, 80, 40), iters=2):
    """The multi-load unstructured configuration at full size: a 2 x 1 x 1
    box of size[0] x size[1] x size[2] cubes split into 6 P1 tetrahedra each
    (3,072,000 tets), interior nodes jittered by U(-0.2 h, 0.2 h) (seed 0),
    bottom face clamped, 4 point-load cases solved as one 4-column block
    right-hand side; log-space MOC, volume fraction 0.25, Helmholtz filter
    r = 0.04.  One untimed iteration, then `iters` timed ones, FP64 and
    mixed; the per-iteration compliance of the mixed path against FP64."""
    import torch
    from sktopt_gb300 import tools
    from sktopt_gb300.core import LogMOC_Config, LogMOC_Optimizer
    from sktopt_gb300.mesh import toy_problem
    dev = torch.device("cuda", 0)
    out = {"probe": "multiload", "size": list(size)}
    hist = {}
    for prec in ("fp64", "mixed"):
        t0 = time.perf_counter()
        tsk = toy_problem.multi_load_tet(*size, 2.0, 1.0, 1.0, jitter=0.2, seed=0)
        cfg = LogMOC_Config(max_iters=iters + 1, filter_type="helmholtz",
                            filter_radius=tools.SchedulerConfig.constant(target_value=0.04),
                            p=tools.SchedulerConfig.constant(target_value=3.0),
                            vol_frac=tools.SchedulerConfig.constant(target_value=0.25),
                            move_limit=tools.SchedulerConfig.constant(target_value=0.2),
                            E_min_coeff=1e-9, solver_option="cg_pyamg", precision=prec)
        opt = LogMOC_Optimizer(cfg, tsk, device=dev)
        opt.parameterize()
        opt.optimize_steps(1)
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        opt.optimize_steps(iters)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / iters
        st = opt.fem.last_stats
        hist[prec] = list(opt.recorder.histories["compliance"])
        out[prec] = {"ms_per_iter": round(dt * 1e3, 1), "setup_and_first_iter_s": round(setup, 1),
                     "n_elem": tsk.mesh.nelements, "n_dof": tsk.n_dof, "loads": tsk.n_tasks,
                     "solve_iters": st.iters, "relres": st.relres}
        del opt
        torch.cuda.empty_cache()
    out["compliance_rel_err_per_iter"] = [abs(a - b) / abs(b)
                                          for a, b in zip(hist["mixed"], hist["fp64"])]
    out["speedup_mixed_vs_fp64"] = round(out["fp64"]["ms_per_iter"] /
                                         out["mixed"]["ms_per_iter"], 2)
    return out


def probe_amg(size=(160, 80, 40)):
    """State solves of the multi-load unstructured configuration (the box of
    `size` cubes split into 6 jittered P1 tetrahedra each, bottom clamped, 4
    point-load cases as one block right-hand side) at a seeded random
    density, to 1e-8, FP64 and mixed, preconditioned by: the GPU-built
    smoothed-aggregation hierarchy (the logical grid dropped, as for a mesh
    read from a file), the geometric multigrid of the logical grid, and block
    Jacobi.  Reports the hierarchy set-up (engine creation), the operator
    update with the preconditioner refresh, and the solve."""
    import numpy as np
    import torch
    from sktopt_gb300.fea.solver_elastic import FEM_SimpLinearElasticity, LinearSolverConfig
    from sktopt_gb300.mesh import LinearElasticity, toy_problem
    from sktopt_gb300.mesh.grid import GridMesh
    dev = torch.device("cuda", 0)
    tsk = toy_problem.multi_load_tet(*size, 2.0, 1.0, 1.0, jitter=0.2, seed=0)
    m = tsk.mesh
    flat = GridMesh(m.p, m.t, "tet")
    dn = np.nonzero(m.node_ijk[2] == 0)[0]
    tsk_flat = LinearElasticity.from_nodes(flat, dn, "all", tsk.neumann_nodes, tsk.neumann_linear,
                                           np.arange(m.nelements), 1.0, 0.3)
    g = np.random.default_rng(0)
    rho = torch.from_numpy(0.05 + 0.95 * g.random(m.nelements)).to(dev)
    out = {"probe": "amg", "size": list(size), "n_elem": m.nelements, "n_dof": tsk.n_dof,
           "loads": tsk.n_tasks}
    for name, task, pre in (("amg", tsk_flat, "mg"), ("geometric_mg", tsk, "mg"),
                            ("block_jacobi", tsk_flat, "jacobi")):
        for prec in ("fp64", "mixed"):
            cfg = LinearSolverConfig(solver="cg_pyamg", rtol=1e-8, precision=prec, precond=pre,
                                     warm_start=False, maxiter=20000)
            fem = FEM_SimpLinearElasticity(task, 1e-9, solver_config=cfg, device=dev)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng = fem.engine
            torch.cuda.synchronize()
            t_setup = time.perf_counter() - t0
            U = torch.zeros((tsk.n_dof, tsk.n_tasks), dtype=torch.float64, device=dev)
            rec = {}
            for rep in range(2):
                U.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fem.build(rho, 3.0)
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                fem.solve_built(U)
                torch.cuda.synchronize()
                t2 = time.perf_counter()
                st = fem.last_stats
                rec = {"setup_s": round(t_setup, 3), "update_ms": round((t1 - t0) * 1e3, 2),
                       "solve_ms": round((t2 - t1) * 1e3, 2), "iters": st.iters,
                       "outer": st.outer, "relres": st.relres, "status": st.status,
                       "levels": eng.n_levels}
            out[f"{name}_{prec}"] = rec
            del fem, eng
            torch.cuda.empty_cache()
    print(json.dumps(out))


def main():
    args = parse()
    if args.probe == "spmv":
        probe_spmv(tuple(args.size))
        return
    if args.probe == "solve":
        probe_solve(tuple(args.size))
        return
    if args.probe == "batch":
        probe_batch(32, 6, 16)
        return
    if args.probe == "autograd":
        print(json.dumps(probe_autograd()))
        return
    if args.probe == "heat_robin":
        probe_heat_robin()
        return
    if args.probe == "multiload":
        print(json.dumps(probe_multiload()))
        return
    if args.probe == "amg":
        probe_amg(tuple(args.size) if args.size != list(SIZE) else (160, 80, 40))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
