"""Benchmark: converged velocity solves/s on the 640 x 80 (1 km, nσ = 4) synthetic channel.

One step = one Picard-converged velocity solve (update_velocities!) of the seeded 8 km channel refined
to 1 km (MISMIP+ bed with 20 m roughness, 300 m thickness with a 5 % perturbation, both drawn on the
8 km grid and interpolated), from the model's initial state (u = 0, default viscosity, the reference's
initial all-true wavelet coarse space) after the update_state! steps that precede the solve.  Every
step restores that state and solves it to ||b - A u|| / ||b|| < 1e-6 (maxiter_picard = 100; the
reference's other solver parameters).

  value    mixed precision (float32 operator / V-cycle, float64 residual and reductions), fields resident
           in HBM, device time per step from CUDA events on the solver's stream, L2 flushed between steps
  e2e      the same solve through the host C ABI (wavi_solve_velocities) from pinned host buffers, the
           host<->device copies inside the timed region
  fp64_gpu the reference algorithm in float64 on the GPU (the comparison the metric names)
  roofline the dominant kernel of the step, the persistent coarse CG (k_srcg_persistent<float>), timed
           with CUDA events around each launch in a host-driven solve of the same state; per CG
           iteration: algorithmic bytes / duration against the measured HBM peak (the kernel's working
           set, ~3 MB, is on chip or in L2: it is bound by the latency of its grid reduction and of the
           neighbour halo exchanges of its operator applications, not by HBM)
  roofline_stencil the fused operator kernel (float32) on a 4096 x 1024 grid (~190 MB per application,
           larger than L2), back-to-back launches timed with CUDA events: the HBM-bound stencil figure
  cpu_baseline the CPU oracle (the FP64 restatement of the reference) on a bounded sample

``--impl reference`` times only the CPU oracle on all host cores and prints its own line.
Under torchrun (N > 1) every rank solves its own replica (no collective); value is the sum.
``--profile solve|op`` runs one small untimed case for ncu (a host-driven solve of the workload capped
at ``--picard`` Picard iterations, or operator launches on the 4096 x 1024 grid) and prints nothing.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

TOL_PICARD = 1e-6
CHEB_STEPS = 3  # operator applications per iteration of the library's Chebyshev coarse solve
MAXITER_PICARD = 100
WORKLOAD = ("8 km channel refined to 640x80 @1km, nsigma=4, 5% thickness perturbation, Picard-converged solve "
            "from the initial state to rel. residual < 1e-6")
METRIC = "converged velocity solves/s (640x80 channel, mixed precision)"


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_state(pkg):
    """The state right before the timed solve (host numpy fields): the 8 km channel refined to 1 km —
    MISMIP+ bed with 20 m roughness and 300 m thickness with a 5 % perturbation, both drawn on the 8 km
    template grid (seeds 0 and 1) and interpolated — at the model's initial state (u = 0, default
    viscosity, the reference's initial all-true wavelet coarse space, UWavelets.jl:38), after the
    update_state! steps that precede the velocity solve."""
    from wavi_gb300 import synthetic
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve
    g, bed, p, sp, ic = synthetic.channel_c2(tol_picard=TOL_PICARD, maxiter_picard=MAXITER_PICARD)
    m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
    pre_solve(m)
    return m


def solve_field_names():
    from wavi_gb300.gpu import ALL_FIELDS
    return ALL_FIELDS


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in (self.out or "").splitlines():
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def time_device_solves(torch, solver, params, snapshot, steps, warmup, flush_bytes=256 << 20):
    """Per-step device time (CUDA events on the solver's stream) of resident solves from the snapshot."""
    names = solve_field_names()
    stream = torch.cuda.ExternalStream(solver.stream())
    dev = {}
    work = {}
    with torch.cuda.stream(stream):
        for k in names:
            a = snapshot[k]
            dev[k] = torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
            work[k] = dev[k].clone()
        flush = torch.empty(flush_bytes // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    times, stats = [], []
    for it in range(warmup + steps):
        with torch.cuda.stream(stream):
            for k in names:
                work[k].copy_(dev[k])
            flush.fill_(float(it))  # evict the previous step's working set from L2 (129 MB)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        st = solver.solve_device(params, work)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        if it >= warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
            stats.append(st)
    out = {k: work[k].cpu().numpy() for k in ("u", "v")}
    return times, stats, out


def time_host_solves(torch, solver, params, snapshot, steps, warmup):
    """e2e: the host C ABI from pinned buffers; H2D and D2H inside the timed region."""
    names = solve_field_names()
    stream = torch.cuda.ExternalStream(solver.stream())
    pinned = {}
    for k in names:
        a = np.asarray(snapshot[k])
        t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.uint8, pin_memory=True)
        pinned[k] = t
    views = {}
    for k in names:
        a = np.asarray(snapshot[k])
        views[k] = pinned[k].numpy().reshape(a.shape, order="F") if a.ndim > 1 else pinned[k].numpy()
    in_bytes = sum(np.asarray(snapshot[k]).nbytes for k in names if k not in (
        "shelf_strain_rate", "av_speed", "bed_speed", "tau_bed", "eta_av", "quad_f1", "beta_eff", "gu_residual",
        "gv_residual"))
    out_bytes = sum(np.asarray(snapshot[k]).nbytes for k in names if k not in (
        "h", "s", "dsdh", "grounded_fraction", "weertman_c", "accumulation", "basal_melt", "gu_h", "gu_s",
        "gu_grounded_fraction", "gv_h", "gv_s", "gv_grounded_fraction", "glen_b", "wu_mask", "wv_mask"))
    times = []
    for it in range(warmup + steps):
        for k in names:
            views[k][...] = snapshot[k]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
        solver.solve(params, views)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        if it >= warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
    return times, in_bytes, out_bytes


STENCIL_GRID = (4096, 1024)


def op_bytes(nx, ny, w):
    """Algorithmic bytes of one operator application: read x, write y, heta_h, dimp (Nh), heta_c (Nc),
    beta_m, h_m (N) in w-byte words plus the interior mask (N bytes)."""
    N = (nx + 1) * ny + nx * (ny + 1)
    Nh, Nc = nx * ny, (nx - 1) * (ny - 1)
    return w * (2.0 * N + 2.0 * Nh + Nc + 2.0 * N) + N


def cg_iteration_bytes(nx, ny, w):
    """Algorithmic bytes of one coarse-CG iteration of the persistent kernel: one operator application
    on the prolonged vector plus its write and the wavelet-mask read (N words, N bytes)."""
    N = (nx + 1) * ny + nx * (ny + 1)
    return op_bytes(nx, ny, w) + w * 2.0 * N + N


def stencil_solver(torch, device):
    from wavi_gb300 import synthetic
    from wavi_gb300.config import SolverParams
    from wavi_gb300.gpu import VelocitySolver
    nx, ny = STENCIL_GRID
    g = synthetic.Grid(nx=nx, ny=ny, nσ=4, dx=1000.0, dy=1000.0, u_iszero=["north"], v_iszero=["west", "east"])
    return VelocitySolver(g, SolverParams(), precision="mixed", device=device)


def op_roofline(torch, solver, n_launch=50, precision="mixed"):
    """Mean duration of the fused operator kernel: n_launch back-to-back launches timed with CUDA events
    on the solver's stream (wavi_time_operator_device), and its algorithmic bytes."""
    g = solver.grid
    N = (g.nx + 1) * g.ny + g.nx * (g.ny + 1)
    w = 4 if precision == "mixed" else 8
    x = torch.randn(N, dtype=torch.float32 if w == 4 else torch.float64, device="cuda")
    y = torch.zeros_like(x)
    torch.cuda.synchronize()
    solver.time_operator_device(x, y, precision, 5)  # warm-up
    dur = solver.time_operator_device(x, y, precision, n_launch)
    return op_bytes(g.nx, g.ny, w), dur


def coarse_roofline(torch, solver, params, snapshot):
    """The persistent coarse CG timed launch by launch (CUDA events around each launch) in a host-driven
    solve of the workload state: (seconds per CG iteration, CG iterations, launches)."""
    names = solve_field_names()
    dev = {k: torch.from_numpy(np.ascontiguousarray(np.asarray(snapshot[k]).ravel(order="F"))).cuda() for k in names}
    st = solver.solve_device(params, dev)
    return st["coarse_ms"] / 1e3 / max(1, st["coarse_cg_iterations"]), st["coarse_cg_iterations"], st["coarse_launches"]


def aggregate_ranks(torch, dist, world, local_seconds, steps, device):
    """Whole-job throughput: max over ranks of the timed-region time, every rank's steps counted."""
    total = float(local_seconds)
    if world > 1:
        tt = torch.tensor([total], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total = float(tt.item())
    return world * steps / total, total


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def ncu_traffic(fn, key):
    """A `key: value` figure (dram bytes) from a committed ncu summary under profiles/, if present."""
    try:
        for ln in open(os.path.join(ROOT, "profiles", fn)):
            if ln.startswith(key + ":"):
                return float(ln.split(":", 1)[1].strip())
    except (OSError, ValueError):
        pass
    return None


# ---------------------------------------------------------------------------------------------------
# CPU oracle (the reference restated in C++), bounded sample on host threads
# ---------------------------------------------------------------------------------------------------
def cpu_sample(threads, picard_iters_sample=1, state=None):
    """Each thread builds the same perturbed-thickness state in its own oracle model and runs
    ``picard_iters_sample`` Picard iterations of the solve.  Returns (seconds per Picard iteration per
    thread, threads, picard count of the full solve measured by the oracle's warm-state run length)."""
    oracle = __graft_entry__.load_oracle()
    pkg = __graft_entry__.load_package()
    from wavi_gb300 import synthetic
    import ctypes as C

    def make():
        g, bed, p, sp, ic = synthetic.channel_c2(tol_picard=TOL_PICARD, maxiter_picard=MAXITER_PICARD)
        om = oracle.build_model(g, bed, p, sp, ic)
        return om, g, p, sp

    results = [None] * threads

    def work(i):
        om, g, p, sp = make()
        om.pre_solve()
        sp1 = type(sp)(**{**sp.__dict__, "maxiter_picard": picard_iters_sample})
        oracle.lib().oracle_set_params(om.h, C.byref(p.to_c()), C.byref(sp1.to_c()), 0.0)
        t0 = time.perf_counter()
        om.update_velocities()
        results[i] = (time.perf_counter() - t0) / picard_iters_sample

    ths = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    wall = time.perf_counter() - t0
    return results, wall


# Picard iterations of the timed solve (same algorithm and state on every arm; the FP64 GPU arm reports
# its own count, which the CPU extrapolation uses when available).
PICARD_FALLBACK = 40


def reference_arm(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    per_iter = []
    for it in range(args.warmup + args.steps):
        res, wall = cpu_sample(threads)
        if it >= args.warmup:
            per_iter.append(statistics.median(res))
    sec_per_iter = statistics.median(per_iter)
    solves_per_s = threads / (sec_per_iter * PICARD_FALLBACK)
    line = {
        "impl": "reference", "metric": METRIC, "value": solves_per_s, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec_per_iter * PICARD_FALLBACK,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": f"{threads} host threads, independent replicas"},
        "cpu_baseline": {"value": solves_per_s, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"first Picard iteration of the solve per thread ({threads} threads), "
                                   f"extrapolated x{PICARD_FALLBACK} Picard iterations"},
        "e2e": {"value": solves_per_s, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def gpu_arm(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    pkg = __graft_entry__.load_package()
    from wavi_gb300 import build
    build.build_library()
    from wavi_gb300.gpu import VelocitySolver
    from wavi_gb300.model import release_solver

    m = build_state(pkg)
    snapshot = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    release_solver(m)
    g, p, sp = m.grid, m.params, m.solver_params

    mixed = VelocitySolver(g, sp, precision="mixed", device=local, coarse_solver=args.coarse_solver,
                           cheb_steps=args.cheb_steps)
    fp64 = VelocitySolver(g, sp, precision="fp64", device=local)

    # float64 reference algorithm on the GPU
    t64, st64, out64 = time_device_solves(torch, fp64, p, snapshot, max(1, args.steps // 2), 1)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        tmix, stmix, outmix = time_device_solves(torch, mixed, p, snapshot, args.steps, args.warmup)
    torch.cuda.synchronize()
    clocks = clk.summary()
    # max over ranks of the timed-region time
    value, total = aggregate_ranks(torch, dist if world > 1 else None, world, sum(tmix), args.steps, "cuda")

    te2e, hb, db = time_host_solves(torch, mixed, p, snapshot, args.steps, max(1, args.warmup // 2))
    e2e_value = world * len(te2e) / sum(te2e)

    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    # dominant kernel: the persistent coarse CG, per CG iteration
    prof = VelocitySolver(g, sp, precision="mixed", device=local, use_graphs=False, coarse_solver=args.coarse_solver,
                          cheb_steps=args.cheb_steps)
    sec_it, cg_its, cg_launches = coarse_roofline(torch, prof, p, snapshot)
    prof.close()
    # operator applications per CG iteration: 1, or CHEB_STEPS with the Chebyshev preconditioner (the
    # library's default mixed coarse solver on full ice masks: CHEB_STEPS - 1 in the preconditioner)
    apps = (args.cheb_steps or CHEB_STEPS) if stmix[-1]["coarse_solver"] in ("srcg_chebyshev", "pipelined_chebyshev") else 1
    cg_bytes = apps * cg_iteration_bytes(g.nx, g.ny, 4)
    cg_achieved = cg_bytes / sec_it / 1e9
    # the fused operator on a grid larger than L2
    big = stencil_solver(torch, local)
    alg_bytes, dur = op_roofline(torch, big)
    big.close()
    achieved = alg_bytes / dur / 1e9

    err = np.sqrt(np.sum((outmix["u"] - out64["u"]) ** 2) + np.sum((outmix["v"] - out64["v"]) ** 2)) / \
        np.sqrt(np.sum(out64["u"] ** 2) + np.sum(out64["v"] ** 2))
    fp64_value = world * len(t64) / sum(t64)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        res, wall = cpu_sample(threads)
        sec = statistics.median(res)
        picard = int(statistics.median([s["picard_iterations"] for s in st64]))
        cpu = {"value": threads / (sec * picard), "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"first Picard iteration of this solve on each of {threads} threads "
                         f"({sec:.2f} s each), extrapolated x{picard} Picard iterations (the FP64 GPU count)"}

    launches = sum(s["kernel_launches"] for s in stmix)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nx": g.nx, "ny": g.ny, "nsigma": g.nσ, "dx_m": g.dx,
                   "unknowns": int(m.u_inner.sum() + m.v_inner.sum()), "tol_picard": TOL_PICARD,
                   "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(hb), "d2h_bytes_per_step": int(db)},
        "gpu_launches": int(launches),
        "fp64_gpu": {"value": fp64_value, "unit": "solves/s", "ms_per_step": 1e3 * sum(t64) / len(t64),
                     "picard_iterations": st64[-1]["picard_iterations"],
                     "coarse_cg_iterations": st64[-1]["coarse_cg_iterations"]},
        "mixed_over_fp64": value / fp64_value if fp64_value else None,
        "rel_err_mixed_vs_fp64": float(err),
        "solve": {k: stmix[-1][k] for k in ("picard_iterations", "coarse_cg_iterations", "op_applications",
                                             "rel_residual", "kernel_launches", "host_syncs", "status_name")},
        "roofline": {"bound": "hbm", "achieved": cg_achieved, "peak": peak, "unit": "GB/s",
                     "frac": cg_achieved / peak,
                     "traffic": ncu_traffic("coarse_cg_c2.md", "traffic_bytes_per_cg_iteration"),
                     "kernel": "k_srcg_persistent<float> (coarse CG, one launch per V-cycle, 640x80)",
                     "per": "CG iteration", "alg_bytes_per_iteration": cg_bytes, "us_per_iteration": sec_it * 1e6,
                     "operator_applications_per_iteration": apps, "coarse_solver": stmix[-1]["coarse_solver"],
                     "cg_iterations": cg_its, "launches": cg_launches, "peak_source": "measured" if peaks else "fallback",
                     "note": "on-chip/L2-resident working set; bound by the latency of one grid reduction and "
                             "operator_applications_per_iteration neighbour halo exchanges per iteration"},
        "roofline_stencil": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak,
                             "traffic": ncu_traffic("op_kernel_4096x1024.md", "traffic_bytes_per_launch"),
                             "kernel": "k_op<float> (fused operator, %dx%d)" % STENCIL_GRID,
                             "alg_bytes_per_launch": alg_bytes, "avg_launch_us": dur * 1e6,
                             "peak_source": "measured" if peaks else "fallback"},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    mixed.close()
    fp64.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


ENSEMBLE_WORKLOAD = ("256 ragged channel domains at 2 km (nx U{64..512}, ny U{16..128}, seed 6), nsigma=4, "
                     "per-member roughness, thickness noise, C log-U(3e3,3e4), accumulation U(0.1,0.5); each solved "
                     "Picard-converged to rel. residual < 1e-6 from its initial state")


def ensemble_arm(args):
    """The batched ensemble: every member solved at once through wavi_ensemble_solve_device (mixed
    precision, launch configuration from the autotuner), against looping the single-domain FP64 GPU
    solve over every 8th member.  Host wall clock around each whole-ensemble solve (the call returns
    when every member is done); member fields restored on the device before each step, untimed."""
    import torch
    __graft_entry__.load_package()
    from wavi_gb300 import build, synthetic
    build.build_library()
    from wavi_gb300.ensemble import EnsembleSolver, autotune
    from wavi_gb300.gpu import VelocitySolver
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve, release_solver
    members = synthetic.ensemble_members(args.members)
    grids, params, sps, snaps = [], [], [], []
    for (g, bed, p, sp, ic) in members:
        m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
        pre_solve(m)
        grids.append(g)
        params.append(m.params)
        sps.append(sp)
        snaps.append({k: np.array(v, copy=True) for k, v in m.fields.items()})
        release_solver(m)
    names = solve_field_names()
    dev = [{k: torch.from_numpy(np.ascontiguousarray(np.asarray(s[k]).ravel(order="F"))).cuda() for k in names}
           for s in snaps]

    def make_tensors():
        return [{k: t.clone() for k, t in d.items()} for d in dev]

    n = len(grids)
    if args.no_tune:
        best, timings = dict(concurrency=16, coarse_kernel="auto"), []
    else:
        best, timings = autotune(grids, sps, params, make_tensors, sync=torch.cuda.synchronize)
    ens = EnsembleSolver(grids, sps, precision="mixed", **best)
    times, stats = [], None
    for it in range(args.warmup + args.steps):
        work = make_tensors()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stats = ens.solve_device(params, work)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    ens.close()
    value = n * len(times) / sum(times)
    # looping the single-domain FP64 GPU solve, on every 8th member
    subset = list(range(0, n, 8))
    t64, errs = 0.0, []
    for k in subset:
        s = VelocitySolver(grids[k], sps[k], precision="fp64")
        s.solve_device(params[k], {kk: t.clone() for kk, t in dev[k].items()})  # graph instantiation
        w = {kk: t.clone() for kk, t in dev[k].items()}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.solve_device(params[k], w)
        t64 += time.perf_counter() - t0
        s.close()
        if stats[k]["status"] == 0:  # a velocity error means something only between two converged solves
            du = torch.cat([work[k]["u"] - w["u"], work[k]["v"] - w["v"]])
            errs.append(float(torch.linalg.norm(du) / torch.linalg.norm(torch.cat([w["u"], w["v"]]))))
    fp64_value = len(subset) / t64
    conv = sum(1 for st in stats if st["status"] == 0)
    line = {
        "metric": "converged velocity solves/s (ragged 256-member ensemble, mixed precision)", "value": value,
        "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": ENSEMBLE_WORKLOAD, "members": n, "h_cells": int(sum(g.nx * g.ny for g in grids)),
                   "launch": best, "timing": "host wall clock around each whole-ensemble solve"},
        "fp64_loop": {"value": fp64_value, "unit": "solves/s", "members_timed": len(subset)},
        "ensemble_over_fp64_loop": value / fp64_value,
        "rel_err_vs_fp64_max": max(errs) if errs else None,
        "rel_err_vs_fp64_median": float(np.median(errs)) if errs else None, "rel_err_members": len(errs),
        "members_converged": conv,
        "note": "members that do not reach 1e-6 within maxiter_picard = 100 stall the same way in FP64 (the "
                "reference algorithm's one V-cycle per Picard iteration); they count as solves at maxiter",
        "picard_iterations_mean": float(np.mean([st["picard_iterations"] for st in stats])),
        "autotune": [{"seconds": t, **c} for t, c in timings],
    }
    print(json.dumps(line), flush=True)
    return 0


def adjoint_arm(args):
    """The adjoint workload on the 640 x 80 channel: J = ½ Σ (|u| − u_obs)² with u_obs from a forward
    solve at log C + 0.1 z (z ~ N(0, 1) per cell, seed 4) plus 2 % Gaussian noise (seed 5); the gradient
    with respect to per-cell log C and log A at the unperturbed state by wavi_adjoint_device; checked by
    the dot-product test against wavi_tangent_device and by central differences of tightly converged
    forward solves along 20 seeded directions (seeds 100-119), with a step sweep on the first."""
    import dataclasses
    import torch
    __graft_entry__.load_package()
    from wavi_gb300 import build, synthetic
    build.build_library()
    from wavi_gb300.gpu import VelocitySolver
    from wavi_gb300.misfit import misfit, misfit_gradient, speed
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve, release_solver
    g, bed, p, sp, ic = synthetic.channel_c2(tol_picard=1e-11, maxiter_picard=600)
    solver = VelocitySolver(g, sp, precision="fp64")
    c0 = np.full((g.nx, g.ny), float(p.weertman_c))
    a0 = np.full((g.nx, g.ny), float(p.glen_a_ref))
    state = {}

    def solve(dlogc=None, dloga=None):
        p2 = dataclasses.replace(p, weertman_c=np.asfortranarray(c0 * np.exp(dlogc if dlogc is not None else 0.0)),
                                 glen_a_ref=np.asfortranarray(a0 * np.exp(dloga if dloga is not None else 0.0)))
        m = Model(g, bed, p2, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
        pre_solve(m)
        f = {k: np.array(v, copy=True, order="F") for k, v in m.fields.items()}
        release_solver(m)
        st = solver.solve(m.params, f)
        state["m"], state["params"] = m, m.params
        return f, st

    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))).cuda()
    z = np.random.default_rng(4).standard_normal((g.nx, g.ny))
    f_true, _ = solve(0.1 * z)
    m = state["m"]
    masks = (m.u_mask, m.v_mask, m.h_mask)
    s_true, _, _ = speed(f_true["u"], f_true["v"], *masks)
    s_obs = s_true * (1.0 + 0.02 * np.random.default_rng(5).standard_normal(s_true.shape))
    f0, st0 = solve()
    params = state["params"]
    gu, gv = misfit_gradient(f0["u"], f0["v"], *masks, s_obs)
    gc = torch.zeros(g.nx * g.ny, dtype=torch.float64, device="cuda")
    ga = torch.zeros_like(gc)
    times, ast = [], None
    for it in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ast = solver.adjoint_device(params, dev(gu), dev(gv), gc, ga, tol=1e-12, maxiter=400)
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    grad_c = gc.cpu().numpy().reshape((g.nx, g.ny), order="F")
    grad_a = ga.cpu().numpy().reshape((g.nx, g.ny), order="F")
    # dot-product test
    rng = np.random.default_rng(6)
    vc, va = rng.standard_normal((g.nx, g.ny)), rng.standard_normal((g.nx, g.ny))
    wu = np.where(m.u_inner, rng.standard_normal((g.nx + 1, g.ny)), 0.0)
    wv = np.where(m.v_inner, rng.standard_normal((g.nx, g.ny + 1)), 0.0)
    du = torch.zeros((g.nx + 1) * g.ny, dtype=torch.float64, device="cuda")
    dv = torch.zeros(g.nx * (g.ny + 1), dtype=torch.float64, device="cuda")
    tst = solver.tangent_device(params, dev(vc), dev(va), du, dv, tol=1e-12, maxiter=400)
    gc2, ga2 = torch.zeros_like(gc), torch.zeros_like(ga)
    solver.adjoint_device(params, dev(wu), dev(wv), gc2, ga2, tol=1e-12, maxiter=400)
    lhs = float(torch.dot(du, dev(wu)) + torch.dot(dv, dev(wv)))
    rhs = float(torch.dot(gc2, dev(vc)) + torch.dot(ga2, dev(va)))
    # central differences
    def fd(vc, va, h):
        fp, _ = solve(h * vc, h * va)
        fm, _ = solve(-h * vc, -h * va)
        return (misfit(fp["u"], fp["v"], *masks, s_obs) - misfit(fm["u"], fm["v"], *masks, s_obs)) / (2 * h)
    dirs = [(np.random.default_rng(100 + k).standard_normal((g.nx, g.ny)),
             np.random.default_rng(200 + k).standard_normal((g.nx, g.ny))) for k in range(args.directions)]
    sweep = {}
    ad0 = float(np.sum(grad_c * dirs[0][0]) + np.sum(grad_a * dirs[0][1]))
    for h in (1e-2, 1e-3, 1e-4, 1e-5):
        sweep[h] = abs(fd(*dirs[0], h) - ad0) / abs(ad0)
    h_best = min(sweep, key=sweep.get)
    errs = []
    for k, (dc, da) in enumerate(dirs):
        ad = float(np.sum(grad_c * dc) + np.sum(grad_a * da))
        fdv = fd(dc, da, h_best)
        errs.append(abs(ad - fdv) / abs(fdv))
    line = {
        "metric": "adjoint gradients/s (d misfit / d(log C, log A), 640x80 channel, converged FP64 state)",
        "value": len(times) / sum(times), "unit": "gradients/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "J = 0.5 sum (|u| - u_obs)^2 on the 640x80 channel, u_obs from log C + 0.1 z "
                               "(seed 4) plus 2% noise (seed 5); forward solves to rel. residual < 1e-11",
                   "timing": "host wall clock around wavi_adjoint_device"},
        "forward": {"picard_iterations": st0["picard_iterations"], "rel_residual": st0["rel_residual"],
                    "status": st0["status_name"]},
        "adjoint": {"fgmres_iterations": ast["iterations"], "rel_residual": ast["rel_residual"]},
        "tangent": {"fgmres_iterations": tst["iterations"], "rel_residual": tst["rel_residual"]},
        "dot_test_rel_err": abs(lhs - rhs) / max(abs(lhs), abs(rhs)),
        "fd_step_sweep": {str(h): e for h, e in sweep.items()}, "fd_step": h_best,
        "fd_directions": len(errs), "fd_max_rel_err": max(errs), "fd_median_rel_err": float(np.median(errs)),
    }
    print(json.dumps(line), flush=True)
    solver.close()
    return 0


def profile_case(args):
    """One untimed case for ncu: the workload solved host-driven (every kernel a separate launch) and
    capped at --picard Picard iterations, or --op-launches operator launches on the stencil grid."""
    import torch
    __graft_entry__.load_package()
    from wavi_gb300 import build
    build.build_library()
    from wavi_gb300.config import SolverParams
    from wavi_gb300.gpu import VelocitySolver
    from wavi_gb300.model import release_solver
    if args.profile == "op":
        big = stencil_solver(torch, 0)
        op_roofline(torch, big, n_launch=args.op_launches)
        big.close()
        return 0
    m = build_state(None)
    snapshot = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    release_solver(m)
    sp = SolverParams(**{**m.solver_params.__dict__, "maxiter_picard": args.picard})
    s = VelocitySolver(m.grid, sp, precision=args.precision, use_graphs=False,
                       coarse_solver=args.coarse_solver if args.precision == "mixed" else "auto",
                       cheb_steps=args.cheb_steps)
    dev = {k: torch.from_numpy(np.ascontiguousarray(np.asarray(snapshot[k]).ravel(order="F"))).cuda()
           for k in solve_field_names()}
    st = s.solve_device(m.params, dev)
    torch.cuda.synchronize()
    s.close()
    print(json.dumps({"profile": args.profile, "stats": st}), file=sys.stderr)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-oracle baseline leg")
    ap.add_argument("--profile", choices=("solve", "op"), help="run one small untimed case for ncu and exit")
    ap.add_argument("--picard", type=int, default=1, help="--profile solve: Picard iterations")
    ap.add_argument("--precision", default="mixed", choices=("mixed", "fp64"), help="--profile solve: precision")
    ap.add_argument("--op-launches", type=int, default=3, help="--profile op: operator launches")
    ap.add_argument("--coarse-solver", default="auto",
                    choices=("auto", "cg", "srcg", "srcg_jacobi", "srcg_chebyshev", "pipelined_chebyshev"),
                    help="coarse solver of the mixed-precision solves (the FP64 solve keeps the reference's)")
    ap.add_argument("--cheb-steps", type=int, default=0,
                    help="Chebyshev steps of the Chebyshev coarse solvers (0: the library's default, 3; else odd)")
    ap.add_argument("--config", default="c2", choices=("c2", "c4", "c5"),
                    help="c2: the 640x80 solve (default); c4: the adjoint on 640x80; c5: the ragged 256-member ensemble")
    ap.add_argument("--directions", type=int, default=20, help="--config c4: finite-difference directions")
    ap.add_argument("--members", type=int, default=256, help="--config c5: ensemble members")
    ap.add_argument("--no-tune", action="store_true", help="--config c5: skip the autotuner")
    args = ap.parse_args()
    if args.profile:
        return profile_case(args)
    if args.config == "c4":
        return adjoint_arm(args)
    if args.config == "c5":
        # more hardware work queues than the default 8, so that concurrent members do not serialise
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
        return ensemble_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
