"""Benchmark: converged velocity solves/s on the 640 x 80 (1 km, nσ = 4) synthetic channel.

One step = one Picard-converged velocity solve (update_velocities!) of the seeded 8 km channel refined
to 1 km (MISMIP+ bed with 20 m roughness, 300 m thickness with a 5 % perturbation, both drawn on the
8 km grid and interpolated), from the model's initial state (u = 0, default viscosity, the reference's
initial all-true wavelet coarse space) after the update_state! steps that precede the solve.  Every
step restores that state and solves it to ||b - A u|| / ||b|| < 1e-6 (maxiter_picard = 100; the
reference's other solver parameters).

  value    mixed precision (float32 operator / V-cycle, float64 residual and reductions) with its default
           Picard iteration (Anderson-accelerated, wavi_picard_accel; --picard-accel) and coarse tolerance
           (adaptive, wavi_coarse_forcing; --coarse-forcing), fields resident in HBM, device time per step
           from CUDA events on the solver's stream, L2 flushed between steps
  mixed_plain / mixed_anderson  the same mixed solve with the reference's Picard iteration and coarse
           tolerance beside the accelerated defaults (or the reverse), with its error against the oracle
  e2e      the same solve through the host C ABI (wavi_solve_velocities) from pinned host buffers, the
           host<->device copies inside the timed region
  fp64_gpu the reference algorithm in float64 on the GPU (cg! coarse solve; the comparison the metric names)
  fp64_gpu_same_solver  float64 with the mixed solve's own coarse solver and Picard iteration:
           mixed_over_fp64_same_solver is the gain of precision alone, mixed_over_fp64 that of precision,
           coarse solver and Picard acceleration together
  rel_err_*_vs_oracle  relative velocity error of each GPU solve against the FP64 oracle's converged solve
           of the same state with the reference's algorithm and stopping rule
           (tests/golden/c2_oracle_solution.npz); *_vs_oracle_fixed_point against the oracle's solve of the
           same state to 1e-11 (tests/golden/c2_oracle_fixed_point.npz)
  mixed_fp64_coarse_sums / mixed_fp64_coarse_solve  the mixed solve with the coarse CG's sums, or the
           whole coarse CG, in FP64 (wavi_coarse_sums): what the default's float-float sums and FP32 coarse
           solve save
  roofline the dominant kernel of the step, the persistent coarse CG (k_srcg_persistent<float>), timed
           with CUDA events around each launch in a host-driven solve of the same state; per CG
           iteration: algorithmic bytes / duration against the measured HBM peak for scale.  Its working
           set (~3 MB) is on chip or in L2: it is bound by the latency of its grid reduction and of the
           neighbour halo exchanges of its operator applications, which latency_model splits from the
           Jacobi and Chebyshev coarse solves' per-iteration times
  roofline_stencil the fused operator kernel (float32, k_op_stream) on a 4096 x 1024 grid (~190 MB per
           application, larger than L2), back-to-back launches timed with CUDA events
  cpu_baseline the CPU oracle (the FP64 restatement of the reference) on a bounded sample: the first
           iterations of the solve on every host thread, scaled by the oracle's own profile
  other_configs compact lines of the 2560 x 320 domain (c3), the adjoint (c4) and the 256-member ensemble
           (c5), measured after the timed work (one GPU; --no-extras leaves them out; --config c3/c4/c5
           gives each in full)

``--impl reference`` times only the CPU oracle on all host cores (a whole converged solve per thread, all
threads at once, one step) and prints its own line.
Under torchrun (N > 1) every rank solves its own replica (no collective); value is the sum.
``--profile solve|op|relin`` runs one small untimed case for ncu (a host-driven solve of the workload
capped at ``--picard`` Picard iterations — of the 2560 x 320 state with ``--config c3`` —, operator launches
on the 4096 x 1024 grid, or the relinearisation kernels on the 2560 x 320, nσ = 8 grid) and prints nothing.
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


def aggregate_ensemble(torch, dist, world, local_seconds, local_converged, steps, device):
    """Whole-job ensemble throughput when the members are split across ranks: every rank's converged
    members summed, over the slowest rank's time.  Returns (converged solves/s, seconds, converged)."""
    total, conv = float(local_seconds), int(local_converged)
    if world > 1:
        tt = torch.tensor([total], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        cc = torch.tensor([conv], dtype=torch.int64, device=device)
        dist.all_reduce(cc, op=dist.ReduceOp.SUM)
        total, conv = float(tt.item()), int(cc.item())
    return conv * steps / total, total, conv


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
# CPU oracle (the reference restated in C++) on the host threads
# ---------------------------------------------------------------------------------------------------
C2_FIXTURE = os.path.join(ROOT, "tests", "golden", "c2_oracle_solution.npz")


def other_iteration(args):
    """The Picard iteration and coarse tolerance of the comparison arm: the reference's (plain Picard,
    fixed tol_coarse) beside an accelerated headline, or the mixed defaults (Anderson, adaptive) beside a
    plain one.  Returns (key suffix, picard_accel, coarse_forcing)."""
    if args.picard_accel == "plain" and args.coarse_forcing == "fixed":
        return "anderson", "anderson", "adaptive"
    return "plain", "plain", "fixed"


def c2_fixture():
    """The FP64 oracle's converged solve of this workload (tests/golden/make_c2_solution.py), or None."""
    try:
        return np.load(C2_FIXTURE)
    except OSError:
        return None


def c2_fixed_point():
    """The FP64 oracle's solve of this workload to 1e-11 (tests/golden/make_c2_fixed_point.py), or None."""
    try:
        return np.load(os.path.join(os.path.dirname(C2_FIXTURE), "c2_oracle_fixed_point.npz"))
    except OSError:
        return None


def rel_err_uv(u, v, ref_u, ref_v):
    """||(u, v) - (u, v)_ref||_2 / ||(u, v)_ref||_2 over the whole u and v grids."""
    num = np.sqrt(np.sum((np.asarray(u).ravel() - np.asarray(ref_u).ravel(order="F")) ** 2) +
                  np.sum((np.asarray(v).ravel() - np.asarray(ref_v).ravel(order="F")) ** 2))
    return float(num / np.sqrt(np.sum(np.asarray(ref_u) ** 2) + np.sum(np.asarray(ref_v) ** 2)))


def c2_config(m):
    """The workload's config keys, the same on the GPU line and the reference line."""
    return {"workload": WORKLOAD, "nx": m.grid.nx, "ny": m.grid.ny, "nsigma": m.grid.nσ, "dx_m": m.grid.dx,
            "unknowns": int(m.u_inner.sum() + m.v_inner.sum()), "tol_picard": TOL_PICARD,
            "maxiter_picard": MAXITER_PICARD,
            "l2": "GPU: flushed between steps (256 MiB write); CPU: not applicable"}


def cpu_solves(threads, maxiter_picard):
    """Every host thread builds the workload's state in its own oracle model and solves it with
    ``maxiter_picard`` (all threads at once, each solve single-threaded).  Returns ([(seconds, picard
    iterations, final relative residual) per thread], wall seconds of the whole batch)."""
    oracle = __graft_entry__.load_oracle()
    __graft_entry__.load_package()
    from wavi_gb300 import synthetic

    results = [None] * threads

    def work(i):
        g, bed, p, sp, ic = synthetic.channel_c2(tol_picard=TOL_PICARD, maxiter_picard=maxiter_picard)
        om = oracle.build_model(g, bed, p, sp, ic)
        om.pre_solve()
        t0 = time.perf_counter()
        om.update_velocities()
        st = om.stats()
        results[i] = (time.perf_counter() - t0, st["picard_iterations"], st["rel_residual"])

    ths = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return results, time.perf_counter() - t0


def cpu_baseline_sample(threads):
    """The GPU line's cpu_baseline: a bounded sample — the first SAMPLE_PICARD Picard iterations of the solve
    on every host thread at once — scaled to a whole solve by the oracle's own single-thread profile of
    this workload (whole solve / those iterations, both timed when the committed fixture was made)."""
    ref = c2_fixture()
    if ref is None:
        return None
    k = int(ref["sample_picard"])
    scale = float(ref["oracle_seconds"]) / float(ref["sample_seconds"])
    res, wall = cpu_solves(threads, k)
    sec = statistics.median(r[0] for r in res) * scale
    return {"value": threads / sec, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"the first {k} Picard iterations of this solve on each of {threads} host threads at once "
                      f"(median {sec / scale:.2f} s), scaled by {scale:.1f} = whole solve / those iterations in the "
                      f"oracle's single-thread profile of this workload ({float(ref['oracle_seconds']):.0f} s / "
                      f"{float(ref['sample_seconds']):.1f} s)"}


def reference_arm(args):
    """The reference's CPU path on the host cores: the FP64 oracle (the C++ restatement of the reference's
    solve) solving the whole workload to convergence on every host thread at once, one single-threaded
    solve per thread.  One step: a whole solve takes minutes, so the requested steps and warm-up (the
    oracle has nothing to warm up) are not repeated; value = solves completed / wall time."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    pkg = __graft_entry__.load_package()
    from wavi_gb300.model import release_solver
    m = build_state(pkg)
    release_solver(m)
    threads = os.cpu_count() or 1
    res, wall = cpu_solves(threads, MAXITER_PICARD)
    per = statistics.median(r[0] for r in res)
    value = threads / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": 1, "warmup": 0, "requested_steps": args.steps, "requested_warmup": args.warmup,
        "ms_per_step": 1e3 * wall, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "config": c2_config(m),
        "parallelism": f"{threads} host threads, one whole single-threaded solve each",
        "single_thread": {"value": 1.0 / per, "unit": "solves/s", "seconds_per_solve": per},
        "solves": {"picard_iterations": sorted({r[1] for r in res}), "rel_residual_max": max(r[2] for r in res)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"one whole Picard-converged solve on each of {threads} host threads at once "
                                   f"(wall {wall:.1f} s; median single-thread solve {per:.1f} s)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
                           cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums,
                           viscosity=args.viscosity, picard_accel=args.picard_accel,
                           coarse_forcing=args.coarse_forcing)
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
    mixed_solver = stmix[-1]["coarse_solver"]

    # float64 with the mixed solve's own coarse solver: precision alone, the algorithm held fixed
    same = None
    if mixed_solver != "pipelined_chebyshev":
        fp64s = VelocitySolver(g, sp, precision="fp64", device=local, coarse_solver=mixed_solver,
                               cheb_steps=args.cheb_steps, picard_accel=stmix[-1]["picard_accel"],
                               coarse_forcing=stmix[-1]["coarse_forcing"])
        t64s, st64s, out64s = time_device_solves(torch, fp64s, p, snapshot, max(1, args.steps // 2), 1)
        fp64s.close()
        same = {"value": world * len(t64s) / sum(t64s), "unit": "solves/s", "ms_per_step": 1e3 * sum(t64s) / len(t64s),
                "coarse_solver": st64s[-1]["coarse_solver"], "picard_accel": st64s[-1]["picard_accel"],
                "coarse_forcing": st64s[-1]["coarse_forcing"],
                "picard_iterations": st64s[-1]["picard_iterations"],
                "coarse_cg_iterations": st64s[-1]["coarse_cg_iterations"], "status_name": st64s[-1]["status_name"]}

    # the mixed solve with its coarse CG's dot products, sums and scalars in FP64 (WAVI_SUMS_FP64) instead of
    # float-float grid sums over FP32 CTA sums
    sums64, outm64 = None, None
    if mixed_solver in ("srcg", "srcg_jacobi", "srcg_chebyshev") and args.coarse_sums == "default":
        try:
            m64 = VelocitySolver(g, sp, precision="mixed", device=local, coarse_solver=mixed_solver,
                                 cheb_steps=args.cheb_steps, coarse_sums="fp64", viscosity=args.viscosity)
        except Exception as e:  # the register-resident kernel may not fit (reported, not fatal)
            sums64 = {"unavailable": str(e)}
        else:
            tm64, stm64, outm64 = time_device_solves(torch, m64, p, snapshot, args.steps, 1)
            m64.close()
            sums64 = {"value": world * len(tm64) / sum(tm64), "unit": "solves/s",
                      "ms_per_step": 1e3 * sum(tm64) / len(tm64), "picard_iterations": stm64[-1]["picard_iterations"],
                      "coarse_cg_iterations": stm64[-1]["coarse_cg_iterations"],
                      "status_name": stm64[-1]["status_name"]}

    # the mixed solve with its whole coarse CG in FP64 (WAVI_SUMS_FP64_SOLVE)
    solve64, outc64 = None, None
    if mixed_solver != "pipelined_chebyshev" and args.coarse_sums == "default":
        try:
            mc64 = VelocitySolver(g, sp, precision="mixed", device=local, coarse_solver=mixed_solver,
                                  cheb_steps=args.cheb_steps, coarse_sums="fp64_solve", viscosity=args.viscosity)
        except Exception as e:  # reported, not fatal
            solve64 = {"unavailable": str(e)}
        else:
            tc64, stc64, outc64 = time_device_solves(torch, mc64, p, snapshot, max(1, args.steps // 2), 1)
            mc64.close()
            solve64 = {"value": world * len(tc64) / sum(tc64), "unit": "solves/s",
                       "ms_per_step": 1e3 * sum(tc64) / len(tc64), "picard_iterations": stc64[-1]["picard_iterations"],
                       "coarse_cg_iterations": stc64[-1]["coarse_cg_iterations"],
                       "status_name": stc64[-1]["status_name"]}

    # the mixed solve with the other Picard iteration and coarse tolerance (wavi_picard_accel,
    # wavi_coarse_forcing): the reference's beside the accelerated defaults, or the reverse
    other_accel, o_accel, o_forcing = other_iteration(args)
    mo = VelocitySolver(g, sp, precision="mixed", device=local, coarse_solver=args.coarse_solver,
                        cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums, viscosity=args.viscosity,
                        picard_accel=o_accel, coarse_forcing=o_forcing)
    tao, stao, outao = time_device_solves(torch, mo, p, snapshot, args.steps, 1)
    mo.close()
    accel_other = {"picard_accel": o_accel, "coarse_forcing": o_forcing, "value": world * len(tao) / sum(tao),
                   "unit": "solves/s",
                   "ms_per_step": 1e3 * sum(tao) / len(tao),
                   **{k: stao[-1][k] for k in ("picard_iterations", "coarse_cg_iterations", "anderson_steps",
                                                "rel_residual", "status_name")}}

    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    # dominant kernel: the persistent coarse CG, per CG iteration, timed launch by launch in host-driven solves;
    # with the Jacobi preconditioner (one operator application and one grid reduction per iteration) beside
    # it, the two per-iteration times split into a grid reduction and an operator application with its
    # neighbour exchange
    prof = VelocitySolver(g, sp, precision="mixed", device=local, use_graphs=False, coarse_solver=args.coarse_solver,
                          cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums,
                           viscosity=args.viscosity)
    sec_it, cg_its, cg_launches = coarse_roofline(torch, prof, p, snapshot)
    prof.close()
    apps = stmix[-1]["cheb_steps"] or 1  # operator applications per coarse-CG iteration (the library reports it)
    latency = None
    if mixed_solver == "srcg_chebyshev" and apps > 1:
        profj = VelocitySolver(g, sp, precision="mixed", device=local, use_graphs=False, coarse_solver="srcg_jacobi",
                               coarse_sums=args.coarse_sums, viscosity=args.viscosity)
        sec_j, cg_j, _ = coarse_roofline(torch, profj, p, snapshot)
        profj.close()
        e_op = (sec_it - sec_j) / (apps - 1)
        latency = {"us_per_iteration": sec_it * 1e6, "us_per_grid_reduction": (sec_j - e_op) * 1e6,
                   "us_per_operator_application": e_op * 1e6, "grid_reductions_per_iteration": 1,
                   "operator_applications_per_iteration": apps, "jacobi_us_per_iteration": sec_j * 1e6,
                   "jacobi_cg_iterations": cg_j,
                   "method": "Jacobi iteration = 1 operator application (prolongation, neighbour halo exchange, "
                             "stresses, restriction) + 1 grid reduction; Chebyshev iteration = %d applications + 1 "
                             "reduction: the difference of the measured per-iteration times gives the "
                             "application, the rest of the Jacobi iteration the reduction" % apps}
    cg_bytes = apps * cg_iteration_bytes(g.nx, g.ny, 4)
    cg_achieved = cg_bytes / sec_it / 1e9
    # the fused operator on a grid larger than L2
    big = stencil_solver(torch, local)
    alg_bytes, dur = op_roofline(torch, big)
    big.close()
    achieved = alg_bytes / dur / 1e9

    err = rel_err_uv(outmix["u"], outmix["v"], out64["u"].reshape((g.nx + 1, g.ny), order="F"),
                     out64["v"].reshape((g.nx, g.ny + 1), order="F"))
    ref = c2_fixture()
    errs_oracle = {}
    if ref is not None:
        errs_oracle["rel_err_mixed_vs_oracle"] = rel_err_uv(outmix["u"], outmix["v"], ref["u"], ref["v"])
        errs_oracle["rel_err_fp64_vs_oracle"] = rel_err_uv(out64["u"], out64["v"], ref["u"], ref["v"])
        if same is not None:
            errs_oracle["rel_err_fp64_same_solver_vs_oracle"] = rel_err_uv(out64s["u"], out64s["v"], ref["u"], ref["v"])
        if outm64 is not None:
            sums64["rel_err_vs_oracle"] = rel_err_uv(outm64["u"], outm64["v"], ref["u"], ref["v"])
        if outc64 is not None:
            solve64["rel_err_vs_oracle"] = rel_err_uv(outc64["u"], outc64["v"], ref["u"], ref["v"])
        accel_other["rel_err_vs_oracle"] = rel_err_uv(outao["u"], outao["v"], ref["u"], ref["v"])
        errs_oracle["oracle"] = {"picard_iterations": int(ref["picard_iterations"]),
                                 "coarse_cg_iterations": int(ref["coarse_cg_iterations"]),
                                 "rel_residual": float(ref["rel_residual"]),
                                 "source": "tests/golden/c2_oracle_solution.npz (FP64 oracle, same state)"}
    fpt = c2_fixed_point()
    if fpt is not None:
        # against the oracle's solve to 1e-11: the fixed point both Picard iterations converge to
        errs_oracle["rel_err_mixed_vs_oracle_fixed_point"] = rel_err_uv(outmix["u"], outmix["v"], fpt["u"], fpt["v"])
        errs_oracle["rel_err_fp64_vs_oracle_fixed_point"] = rel_err_uv(out64["u"], out64["v"], fpt["u"], fpt["v"])
        accel_other["rel_err_vs_oracle_fixed_point"] = rel_err_uv(outao["u"], outao["v"], fpt["u"], fpt["v"])
        errs_oracle["oracle_fixed_point"] = {"picard_iterations": int(fpt["picard_iterations"]),
                                             "rel_residual": float(fpt["rel_residual"]),
                                             "source": "tests/golden/c2_oracle_fixed_point.npz (FP64 oracle, same "
                                                       "state, solved to 1e-11)"}
    fp64_value = world * len(t64) / sum(t64)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(os.cpu_count() or 1)

    launches = sum(s["kernel_launches"] for s in stmix)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": c2_config(m), "parallelism": f"replicas x{world}",
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(hb), "d2h_bytes_per_step": int(db)},
        "gpu_launches": int(launches),
        "fp64_gpu": {"value": fp64_value, "unit": "solves/s", "ms_per_step": 1e3 * sum(t64) / len(t64),
                     "coarse_solver": st64[-1]["coarse_solver"],
                     "picard_iterations": st64[-1]["picard_iterations"],
                     "coarse_cg_iterations": st64[-1]["coarse_cg_iterations"]},
        "fp64_gpu_same_solver": same,
        "mixed_over_fp64": value / fp64_value if fp64_value else None,
        "mixed_over_fp64_same_solver": value / same["value"] if same else None,
        "picard_accel": stmix[-1]["picard_accel"], "coarse_forcing": stmix[-1]["coarse_forcing"],
        "mixed_" + other_accel: accel_other,
        "mixed_fp64_coarse_sums": sums64,
        "mixed_fp64_coarse_solve": solve64,
        "rel_err_mixed_vs_fp64": float(err),
        **errs_oracle,
        "solve": {k: stmix[-1][k] for k in ("picard_iterations", "coarse_cg_iterations", "op_applications",
                                             "rel_residual", "kernel_launches", "host_syncs", "status_name",
                                             "coarse_solver", "coarse_kernel", "cheb_steps", "anderson_steps",
                                             "picard_accel", "coarse_forcing")},
        "roofline": {"bound": "latency", "achieved": cg_achieved, "peak": peak, "unit": "GB/s",
                     "frac": cg_achieved / peak,
                     "traffic": ncu_traffic("coarse_cg_c2.md", "traffic_bytes_per_cg_iteration"),
                     "kernel": "k_srcg_persistent<float> (coarse CG, one launch per V-cycle, 640x80)",
                     "per": "CG iteration", "alg_bytes_per_iteration": cg_bytes, "us_per_iteration": sec_it * 1e6,
                     "operator_applications_per_iteration": apps, "coarse_solver": mixed_solver,
                     "cg_iterations": cg_its, "launches": cg_launches, "peak_source": "measured" if peaks else "fallback",
                     "latency_model": latency,
                     "note": "achieved = algorithmic bytes (L2-level: the working set, ~3 MB, stays on chip or in "
                             "L2) / time, against the HBM peak for scale only; traffic = ncu DRAM bytes per "
                             "iteration. The kernel is bound by the latency of its grid reduction and of the "
                             "neighbour halo exchanges of its operator applications (latency_model)"},
        "roofline_stencil": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak,
                             "traffic": ncu_traffic("op_kernel_4096x1024.md", "traffic_bytes_per_launch"),
                             "kernel": "k_op_stream<float> (fused operator, row streaming, %dx%d)" % STENCIL_GRID,
                             "alg_bytes_per_launch": alg_bytes, "avg_launch_us": dur * 1e6,
                             "peak_source": "measured" if peaks else "fallback"},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    mixed.close()
    fp64.close()
    if rank == 0 and world == 1 and not args.no_extras:
        line["other_configs"] = other_configs(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def other_configs(args):
    """Compact lines of the other configurations, measured in the same run after the timed 640 x 80 work (one GPU,
    rank 0): the large single domain (2560x320, nσ = 8), the 256-member ensemble (the autotuner's choice
    on GB300, one timed ensemble) and the adjoint (two finite-difference directions).  Each runs on its
    own; a failure is reported in its entry and leaves the 640 x 80 line intact."""
    import copy
    out = {}
    legs = (("c3", c3_arm, dict(steps=1, warmup=1),
             ("metric", "value", "unit", "ms_per_step", "solve", "picard_accel", "coarse_forcing", "mixed_anderson",
              "mixed_plain",
              "mixed_uncapped", "fp64_gpu", "mixed_over_fp64",
              "rel_err_mixed_vs_fp64", "roofline", "roofline_relin_fp64", "roofline_stencil", "coarse_cg_share")),
            ("c5", ensemble_arm, dict(steps=1, warmup=1, no_tune=True, members=256),
             ("metric", "value", "unit", "ms_per_step", "members_converged", "picard_accel", "coarse_forcing",
              "mixed_anderson",
              "mixed_plain", "all_members", "fp64_loop",
              "ensemble_over_fp64_loop", "rel_err_vs_fp64_max", "rel_err_vs_fp64_median", "picard_iterations_mean")),
            ("c4", adjoint_arm, dict(steps=2, warmup=1, directions=2),
             ("metric", "value", "unit", "ms_per_step", "forward", "adjoint", "adjoint_fp64_precond",
              "dot_test_rel_err", "fd_step",
              "fd_directions", "fd_max_rel_err")))
    for name, arm, kw, keys in legs:
        sub = copy.copy(args)
        for k, v in kw.items():
            setattr(sub, k, v)
        sub.quiet = True
        t0 = time.perf_counter()
        try:
            ln = arm(sub)
            entry = {k: ln[k] for k in keys if k in ln}
            if name == "c5":
                entry["launch"] = ln["config"]["launch"]
        except Exception as e:  # reported, not fatal: the 640 x 80 line stands on its own
            entry = {"error": f"{type(e).__name__}: {e}"}
        entry["wall_s"] = time.perf_counter() - t0
        out[name] = entry
    return out


C3_WORKLOAD = ("2560x320 channel @250m, nsigma=8, log-normal C (median 1e4, sigma_log 0.5, 20 km correlation, seed 3), "
               "A from a 243-268 K vertical temperature profile; Picard solve from the initial state, at most 30 "
               "iterations, to ||du||/||u|| <= 1e-6 and ||b - A u||/||b|| < 1e-6")


def relin_h_bytes(nx, ny, ns, mixed):
    """Algorithmic bytes of one launch of the relinearisation's h-grid kernel, per h cell: reads u and v
    (about one value of each per cell), the previous F2 and β, C·gf, h, ds/dh, and B and η on every σ level;
    writes η on every level and twelve 2-D fields (strain rate, speeds, β, τ_b, ηav, F1, F2, βeff, hηav, the
    two operator coefficients), plus their FP32 copies in mixed precision; one byte each of the h, c and
    u/v masks (the u/v mask about twice)."""
    Nh = nx * ny
    return Nh * (8.0 * (7 + 2 * ns) + 8.0 * (12 + ns) + (8.0 if mixed else 0.0) + 4.0)


def relin_uv_bytes(nx, ny):
    """Algorithmic bytes of one launch of the u/v-grid relinearisation kernel: per u or v point the h-grid
    βeff, grounded fraction and h ηav of its two neighbours (about one value of each per point), its own
    grounded fraction and thickness, βeff written, and the operator coefficients β_m, h_m (FP64 and FP32) and
    hη_c (per c cell), plus the masks."""
    N = (nx + 1) * ny + nx * (ny + 1)
    Nc = (nx - 1) * (ny - 1)
    return N * (8.0 * 5 + 8.0 * 3 + 4.0 * 2 + 1.0) + Nc * (8.0 + 4.0 + 8.0) + 2.0 * nx * ny


def c3_arm(args):
    """The large single domain (2560 x 320 at 250 m, nσ = 8): the mixed solve (value) and the FP64 reference
    algorithm once (fp64_gpu), both with the update-norm test of the configuration (picard_test = 1), and
    the HBM rooflines of the relinearisation kernel (~285 MB per launch, larger than L2) and of the fused
    operator on this grid, plus the persistent coarse CG's share."""
    import torch
    pkg = __graft_entry__.load_package()
    from wavi_gb300 import build, synthetic
    build.build_library()
    from wavi_gb300.gpu import VelocitySolver
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve, release_solver
    g, bed, p, sp, ic = synthetic.channel_c3(tol_picard=1e-6, maxiter_picard=30)
    m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
    pre_solve(m)
    snapshot = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    release_solver(m)
    p = m.params
    mixed = VelocitySolver(g, sp, precision="mixed", picard_test=1, coarse_solver=args.coarse_solver,
                           cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums,
                           viscosity=args.viscosity, picard_accel=args.picard_accel,
                           coarse_forcing=args.coarse_forcing)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        tmix, stmix, outmix = time_device_solves(torch, mixed, p, snapshot, args.steps, args.warmup)
    clocks = clk.summary()
    value = len(tmix) / sum(tmix)
    # the same mixed solve without the 30-iteration cap: where (if at all) it meets the configuration's test
    from dataclasses import replace as _replace
    long_sp = _replace(sp, maxiter_picard=200)
    mlong = VelocitySolver(g, long_sp, precision="mixed", picard_test=1, coarse_solver=args.coarse_solver,
                           cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums, viscosity=args.viscosity,
                           picard_accel="plain", coarse_forcing="fixed")
    tl, stl, _ = time_device_solves(torch, mlong, p, snapshot, 1, 0)
    mlong.close()
    # the mixed solve with the other Picard iteration and coarse tolerance, at the configuration's cap
    other_accel, o_accel, o_forcing = other_iteration(args)
    mo = VelocitySolver(g, sp, precision="mixed", picard_test=1, coarse_solver=args.coarse_solver,
                        cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums, viscosity=args.viscosity,
                        picard_accel=o_accel, coarse_forcing=o_forcing)
    tao, stao, outao = time_device_solves(torch, mo, p, snapshot, 1, 1)
    mo.close()
    fp64 = VelocitySolver(g, sp, precision="fp64", picard_test=1)
    t64, st64, out64 = time_device_solves(torch, fp64, p, snapshot, 1, 1)
    err = rel_err_uv(outmix["u"], outmix["v"], out64["u"].reshape((g.nx + 1, g.ny), order="F"),
                     out64["v"].reshape((g.nx, g.ny + 1), order="F"))
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    src = "measured" if peaks else "fallback"
    # relinearisation kernels on the solved state (each launch > L2 at nσ = 8)
    rel = {}
    for name, s_ in (("mixed", mixed), ("fp64", fp64)):
        th, tuv = s_.time_relinearise_device(20)
        bh = relin_h_bytes(g.nx, g.ny, g.nσ, name == "mixed")
        rel[name] = {"kernel": "k_relin_h<%s>" % ("float" if name == "mixed" else "double"), "bound": "hbm",
                     "alg_bytes_per_launch": bh, "avg_launch_us": th * 1e6, "achieved": bh / th / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": bh / th / 1e9 / peak, "peak_source": src,
                     "uv_kernel": {"kernel": "k_relin_uv", "alg_bytes_per_launch": relin_uv_bytes(g.nx, g.ny),
                                   "avg_launch_us": tuv * 1e6,
                                   "achieved": relin_uv_bytes(g.nx, g.ny) / tuv / 1e9}}
    # the fused FP32 operator on this grid: back to back (its ~38 MB stay in L2), and with L2 flushed
    # (a 256 MiB write) before each launch
    N = (g.nx + 1) * g.ny + g.nx * (g.ny + 1)
    x = torch.randn(N, dtype=torch.float32, device="cuda")
    y = torch.zeros_like(x)
    ob = op_bytes(g.nx, g.ny, 4)
    warm = mixed.time_operator_device(x, y, "mixed", 50)
    stream = torch.cuda.ExternalStream(mixed.stream())
    flush = torch.empty((256 << 20) // 4, dtype=torch.float32, device="cuda")
    cold = []
    for k in range(20):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        cold.append(mixed.time_operator_device(x, y, "mixed", 1))
    cold_s = statistics.median(cold)
    # the persistent coarse CG's share of a host-driven mixed solve
    prof = VelocitySolver(g, sp, precision="mixed", use_graphs=False, picard_test=1, coarse_solver=args.coarse_solver,
                          cheb_steps=args.cheb_steps, coarse_sums=args.coarse_sums,
                           viscosity=args.viscosity)
    names = solve_field_names()
    dev = {k: torch.from_numpy(np.ascontiguousarray(np.asarray(snapshot[k]).ravel(order="F"))).cuda() for k in names}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    stp = prof.solve_device(p, dev)
    wall = time.perf_counter() - t0
    prof.close()
    mixed.close()
    fp64.close()
    last = stmix[-1]
    line = {
        "metric": "converged velocity solves/s (2560x320 channel, nsigma=8, mixed precision)", "value": value,
        "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(tmix) / len(tmix), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": C3_WORKLOAD, "nx": g.nx, "ny": g.ny, "nsigma": g.nσ, "dx_m": g.dx,
                   "unknowns": int(m.u_inner.sum() + m.v_inner.sum()), "tol_picard": 1e-6, "maxiter_picard": 30,
                   "picard_test": "||du||/||u|| <= tol and ||b - A u||/||b|| < tol",
                   "l2": "flushed between steps (256 MiB write)"},
        "solve": {k: last[k] for k in ("status_name", "picard_iterations", "coarse_cg_iterations", "rel_residual",
                                       "rel_update", "coarse_solver", "kernel_launches", "anderson_steps")},
        "fp64_gpu": {"value": len(t64) / sum(t64), "unit": "solves/s", "ms_per_step": 1e3 * sum(t64) / len(t64),
                     **{k: st64[-1][k] for k in ("status_name", "picard_iterations", "coarse_cg_iterations",
                                                  "rel_residual", "rel_update", "coarse_solver")}},
        "mixed_uncapped": {"maxiter_picard": 200, "picard_accel": "plain", "coarse_forcing": "fixed",
                           "seconds": tl[0],
                           **{k: stl[-1][k] for k in ("status_name", "picard_iterations", "coarse_cg_iterations",
                                                      "rel_residual", "rel_update")}},
        "picard_accel": last["picard_accel"], "coarse_forcing": last["coarse_forcing"],
        "mixed_" + other_accel: {"picard_accel": o_accel, "coarse_forcing": o_forcing, "value": len(tao) / sum(tao),
                                 "unit": "solves/s",
                                 "ms_per_step": 1e3 * sum(tao) / len(tao),
                                 **{k: stao[-1][k] for k in ("status_name", "picard_iterations", "coarse_cg_iterations",
                                                              "anderson_steps", "rel_residual", "rel_update")}},
        "mixed_over_fp64": value / (len(t64) / sum(t64)),
        "rel_err_mixed_vs_fp64": err,
        "roofline": rel["mixed"],
        "roofline_relin_fp64": rel["fp64"],
        "roofline_stencil": {"kernel": "k_op_stream<float> (fused operator, row streaming, 2560x320)", "bound": "hbm",
                             "alg_bytes_per_launch": ob, "avg_launch_us_l2_flushed": cold_s * 1e6,
                             "achieved": ob / cold_s / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": ob / cold_s / 1e9 / peak, "peak_source": src,
                             "avg_launch_us_back_to_back": warm * 1e6, "achieved_back_to_back": ob / warm / 1e9,
                             "note": "back to back the operator's ~38 MB stay in L2 (129 MB)"},
        "coarse_cg_share": {"coarse_ms": stp["coarse_ms"], "solve_wall_ms": 1e3 * wall,
                            "coarse_cg_iterations": stp["coarse_cg_iterations"], "coarse_solver": stp["coarse_solver"],
                            "us_per_cg_iteration": 1e3 * stp["coarse_ms"] / max(1, stp["coarse_cg_iterations"])},
        "clocks": clocks,
    }
    if getattr(args, "quiet", False):
        return line
    print(json.dumps(line), flush=True)
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
    rank, world, local = dist_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    __graft_entry__.load_package()
    from wavi_gb300 import build, synthetic
    build.build_library()
    from wavi_gb300.ensemble import EnsembleSolver, autotune, shard_members
    from wavi_gb300.gpu import VelocitySolver
    from wavi_gb300.model import GPUParallelSpec, Model, pre_solve, release_solver
    all_members = synthetic.ensemble_members(args.members)
    # over N GPUs each rank solves its share of the members (no exchange: they are independent)
    mine = shard_members([g.nx * g.ny for (g, *_rest) in all_members], world)[rank]
    members = [all_members[k] for k in mine]
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
    if args.no_tune:  # the autotuner's choice on GB300 for this workload
        best, timings = dict(concurrency=16, coarse_kernel="auto", stencil_kernel="tiled"), []
    else:
        best, timings = autotune(grids, sps, params, make_tensors, sync=torch.cuda.synchronize)
    ens = EnsembleSolver(grids, sps, precision="mixed", picard_accel=args.picard_accel,
                         coarse_forcing=args.coarse_forcing, **best)
    times, stats = [], None
    for it in range(args.warmup + args.steps):
        work = make_tensors()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        stats = ens.solve_device(params, work)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    ens.close()
    conv_local = sum(1 for st in stats if st["status"] == 0)
    # converged solves only, every rank's members over the slowest rank's time
    value, total_s, conv = aggregate_ensemble(torch, dist, world, sum(times), conv_local, len(times),
                                              "cuda" if world > 1 and torch.cuda.is_available() else "cpu")
    if world > 1:  # the comparisons below are single-GPU measurements: rank 0 alone reports its line
        line = {"metric": "converged velocity solves/s (ragged 256-member ensemble, mixed precision)",
                "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * total_s / len(times), "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": {"workload": ENSEMBLE_WORKLOAD, "members": args.members, "members_this_rank": len(mine),
                           "launch": best, "sharding": "members split over ranks by h cells, longest first onto "
                                                       "the least-loaded rank; no collective on the data path",
                           "timing": "host wall clock around each whole-ensemble solve, barrier on both sides"},
                "members_converged": conv, "picard_accel": stats[0]["picard_accel"],
                "coarse_forcing": stats[0]["coarse_forcing"]}
        dist.destroy_process_group()
        if rank == 0:
            print(json.dumps(line), flush=True)
        return line if getattr(args, "quiet", False) else 0
    # one ensemble solve with the other Picard iteration and coarse tolerance
    other_accel, o_accel, o_forcing = other_iteration(args)
    eo = EnsembleSolver(grids, sps, precision="mixed", picard_accel=o_accel, coarse_forcing=o_forcing, **best)
    eo.solve_device(params, make_tensors())  # graph instantiation
    work_o = make_tensors()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    stats_o = eo.solve_device(params, work_o)
    t_o = time.perf_counter() - t0
    eo.close()
    conv_o = sum(1 for st in stats_o if st["status"] == 0)
    accel_other = {"picard_accel": o_accel, "coarse_forcing": o_forcing, "value": conv_o / t_o, "unit": "solves/s",
                   "seconds": t_o,
                   "members_converged": conv_o,
                   "picard_iterations_mean": float(np.mean([st["picard_iterations"] for st in stats_o]))}
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
    line = {
        "metric": "converged velocity solves/s (ragged 256-member ensemble, mixed precision)", "value": value,
        "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": ENSEMBLE_WORKLOAD, "members": n, "h_cells": int(sum(g.nx * g.ny for g in grids)),
                   "launch": best, "timing": "host wall clock around each whole-ensemble solve"},
        "all_members": {"value": n * len(times) / sum(times), "unit": "member solves/s",
                        "note": "every member, converged or stopped at maxiter_picard"},
        "fp64_loop": {"value": fp64_value, "unit": "solves/s", "members_timed": len(subset)},
        "ensemble_over_fp64_loop": (n * len(times) / sum(times)) / fp64_value,
        "rel_err_vs_fp64_max": max(errs) if errs else None,
        "rel_err_vs_fp64_median": float(np.median(errs)) if errs else None, "rel_err_members": len(errs),
        "members_converged": conv,
        "picard_accel": stats[0]["picard_accel"], "coarse_forcing": stats[0]["coarse_forcing"],
        "mixed_" + other_accel: accel_other,
        "note": "value counts the members that reach 1e-6 within maxiter_picard = 100 (members_converged); the "
                "others stall the same way in FP64 (the reference algorithm's one V-cycle per Picard iteration). "
                "ensemble_over_fp64_loop compares member solves per second, converged or not, on both sides",
        "picard_iterations_mean": float(np.mean([st["picard_iterations"] for st in stats])),
        "autotune": [{"seconds": t, "stage": stage, **c} for t, c, stage in timings],
    }
    if getattr(args, "quiet", False):
        return line
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
    # the same gradient with the solve's own FP64 V-cycle as the FGMRES preconditioner (wavi_adjoint_precond)
    s64 = VelocitySolver(g, sp, precision="fp64", adjoint_precond="fp64")
    s64.solve(params, {k: np.array(v, copy=True, order="F") for k, v in state["m"].fields.items()})
    gc64, ga64 = torch.zeros_like(gc), torch.zeros_like(ga)
    t64 = []
    for it in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ast64 = s64.adjoint_device(params, dev(gu), dev(gv), gc64, ga64, tol=1e-12, maxiter=400)
        t64.append(time.perf_counter() - t0)
    s64.close()
    gdiff = float(torch.linalg.norm(torch.cat([gc - gc64, ga - ga64])) / torch.linalg.norm(torch.cat([gc64, ga64])))
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
        "adjoint": {"fgmres_iterations": ast["iterations"], "rel_residual": ast["rel_residual"],
                    "preconditioner": "V-cycle in FP32 where it fits (wavi_adjoint_precond auto)"},
        "adjoint_fp64_precond": {"seconds": min(t64), "fgmres_iterations": ast64["iterations"],
                                 "rel_residual": ast64["rel_residual"], "gradient_rel_diff": gdiff,
                                 "note": "the same gradient with the solve's FP64 V-cycle as the preconditioner"},
        "tangent": {"fgmres_iterations": tst["iterations"], "rel_residual": tst["rel_residual"]},
        "dot_test_rel_err": abs(lhs - rhs) / max(abs(lhs), abs(rhs)),
        "fd_step_sweep": {str(h): e for h, e in sweep.items()}, "fd_step": h_best,
        "fd_directions": len(errs), "fd_max_rel_err": max(errs), "fd_median_rel_err": float(np.median(errs)),
    }
    solver.close()
    if getattr(args, "quiet", False):
        return line
    print(json.dumps(line), flush=True)
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
    if args.profile == "relin":
        # the relinearisation kernels on the 2560 x 320, nσ = 8 state (one relinearisation, then
        # --op-launches timed launches of each kernel)
        from wavi_gb300 import synthetic
        from wavi_gb300.model import GPUParallelSpec, Model, pre_solve
        g, bed, p, sp, ic = synthetic.channel_c3(tol_picard=1e-6, maxiter_picard=30)
        m = Model(g, bed, p, sp, ic, parallel_spec=GPUParallelSpec(precision="fp64"))
        pre_solve(m)
        snap = {k: np.array(v, copy=True) for k, v in m.fields.items()}
        release_solver(m)
        s = VelocitySolver(g, sp, precision=args.precision, viscosity=args.viscosity)
        dev = {k: torch.from_numpy(np.ascontiguousarray(np.asarray(snap[k]).ravel(order="F"))).cuda()
               for k in solve_field_names()}
        s.relinearise_device(m.params, dev)
        s.time_relinearise_device(args.op_launches)
        torch.cuda.synchronize()
        s.close()
        return 0
    if args.config == "c3":  # the 2560 x 320, nσ = 8 state instead of the 640 x 80 workload
        from wavi_gb300 import synthetic
        from wavi_gb300.model import GPUParallelSpec, Model, pre_solve
        g3, bed3, p3, sp3, ic3 = synthetic.channel_c3(tol_picard=1e-6, maxiter_picard=30)
        m = Model(g3, bed3, p3, sp3, ic3, parallel_spec=GPUParallelSpec(precision="fp64"))
        pre_solve(m)
    else:
        m = build_state(None)
    snapshot = {k: np.array(v, copy=True) for k, v in m.fields.items()}
    release_solver(m)
    sp = SolverParams(**{**m.solver_params.__dict__, "maxiter_picard": args.picard})
    s = VelocitySolver(m.grid, sp, precision=args.precision, use_graphs=False,
                       coarse_solver=args.coarse_solver if args.precision == "mixed" else "auto",
                       cheb_steps=args.cheb_steps, coarse_kernel=args.coarse_kernel, viscosity=args.viscosity)
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
    ap.add_argument("--profile", choices=("solve", "op", "relin"), help="run one small untimed case for ncu and exit")
    ap.add_argument("--coarse-kernel", default="auto", choices=("auto", "persistent", "iterations", "persistent_global"),
                    help="--profile solve: the coarse-CG kernel")
    ap.add_argument("--picard", type=int, default=1, help="--profile solve: Picard iterations")
    ap.add_argument("--precision", default="mixed", choices=("mixed", "fp64"), help="--profile solve: precision")
    ap.add_argument("--op-launches", type=int, default=3, help="--profile op: operator launches")
    ap.add_argument("--coarse-solver", default="auto",
                    choices=("auto", "cg", "srcg", "srcg_jacobi", "srcg_chebyshev", "pipelined_chebyshev"),
                    help="coarse solver of the mixed-precision solves (the FP64 solve keeps the reference's)")
    ap.add_argument("--coarse-sums", default="default", choices=("default", "float_float", "fp64", "fp64_solve"),
                    help="accumulation of the mixed coarse CG's dot products (wavi_coarse_sums)")
    ap.add_argument("--viscosity", default="default", choices=("default", "fp32", "fp64"),
                    help="precision of the mixed solves' viscosity sweeps (wavi_viscosity)")
    ap.add_argument("--picard-accel", default="auto", choices=("auto", "plain", "anderson"),
                    help="Picard iteration of the timed mixed solves (wavi_picard_accel; auto = Anderson in mixed "
                         "precision); the other one is reported beside it")
    ap.add_argument("--coarse-forcing", default="auto", choices=("auto", "fixed", "adaptive"),
                    help="coarse-CG tolerance of the timed mixed solves (wavi_coarse_forcing; auto = adaptive in "
                         "mixed precision)")
    ap.add_argument("--cheb-steps", type=int, default=0,
                    help="Chebyshev steps of the Chebyshev coarse solvers (0: the library's default, 3; else odd)")
    ap.add_argument("--config", default="c2", choices=("c2", "c3", "c4", "c5"),
                    help="c2: the 640x80 solve (default); c3: the 2560x320 nsigma=8 solve; c4: the adjoint on 640x80; "
                         "c5: the ragged 256-member ensemble")
    ap.add_argument("--directions", type=int, default=20, help="--config c4: finite-difference directions")
    ap.add_argument("--members", type=int, default=256, help="--config c5: ensemble members")
    ap.add_argument("--no-tune", action="store_true", help="--config c5: skip the autotuner")
    ap.add_argument("--no-extras", action="store_true",
                    help="c2: leave out the compact c3/c4/c5 lines measured after the timed work")
    args = ap.parse_args()
    # more hardware work queues than the default 8, so that the ensemble's concurrent members do not
    # serialise (set before the first CUDA call: the default line measures the ensemble too)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    if args.profile:
        return profile_case(args)
    if args.config == "c3":
        return c3_arm(args)
    if args.config == "c4":
        return adjoint_arm(args)
    if args.config == "c5":
        return ensemble_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
