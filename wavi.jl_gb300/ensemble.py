"""Ensembles of independent domains solved at once (include/wavi_gpu.h, wavi_ensemble_*), and the
autotuner that picks their launch configuration.

An ensemble holds one solver context per member (grids of different sizes); a solve issues every
member's whole Picard-converged solve (a CUDA graph) on the member's own stream, with at most
``concurrency`` members in flight, and returns when all are done.  There is no CPU fallback.
"""
import ctypes as C
import dataclasses
import time

from . import abi
from .gpu import PRECISIONS, VelocitySolver, device_fields, stats_dict


class EnsembleSolver:
    """``wavi_ensemble``: one context per member grid, solved concurrently."""

    def __init__(self, grids, solver_params, precision="mixed", device=0, concurrency=16, coarse_kernel="auto",
                 coarse_solver="auto", stencil_kernel="auto", picard_accel="auto",
                 coarse_forcing="auto"):
        self.lib = abi.load_library()
        self.n = n = len(grids)
        if len(solver_params) != n:
            raise ValueError("one SolverParams per member")
        self.grids = grids
        descs = [g.descriptor() for g in grids]  # keeps the mask arrays alive through the create call
        garr = (abi.GridDesc * n)(*[d.desc for d in descs])
        sparr = (abi.SolverParams * n)(*[sp.to_c() for sp in solver_params])
        opt = abi.Options(int(device), PRECISIONS[precision], 1, 0, VelocitySolver.COARSE_KERNELS[coarse_kernel],
                          abi.COARSE_SOLVERS[coarse_solver], VelocitySolver.STENCIL_KERNELS[stencil_kernel], 0)
        opt.picard_accel = abi.PICARD_ACCEL[picard_accel]
        opt.coarse_forcing = abi.COARSE_FORCING[coarse_forcing]
        ens = C.c_void_p()
        st = self.lib.wavi_ensemble_create(n, garr, sparr, C.byref(opt), int(concurrency), C.byref(ens))
        if st != 0:
            raise abi.WaviError(st, self.lib.wavi_last_error(None).decode())
        self.ens = ens
        self.config = dict(concurrency=int(concurrency), coarse_kernel=coarse_kernel, coarse_solver=coarse_solver,
                           stencil_kernel=stencil_kernel, picard_accel=picard_accel,
                           coarse_forcing=coarse_forcing)

    def close(self):
        if getattr(self, "ens", None) and self.ens.value:
            self.lib.wavi_ensemble_destroy(self.ens)
            self.ens = C.c_void_p()

    __del__ = close

    def solve_device(self, params, tensors):
        """update_velocities! for every member: params and tensors (dicts of device tensors, modified in
        place) are lists of n.  Returns the members' stats dicts."""
        n = self.n
        parr = (abi.Params * n)(*[p.to_c() for p in params])
        farr = (abi.Fields * n)(*[device_fields(t) for t in tensors])
        starr = (abi.Stats * n)()
        st = self.lib.wavi_ensemble_solve_device(self.ens, parr, farr, starr)
        if st != 0:
            raise abi.WaviError(st, self.lib.wavi_ensemble_last_error(self.ens).decode())
        return [stats_dict(starr[k]) for k in range(n)]


def shard_members(costs, world):
    """The members each of `world` GPUs solves when an ensemble is split across GPUs (one process per GPU,
    no exchange between them: the members are independent): longest first onto the least-loaded rank, by
    the estimated cost of each member (its h cells), ties to the lower rank.  Returns one ascending index
    list per rank; every member appears exactly once, and no rank carries more than the average load plus
    the largest member."""
    world = int(world)
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for k in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(k)
        load[r] += float(costs[k])
    return [sorted(ix) for ix in out]


# Members in flight and stencil kernel of the operator and smoother sweeps (shared-memory 32 x 8 tiles, or
# row streaming), with the persistent coarse-CG kernel (register-resident where a member's share of the device
# holds its tiles, else global-memory).  On the 256-member workload per-iteration coarse kernels and 32 or 64
# members in flight were slower in every trial (GB300), so they are left out of the default set.
DEFAULT_CANDIDATES = tuple(dict(concurrency=s, coarse_kernel="auto", stencil_kernel=sk) for s in (8, 12, 16, 24)
                           for sk in ("tiled", "streaming"))


def autotune(grids, solver_params, params, make_tensors, precision="mixed", device=0, candidates=DEFAULT_CANDIDATES,
             picard=8, finalists=3, sync=None):
    """Pick the ensemble launch configuration in two stages.  First, for each candidate (keyword arguments
    of EnsembleSolver: members in flight, coarse-CG kernel, stencil kernel), time one ensemble solve capped
    at `picard` Picard iterations, after one untimed solve that instantiates the graphs.  Then time one
    whole solve (the members' own Picard limits) of each of the `finalists` fastest and keep the fastest of
    those.  The capped solves are dominated by the first V-cycles, on the cold all-true coarse space, and
    miss the tail of members that take many Picard iterations, so they rank the candidates only roughly.
    `make_tensors()` returns fresh device copies of every member's fields.  Returns (best candidate,
    [(seconds, candidate, stage), ...])."""
    capped = [dataclasses.replace(sp, maxiter_picard=picard) for sp in solver_params]
    timings = []

    def timed(cand, sps):
        ens = EnsembleSolver(grids, sps, precision=precision, device=device, **cand)
        try:
            ens.solve_device(params, make_tensors())
            tensors = make_tensors()
            if sync:
                sync()
            t0 = time.perf_counter()
            ens.solve_device(params, tensors)
            return time.perf_counter() - t0
        finally:
            ens.close()

    for cand in candidates:
        timings.append((timed(cand, capped), cand, "capped"))
    ranked = sorted(timings, key=lambda t: t[0])[:max(1, finalists)]
    full = []
    for _, cand, _ in ranked:
        full.append((timed(cand, solver_params), cand, "whole"))
    timings += full
    best = min(full, key=lambda t: t[0])[1]
    return best, timings
