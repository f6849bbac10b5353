"""Restricted additive Schwarz (RAS) over overlapping subdomains: the decomposition of the reference's
SharedMemorySpec (src/SharedMemorySpec.jl).

The reference's precondition!(model, ::SharedMemorySpec) (:78-158) tests the global residual and then, for
niterations, copies the global velocities into every subdomain model (schwarzRestrictVelocities!), runs
update_state! on each subdomain (a nested solve with the subdomain's halo velocities held fixed), scales the
global velocities by `damping` and adds (1 - damping) times each subdomain's velocities weighted by a
partition of unity (schwarzProlongVelocities!).  This module restates the pieces of that loop that live on
the host — subdomain ranges, subdomain problems, restriction, prolongation and the partition of unity —
with the reference's 1-based index arithmetic written 0-based — and the sweep loop, whose subdomain solve
is a callable (by default update_state on a host Model, i.e. one velocity-solver context per subdomain).

Because a subdomain's edge cells miss the shear-strain corners beyond the cut, their viscosity differs from
the global model's, so a sweep of the converged global solution moves it by the order of the Picard
tolerance times the ramp weights — in the reference as here; the sweeps are a preconditioner, not a solver.
"""
from dataclasses import dataclass, replace

import numpy as np

from .config import Grid, InitialConditions


@dataclass
class SchwarzSpec:
    """SharedMemorySpec (src/SharedMemorySpec.jl:5-12) as a model's parallel spec: ngridsx x ngridsy
    subdomains, `overlap` h cells of overlap on each side, niterations Schwarz iterations per Picard
    iteration, and the damping of the prolongation.  ``subdomain_spec`` is the parallel spec of the
    subdomain models (the reference gives them BasicParallelSpec(), :275); by default a GPUParallelSpec."""
    ngridsx: int = 1
    ngridsy: int = 1
    overlap: int = 1
    niterations: int = 0
    damping: float = 0.0
    subdomain_spec: object = None

    def __post_init__(self):
        if self.subdomain_spec is None:
            from .model import GPUParallelSpec
            self.subdomain_spec = GPUParallelSpec()
        # the reference does not check these; overlap 0 gives its partition of unity ramps of length 0 and
        # -1, and NaN weights
        if self.ngridsx < 1 or self.ngridsy < 1:
            raise ValueError("ngridsx and ngridsy must be >= 1")
        if self.overlap < 1:
            raise ValueError("overlap must be >= 1")
        if self.niterations < 0:
            raise ValueError("niterations must be >= 0")


def subdomain_range(nx, ny, igrid, jgrid, spec):
    """The h cells of subdomain (igrid, jgrid) (1-based, as in the reference) as 0-based half-open ranges
    (i0, i1, j0, j1): the subdomain's block of nx/ngridsx x ny/ngridsy cells and `overlap` more cells on
    each side, clipped to the domain (schwarzModel, :181-201)."""
    if nx % spec.ngridsx or ny % spec.ngridsy:
        raise ValueError("Model domain is not an integer number of subdomains")
    if not (1 <= igrid <= spec.ngridsx and 1 <= jgrid <= spec.ngridsy):
        raise IndexError((igrid, jgrid))
    nxd, nyd = nx // spec.ngridsx, ny // spec.ngridsy
    i_start = (igrid - 1) * nxd + 1
    i_stop = igrid * nxd
    j_start = (jgrid - 1) * nyd + 1
    j_stop = jgrid * nyd
    i_start_g = max(i_start - spec.overlap, 1)
    i_stop_g = min(i_stop + spec.overlap, nx)
    j_start_g = max(j_start - spec.overlap, 1)
    j_stop_g = min(j_stop + spec.overlap, ny)
    return i_start_g - 1, i_stop_g, j_start_g - 1, j_stop_g


def partition_of_unity(m, n, leavei1, leaveim, leavej1, leavejn, overlapi, overlapj):
    """The m x n weights of schwarzPartitionOfUnity (:398-407): 1 inside, ramping linearly to 0 over
    `overlapi` (`overlapj`) points towards each edge whose flag is not set.  The ramps of two neighbouring
    subdomains add to 1 across their overlap."""
    if not m > (0 if leavei1 else overlapi) + (0 if leaveim else overlapi):
        raise ValueError("partition of unity: too few points in i for the ramps")
    if not n > (0 if leavej1 else overlapj) + (0 if leavejn else overlapj):
        raise ValueError("partition of unity: too few points in j for the ramps")
    i = np.arange(1, m + 1, dtype=np.float64)
    j = np.arange(1, n + 1, dtype=np.float64)
    fi = np.ones(m)
    if not leavei1:
        fi = np.minimum(fi, (i - 1) / overlapi)
    if not leaveim:
        fi = np.minimum(fi, (m - i) / overlapi)
    fj = np.ones(n)
    if not leavej1:
        fj = np.minimum(fj, (j - 1) / overlapj)
    if not leavejn:
        fj = np.minimum(fj, (n - j) / overlapj)
    return np.asfortranarray(fi[:, None] * fj[None, :])


def subdomain_problem(model, igrid, jgrid, spec):
    """The inputs of subdomain (igrid, jgrid)'s model, taken from the global model's grid, parameters and
    current fields (schwarzModel, :180-287): (grid, bed, params, initial conditions).  The subdomain's
    velocity points on its cut boundaries (not the domain's own boundary) are fixed (:218-225): the global
    solution enters there as Dirichlet values."""
    g = model.grid
    i0, i1, j0, j1 = subdomain_range(g.nx, g.ny, igrid, jgrid, spec)
    nxg, nyg = i1 - i0, j1 - j0
    u_isfixed = g.u_isfixed[i0:i1 + 1, j0:j1].copy(order="F")
    v_isfixed = g.v_isfixed[i0:i1, j0:j1 + 1].copy(order="F")
    if igrid != 1:
        u_isfixed[0, :] = True
        v_isfixed[0, :] = True
    if igrid != spec.ngridsx:
        u_isfixed[nxg, :] = True
        v_isfixed[nxg - 1, :] = True
    if jgrid != 1:
        v_isfixed[:, 0] = True
        u_isfixed[:, 0] = True
    if jgrid != spec.ngridsy:
        v_isfixed[:, nyg] = True
        u_isfixed[:, nyg - 1] = True
    grid = Grid(nx=nxg, ny=nyg, dx=g.dx, dy=g.dy, nσ=g.nσ, x0=g.x0 + i0 * g.dx, y0=g.y0 + j0 * g.dy,
                h_mask=g.h_mask[i0:i1, j0:j1].copy(order="F"), h_isfixed=g.h_isfixed[i0:i1, j0:j1].copy(order="F"),
                u_iszero=g.u_iszero[i0:i1 + 1, j0:j1].copy(order="F"),
                v_iszero=g.v_iszero[i0:i1, j0:j1 + 1].copy(order="F"), u_isfixed=u_isfixed, v_isfixed=v_isfixed,
                quadrature_weights=g.quadrature_weights, σ=g.σ)
    f = model.fields
    crop = lambda a: np.asfortranarray(np.asarray(a)[i0:i1, j0:j1]).copy(order="F")
    glen_a_ref = np.broadcast_to(np.asarray(model.params.glen_a_ref, np.float64), (g.nx, g.ny))
    params = replace(model.params, weertman_c=crop(model.weertman_c_param),
                     accumulation_rate=crop(model.accumulation_param), glen_a_ref=crop(glen_a_ref))
    ic = InitialConditions(initial_thickness=crop(f["h"]), initial_grounded_fraction=crop(f["grounded_fraction"]),
                           initial_u_veloc=np.asfortranarray(f["u"][i0:i1 + 1, j0:j1]).copy(order="F"),
                           initial_v_veloc=np.asfortranarray(f["v"][i0:i1, j0:j1 + 1]).copy(order="F"),
                           initial_viscosity=np.asfortranarray(f["eta"][i0:i1, j0:j1, :]).copy(order="F"),
                           initial_temperature=np.asfortranarray(f["temperature"][i0:i1, j0:j1, :]).copy(order="F"),
                           initial_damage=np.asfortranarray(f["damage"][i0:i1, j0:j1, :]).copy(order="F"))
    return grid, crop(f["b"]), params, ic


def restrict_velocities(model_g, model, igrid, jgrid, spec):
    """schwarzRestrictVelocities! (:306-330): the global velocities on the subdomain's points."""
    g = model.grid
    i0, i1, j0, j1 = subdomain_range(g.nx, g.ny, igrid, jgrid, spec)
    model_g.fields["u"][...] = model.fields["u"][i0:i1 + 1, j0:j1]
    model_g.fields["v"][...] = model.fields["v"][i0:i1, j0:j1 + 1]


def prolong_velocities(model, model_g, igrid, jgrid, spec):
    """schwarzProlongVelocities! (:350-380): add (1 - damping) times the subdomain's velocities, weighted
    by its partition of unity (ramps over 2 overlap u points and 2 overlap - 1 v points across x, and the
    reverse across y), to the global velocities.  The caller has scaled the global velocities by damping
    before the first subdomain is added (precondition!, :124-125)."""
    g = model.grid
    i0, i1, j0, j1 = subdomain_range(g.nx, g.ny, igrid, jgrid, spec)
    nxg, nyg = i1 - i0, j1 - j0
    edges = (igrid == 1, igrid == spec.ngridsx, jgrid == 1, jgrid == spec.ngridsy)
    upou = partition_of_unity(nxg + 1, nyg, *edges, 2 * spec.overlap, 2 * spec.overlap - 1)
    vpou = partition_of_unity(nxg, nyg + 1, *edges, 2 * spec.overlap - 1, 2 * spec.overlap)
    w = 1.0 - spec.damping
    model.fields["u"][i0:i1 + 1, j0:j1] += w * upou * model_g.fields["u"]
    model.fields["v"][i0:i1, j0:j1 + 1] += w * vpou * model_g.fields["v"]


def build_subdomains(model, spec, make=None):
    """update_preconditioner!(model, ::SharedMemorySpec) (:53-69): one subdomain model per (igrid, jgrid)
    from the global model's current state.  ``make(grid, bed, params, solver_params, initial_conditions)``
    builds each one; by default a host Model with the global model's solver parameters and the spec's
    subdomain_spec (so each subdomain solves through its own velocity-solver context)."""
    if make is None:
        from .model import Model
        make = lambda grid, bed, params, solver_params, ic: Model(grid, bed, params, solver_params, ic,
                                                                   parallel_spec=spec.subdomain_spec)
    subs = {}
    for igrid in range(1, spec.ngridsx + 1):
        for jgrid in range(1, spec.ngridsy + 1):
            grid, bed, params, ic = subdomain_problem(model, igrid, jgrid, spec)
            subs[igrid, jgrid] = make(grid, bed, params, model.solver_params, ic)
    return subs


def ras_sweeps(model, spec, subdomains, solve=None, solve_all=None):
    """The Schwarz iterations of precondition!(model, ::SharedMemorySpec) (:98-155), run spec.niterations
    times: restrict the global velocities into every subdomain, solve every subdomain (``solve_all`` on
    all of them at once, e.g. an EnsembleSubdomainSolver; else ``solve`` on each, by default update_state
    on a host Model), scale the global velocities by damping and add every subdomain's velocities back
    through its partition of unity.  The residual test that precedes the sweeps in the reference belongs
    to the caller's Picard loop."""
    if solve is None and solve_all is None:
        from .model import update_state
        solve = update_state
    for _ in range(spec.niterations):
        for (igrid, jgrid), sub in subdomains.items():
            restrict_velocities(sub, model, igrid, jgrid, spec)
        if solve_all is not None:
            solve_all(subdomains)
        else:
            for sub in subdomains.values():
                solve(sub)
        model.fields["u"] *= spec.damping
        model.fields["v"] *= spec.damping
        for (igrid, jgrid), sub in subdomains.items():
            prolong_velocities(model, sub, igrid, jgrid, spec)
    return model


class EnsembleSubdomainSolver:
    """update_state on every subdomain with the velocity solves batched: the host steps before and after
    the solve (pre_solve, post_solve_steps) run per subdomain, and the subdomains' velocity solves run as
    the members of one ensemble (wavi_ensemble_solve_device: one context and stream per member, members of
    different sizes), the way the reference runs them on threads (:112-120).

    The ensemble is made once from the subdomains' grids and serves every sweep, and every set of
    subdomain models built later from the same decomposition (build_subdomains after each Picard
    relinearisation).  ``ensemble`` replaces it with any object that has the same solve_device, and
    ``device`` names the torch device the member fields are staged on."""

    def __init__(self, subdomains, precision="fp64", device=0, concurrency=16, ensemble=None):
        subs = list(subdomains.values())
        if ensemble is None:
            from .ensemble import EnsembleSolver
            ensemble = EnsembleSolver([s.grid for s in subs], [s.solver_params for s in subs], precision=precision,
                                      device=device, concurrency=concurrency)
            device = f"cuda:{device}"
        self.ensemble = ensemble
        self.device = device
        self.shapes = [(s.grid.nx, s.grid.ny) for s in subs]

    def __call__(self, subdomains):
        from .model import post_solve_steps, pre_solve
        subs = list(subdomains.values())
        if [(s.grid.nx, s.grid.ny) for s in subs] != self.shapes:
            raise ValueError("the subdomains do not match the ensemble's members")
        for s in subs:
            pre_solve(s)
        tensors = [_member_tensors(s.fields, self.device) for s in subs]
        stats = self.ensemble.solve_device([s.params for s in subs], tensors)
        for s, t, st in zip(subs, tensors, stats):
            _member_fields_back(s.fields, t)
            s.last_stats = st
        for s in subs:
            post_solve_steps(s)
        return stats


_COARSE = ("wu_correction_coarse", "wv_correction_coarse")


def _member_tensors(fields, device):
    """The velocity solve's fields (column-major, masks as bytes) as flat tensors on ``device``.  A
    subdomain's adaptive coarse space can be empty (update_wavelets! found no coefficient above the
    threshold); its compact correction then has no entries, and a tensor of none has no device address,
    so it is staged with one unused entry (the solve reads and writes count(mask) entries only)."""
    import torch
    from .gpu import ALL_FIELDS
    out = {}
    for name in ALL_FIELDS:
        a = np.asarray(fields[name])
        dt = np.uint8 if name in ("wu_mask", "wv_mask") else np.float64
        flat = np.ascontiguousarray(a.astype(dt).ravel(order="F"))
        if name in _COARSE and flat.size == 0:
            flat = np.zeros(1)
        out[name] = torch.from_numpy(flat).to(device)
    return out


def _member_fields_back(fields, tensors):
    """The solved member's fields back into the host model, in place where the shape is unchanged (the
    compact coarse corrections keep count(wavelet mask) entries)."""
    from .gpu import ALL_FIELDS
    for name in ALL_FIELDS:
        host = tensors[name].cpu().numpy()
        cur = fields[name]
        if name in _COARSE:
            mask = fields["wu_mask" if name == "wu_correction_coarse" else "wv_mask"]
            fields[name] = host[:int(np.count_nonzero(mask))].copy()
        else:
            cur[...] = host.reshape(cur.shape, order="F")


_RESIDUAL_SOLVERS = {}


def gpu_global_residual(model):
    """inner_update!(model) and the residual test of precondition!(model, ::SharedMemorySpec) (:84-95) on
    the GPU: one Picard iteration of the velocity solve relinearises the model at its velocities and reports
    ‖b − A u‖/‖b‖ before its V-cycle correction, which is then undone (velocities and coarse cache
    restored).  The model keeps the relinearised fields and the residual, as after inner_update! and
    set_residual!.  Costs one V-cycle more than the test needs.  Returns the relative residual."""
    from dataclasses import replace as _replace
    from . import gpu
    key = id(model)
    s = _RESIDUAL_SOLVERS.get(key)
    if s is None:
        ps = model.parallel_spec
        if isinstance(ps, SchwarzSpec):
            ps = ps.subdomain_spec
        s = gpu.VelocitySolver(model.grid, _replace(model.solver_params, maxiter_picard=1),
                               precision=getattr(ps, "precision", "fp64"), device=getattr(ps, "device", 0))
        _RESIDUAL_SOLVERS[key] = s
    f = model.fields
    keep = {k: np.array(f[k], copy=True) for k in ("u", "v", "wu_correction_coarse", "wv_correction_coarse")}
    st = s.solve(model.params, f)
    for k, a in keep.items():
        if k in ("u", "v"):
            f[k][...] = a
        else:
            f[k] = a
    return float(st["rel_residual"])


def release_residual_solver(model):
    s = _RESIDUAL_SOLVERS.pop(id(model), None)
    if s is not None:
        s.close()


def update_velocities_schwarz(model, spec, global_residual=None, solve=None, solve_all=None, make=None):
    """update_velocities!(model) with the reference's SharedMemorySpec (update_velocities.jl:11-29 with
    SharedMemorySpec.jl:53-69 and :78-158): the subdomain models built once from the model's state
    (update_preconditioner!), then Picard iterations of inner_update! and precondition!, the global
    residual test (``global_residual(model)``, by default gpu_global_residual) followed, unless it passes,
    by spec.niterations Schwarz sweeps (ras_sweeps with ``solve`` or ``solve_all``), until the test passes
    or maxiter_picard.  There is no global coarse correction: as in the reference, the sweeps' fixed point
    differs from the global solution near the subdomains' cut boundaries, so the residual levels off (at
    ~1e-3 on a 32 x 16 channel in 2 x 2 subdomains).  Returns (converged, relative residual, iterations)."""
    if global_residual is None:
        global_residual = gpu_global_residual
    subdomains = build_subdomains(model, spec, make)
    sp = model.solver_params
    converged, i, rel = False, 0, float("inf")
    while not converged and i < sp.maxiter_picard:
        i += 1
        rel = global_residual(model)
        converged = rel < sp.tol_picard
        if not converged:
            ras_sweeps(model, spec, subdomains, solve=solve, solve_all=solve_all)
    print(f"Solved momentum equation with residual {rel:.3g} at iteration {i}")
    model.last_stats = {"picard_iterations": i, "rel_residual": rel, "converged": converged}
    return converged, rel, i
