"""Host-side mirror of the reference's Model / update_state! / Simulation, with the velocity solve
dispatched on the model's parallel spec exactly where the reference dispatches it.

  Model(...)                      src/Models/Model.jl:34-93, check_initial_conditions
                                  src/Models/model_utilities.jl:7-60, setup_fields src/Fields/Fields.jl:26-115
  update_state!                   src/Models/update_state.jl:7-42 (surface, geometry on u/v, HAF, grounded
                                  fraction, accumulation, melt, Weertman C, dsdh, VELOCITY SOLVE, h-grid
                                  velocities, dh/dt, wavelets)
  pos_fraction                    src/utilities.jl:255-396
  update_wavelets!                src/Wavelets/update_wavelets.jl:6-32
  update_thickness!, timestep!,   src/Simulations/run_simulation.jl:6-57, :61-100
  run_simulation!

The velocity solve itself is ``update_velocities(model)``: with ``GPUParallelSpec`` it calls
libwavi_gpu.so through ``gpu.VelocitySolver`` (the drop-in for src/Models/update_velocities.jl:11-29).
Everything here is O(N) numpy host work around that call.
"""
from dataclasses import dataclass

import numpy as np

from .config import Grid, InitialConditions, OutputParams, Params, SolverParams, TimesteppingParams
from . import gpu


@dataclass
class GPUParallelSpec:
    """The backend selector (a new AbstractParallelSpec subtype in the reference's type tree,
    src/WAVI.jl:17).  Plain data only, so a saved model never holds a device handle."""
    device: int = 0
    precision: str = "fp64"     # "fp64" (reference algorithm) or "mixed"
    use_graphs: bool = True
    picard_test: int = 0
    coarse_solver: str = "auto"  # "auto", "cg" (reference), "srcg", "srcg_jacobi", "srcg_chebyshev" (single-reduction
    #                              CG), "pipelined_chebyshev" (opt-in)
    device_run: bool = False     # run_simulation without a callback keeps the model on the device (wavi_run_device)
    picard_accel: str = "auto"   # "auto" (fp64: the reference's Picard iteration; mixed: Anderson acceleration),
    #                              "plain" or "anderson"
    coarse_forcing: str = "auto"  # "auto" (fp64: the reference's fixed tol_coarse; mixed: adaptive), "fixed",
    #                               "adaptive"


_SOLVERS = {}


def _solver_for(model):
    key = id(model)
    s = _SOLVERS.get(key)
    if s is None:
        ps = model.parallel_spec
        s = gpu.VelocitySolver(model.grid, model.solver_params, precision=ps.precision, device=ps.device,
                               use_graphs=ps.use_graphs, picard_test=ps.picard_test,
                               coarse_solver=ps.coarse_solver, picard_accel=ps.picard_accel,
                               coarse_forcing=ps.coarse_forcing)
        _SOLVERS[key] = s
    return s


def release_solver(model):
    s = _SOLVERS.pop(id(model), None)
    if s is not None:
        s.close()


def glen_b(temperature, damage, glen_a_ref, glen_n, glen_a_activation_energy, glen_temperature_ref, gas_const):
    """src/utilities.jl:462-466"""
    a0 = glen_a_ref * np.exp(+glen_a_activation_energy / (glen_temperature_ref * gas_const))
    return (1 - damage) * (a0 * np.exp(-glen_a_activation_energy / (temperature * gas_const))) ** (-1.0 / glen_n)


def get_u_mask(h_mask):
    nx, ny = h_mask.shape
    m = np.zeros((nx + 1, ny), bool)
    m[:-1, :] |= h_mask
    m[1:, :] |= h_mask
    return m


def get_v_mask(h_mask):
    nx, ny = h_mask.shape
    m = np.zeros((nx, ny + 1), bool)
    m[:, :-1] |= h_mask
    m[:, 1:] |= h_mask
    return m


def get_c_mask(h_mask):
    return h_mask[:-1, :-1] & h_mask[:-1, 1:] & h_mask[1:, :-1] & h_mask[1:, 1:]


def _F(a):
    return np.asfortranarray(a, dtype=np.float64)


class Model:
    """Mirror of WAVI.Model: grid, params, solver_params and the fields the solve reads and writes."""

    def __init__(self, grid: Grid, bed_elevation, params: Params = None, solver_params: SolverParams = None,
                 initial_conditions: InitialConditions = None, melt_rate: float = 0.0, parallel_spec=None):
        if grid is None:
            raise ValueError("You must specify an input grid")
        if bed_elevation is None:
            raise ValueError("You must input a bed elevation")
        params = params or Params()
        solver_params = solver_params or SolverParams()
        ic = initial_conditions or InitialConditions()
        self.grid, self.params, self.solver_params = grid, params, solver_params
        self.parallel_spec = parallel_spec or GPUParallelSpec()
        self.melt_rate = float(melt_rate)  # UniformMeltRate(m), src/MeltRate/MeltRate.jl:37-54
        nx, ny, ns = grid.nx, grid.ny, grid.nσ
        bed = np.vectorize(bed_elevation)(grid.xxh, grid.yyh) if callable(bed_elevation) else bed_elevation
        bed = _F(bed)
        if bed.shape != (nx, ny):
            raise ValueError("bed elevation must be nx x ny")

        def pick(v, default, shape):
            a = default if v is None else _F(v)
            if a.shape != shape:
                raise ValueError(f"DimensionMismatch: initial condition of shape {a.shape}, expected {shape}")
            return _F(a).copy(order="F")

        h = pick(ic.initial_thickness, params.default_thickness * np.ones((nx, ny)), (nx, ny))
        gf = pick(ic.initial_grounded_fraction, np.ones((nx, ny)), (nx, ny))
        u = pick(ic.initial_u_veloc, np.zeros((nx + 1, ny)), (nx + 1, ny))
        v = pick(ic.initial_v_veloc, np.zeros((nx, ny + 1)), (nx, ny + 1))
        eta = pick(ic.initial_viscosity, params.default_viscosity * np.ones((nx, ny, ns)), (nx, ny, ns))
        temp = pick(ic.initial_temperature, params.default_temperature * np.ones((nx, ny, ns)), (nx, ny, ns))
        dmg = pick(ic.initial_damage, params.default_damage * np.ones((nx, ny, ns)), (nx, ny, ns))
        self.weertman_c_param = _F(np.broadcast_to(np.asarray(params.weertman_c, np.float64), (nx, ny)))
        self.accumulation_param = _F(np.broadcast_to(np.asarray(params.accumulation_rate, np.float64), (nx, ny)))
        glen_a_ref = _F(np.broadcast_to(np.asarray(params.glen_a_ref, np.float64), (nx, ny)))
        # masks (Fields.jl:28-35)
        self.h_mask = grid.h_mask.copy(order="F")
        self.h_isfixed = grid.h_isfixed.copy(order="F")
        self.u_mask = get_u_mask(self.h_mask)
        self.v_mask = get_v_mask(self.h_mask)
        self.c_mask = get_c_mask(self.h_mask)
        self.u_mask[grid.u_iszero] = False
        self.v_mask[grid.v_iszero] = False
        self.u_inner = self.u_mask & ~grid.u_isfixed
        self.v_inner = self.v_mask & ~grid.v_isfixed
        z = lambda *s: np.zeros(s, order="F")
        f = {}
        f["b"] = bed
        f["h"] = h
        f["s"] = z(nx, ny)
        f["dhdt"] = z(nx, ny)
        f["accumulation"] = z(nx, ny)
        f["basal_melt"] = z(nx, ny)
        f["haf"] = z(nx, ny)
        f["grounded_fraction"] = gf
        f["dsdh"] = np.ones((nx, ny), order="F")
        for k in ("shelf_strain_rate", "av_speed", "uh", "vh", "us", "vs", "ub", "vb", "bed_speed", "weertman_c",
                  "beta", "beta_eff", "tau_bed", "quad_f1"):
            f[k] = z(nx, ny)
        f["eta_av"] = eta[:, :, 0].copy(order="F")
        f["quad_f2"] = z(nx, ny)
        f["quad_f2"][self.h_mask] = h[self.h_mask] / (3 * f["eta_av"][self.h_mask])  # HGrid.jl:114
        for k in ("gu_s", "gu_h", "gu_beta_eff", "gu_residual"):
            f[k] = z(nx + 1, ny)
        f["gu_grounded_fraction"] = np.ones((nx + 1, ny), order="F")
        for k in ("gv_s", "gv_h", "gv_beta_eff", "gv_residual"):
            f[k] = z(nx, ny + 1)
        f["gv_grounded_fraction"] = np.ones((nx, ny + 1), order="F")
        f["u"], f["v"], f["eta"] = u, v, eta
        f["temperature"], f["damage"] = temp, dmg
        f["glen_b"] = _F(glen_b(temp, dmg, glen_a_ref[:, :, None], params.glen_n, params.glen_a_activation_energy,
                                params.glen_temperature_ref, params.gas_const))
        f["wu_mask"] = np.ones((nx + 1, ny), dtype=np.uint8, order="F")  # UWavelets.jl:38
        f["wv_mask"] = np.ones((nx, ny + 1), dtype=np.uint8, order="F")
        f["wu_correction_coarse"] = np.zeros(int(f["wu_mask"].sum()))
        f["wv_correction_coarse"] = np.zeros(int(f["wv_mask"].sum()))
        self.fields = f
        self.last_stats = None

    def solve_fields(self):
        return self.fields


# ---------------------------------------------------------------------------------------------------
# update_state! neighbours (src/Models/update_state.jl)
# ---------------------------------------------------------------------------------------------------
def _cent_T_u_ordered(fh):
    nx, ny = fh.shape
    lo = np.zeros((nx + 1, ny))
    hi = np.zeros((nx + 1, ny))
    lo[1:, :] = fh          # f[i-1]
    hi[:-1, :] = fh         # f[i]
    return np.asfortranarray(0.5 * lo + 0.5 * hi)


def _cent_T_v_ordered(fh):
    nx, ny = fh.shape
    lo = np.zeros((nx, ny + 1))
    hi = np.zeros((nx, ny + 1))
    lo[:, 1:] = fh
    hi[:, :-1] = fh
    return np.asfortranarray(0.5 * lo + 0.5 * hi)


def interp_h_to_uv(model, fh):
    """samp*(centᵀ*(crop_h*f)) ./ samp*(centᵀ*(crop_h*1)) at the u / v mask points (update_state.jl:68)."""
    hm = model.h_mask.astype(np.float64)
    fu = _cent_T_u_ordered(hm * fh)
    du = _cent_T_u_ordered(hm)
    fv = _cent_T_v_ordered(hm * fh)
    dv = _cent_T_v_ordered(hm)
    with np.errstate(invalid="ignore", divide="ignore"):
        return fu / du, fv / dv


def update_surface_elevation(model):
    p, f, m = model.params, model.fields, model.h_mask
    f["s"][m] = np.maximum(f["b"][m] + f["h"][m],
                           p.sea_level_wrt_geoid + f["h"][m] * (1 - p.density_ice / p.density_ocean))


def update_geometry_on_uv_grids(model):
    f = model.fields
    hu, hv = interp_h_to_uv(model, f["h"])
    su, sv = interp_h_to_uv(model, f["s"])
    f["gu_h"][model.u_mask] = hu[model.u_mask]
    f["gu_s"][model.u_mask] = su[model.u_mask]
    f["gv_h"][model.v_mask] = hv[model.v_mask]
    f["gv_s"][model.v_mask] = sv[model.v_mask]


def height_above_floatation(h, b, params):
    """height_above_floatation (src/utilities.jl:445)."""
    return h - (params.density_ocean / params.density_ice) * (params.sea_level_wrt_geoid - b)


def update_height_above_floatation(model):
    f = model.fields
    f["haf"][...] = height_above_floatation(f["h"], f["b"], model.params)


def volume_above_floatation(h, b, params, grid):
    """volume_above_floatation (src/utilities.jl:453): the positive heights above floatation times the
    cell area."""
    haf = height_above_floatation(np.asarray(h, np.float64), np.asarray(b, np.float64), params)
    return float(np.sum(haf[haf > 0])) * grid.dx * grid.dy


def grounding_line_x(haf, xxh):
    """The x of the grounding line in each row of cells along y (get_glx, src/utilities.jl:417-426): where
    the height above floatation changes from positive to negative along x, interpolated linearly between
    the two cells; in the reference's column-major order (by row, then by x)."""
    glm = (np.diff(np.sign(haf), axis=0) == -2).T
    x1, x2 = xxh[:-1, :].T[glm], xxh[1:, :].T[glm]
    h1, h2 = haf[:-1, :].T[glm], haf[1:, :].T[glm]
    return x1 + (x2 - x1) * (0.0 - h1) / (h2 - h1)


def get_glx(model):
    """get_glx(model) (src/utilities.jl:417-426) on the model's current height above floatation."""
    return grounding_line_x(model.fields["haf"], model.grid.xxh)


def pos_fraction(z1, mask=None):
    """Fraction of each cell where the bilinear-by-quadrant interpolant of z1 is positive
    (src/utilities.jl:255-396), with the h, u and v grid fractions."""
    z1 = np.asarray(z1, dtype=np.float64)
    m, n = z1.shape
    mask = np.ones((m, n), bool) if mask is None else np.asarray(mask, bool)
    af = np.zeros((m, n))
    afu = np.zeros((m + 1, n))
    afv = np.zeros((m, n + 1))
    ip = np.r_[1:m, m - 1]
    im = np.r_[0, 0:m - 1]
    jp = np.r_[1:n, n - 1]
    jm = np.r_[0, 0:n - 1]
    for q in (1, 2, 3, 4):
        if q == 1:
            s2, s3 = (ip, slice(None)), (slice(None), jp)
        elif q == 2:
            s2, s3 = (slice(None), jp), (im, slice(None))
        elif q == 3:
            s2, s3 = (im, slice(None)), (slice(None), jm)
        else:
            s2, s3 = (slice(None), jm), (ip, slice(None))
        z2 = z1[s2].copy()
        bad2 = ~mask[s2]
        z2[bad2] = z1[bad2]
        z3 = z1[s3].copy()
        bad3 = ~mask[s3]
        z3[bad3] = z1[bad3]
        afq = np.zeros((m, n))
        sc = ~((np.sign(z1) == np.sign(z2)) & (np.sign(z1) == np.sign(z3)))
        if sc.any():
            a1_, a2_, a3_ = z1[sc], z2[sc], z3[sc]
            flip = np.abs(a3_ - a1_) < np.abs(a2_ - a1_)
            with np.errstate(divide="ignore", invalid="ignore"):
                a = np.where(~flip, -(a2_ - a1_) / (a3_ - a1_), -(a3_ - a1_) / (a2_ - a1_))
                b = np.where(~flip, -2 * a1_ / (a3_ - a1_), -2 * a1_ / (a2_ - a1_))
                A1 = 0.5 * (b ** 2) / a
                A2 = 0.5 * ((1.0 - b) ** 2) / a
                A3 = 0.5 * a + b
                t1 = (b > 0.0).astype(int) + (b > 1.0)
                t2 = ((a + b) > 0.0).astype(int) + ((a + b) > 1.0)
                ix = 1 + t1 + 3 * t2
                # every candidate is evaluated; the ones a cell does not select may be inf or NaN
                area = np.select([ix == 1, ix == 2, ix == 3, ix == 4, ix == 5, ix == 6, ix == 7, ix == 8],
                                 [0.0 * a, -A1, A2 - A1, A1 + A3, A3, A2 + A3, 1.0 - A2 + A1, 1.0 - A2], 1.0)
                area = np.where(b < 0.0, 1.0 - area, area)  # b may be NaN where no candidate is selected
                area = np.where(a1_ < 0.0, 1.0 - area, area)
            afq[sc] = area
        afq[(z1 > 0.0) & (z2 > 0.0) & (z3 > 0.0)] = 1.0
        afq[(z1 <= 0.0) & (z2 <= 0.0) & (z3 <= 0.0)] = 0.0
        afq[~mask] = 0.0
        af = af + 0.25 * afq
        if q in (1, 4):
            afu[1:, :] = afu[1:, :] + 0.25 * afq
        else:
            afu[:-1, :] = afu[:-1, :] + 0.25 * afq
        if q in (1, 2):
            afv[:, 1:] = afv[:, 1:] + 0.25 * afq
        else:
            afv[:, :-1] = afv[:, :-1] + 0.25 * afq
    return np.asfortranarray(af), np.asfortranarray(afu), np.asfortranarray(afv)


def update_grounded_fraction_on_huv_grids(model):
    f = model.fields
    gh, gu, gv = pos_fraction(f["haf"], mask=model.h_mask)
    f["grounded_fraction"][...] = gh
    f["gu_grounded_fraction"][...] = gu
    f["gv_grounded_fraction"][...] = gv


def update_accumulation_rate(model):
    model.fields["accumulation"][...] = model.accumulation_param


def update_basal_melt(model):
    model.fields["basal_melt"][...] = model.melt_rate


def update_weertman_c(model):
    f = model.fields
    f["weertman_c"][...] = model.weertman_c_param * f["grounded_fraction"]


def update_dsdh(model):
    p, f = model.params, model.fields
    r = p.density_ice / p.density_ocean
    f["dsdh"][...] = (1.0 - r) + r * f["grounded_fraction"]


def update_velocities(model):
    """update_velocities!(model) dispatched on the parallel spec (update_velocities.jl:11-29): the GPU solve
    for a GPUParallelSpec, restricted additive Schwarz for a schwarz.SchwarzSpec (SharedMemorySpec)."""
    from .schwarz import SchwarzSpec, update_velocities_schwarz
    if isinstance(model.parallel_spec, SchwarzSpec):
        update_velocities_schwarz(model, model.parallel_spec)
        return model
    if not isinstance(model.parallel_spec, GPUParallelSpec):
        raise TypeError("the parallel spec must be a GPUParallelSpec or a SchwarzSpec")
    solver = _solver_for(model)
    model.last_stats = solver.solve(model.params, model.fields)
    return model


def update_velocities_on_h_grid(model):
    f = model.fields
    f["uh"][...] = 0.5 * f["u"][:-1, :] + 0.5 * f["u"][1:, :]
    f["vh"][...] = 0.5 * f["v"][:, :-1] + 0.5 * f["v"][:, 1:]
    f["ub"][...] = f["uh"] / (1 + (f["beta"] * f["quad_f2"]))
    f["vb"][...] = f["vh"] / (1 + (f["beta"] * f["quad_f2"]))
    f["us"][...] = f["ub"] * (1 + (f["beta"] * f["quad_f1"]))
    f["vs"][...] = f["vb"] * (1 + (f["beta"] * f["quad_f1"]))


def update_dhdt(model):
    g, f, m = model.grid, model.fields, model.h_mask
    qx = np.where(model.u_mask, f["gu_h"] * f["u"], 0.0)
    qy = np.where(model.v_mask, f["gv_h"] * f["v"], 0.0)
    rdx, rdy = 1.0 / g.dx, 1.0 / g.dy
    a = qx[1:, :] * rdx - qx[:-1, :] * rdx
    c = qy[:, 1:] * rdy - qy[:, :-1] * rdy
    dh = f["accumulation"] - f["basal_melt"] - (a + c)
    f["dhdt"][m] = dh[m]


def haar_forward_1d(x, levels, axis):
    """wavelet_matrix(n, levels, "forward") applied along ``axis`` by lifting (update_wavelets.jl:38-89)."""
    x = np.moveaxis(np.array(x, dtype=np.float64), axis, 0)
    n = x.shape[0]
    step = 1
    for _ in range(levels, -1, -1):
        step *= 2
        half = step // 2
        o = np.arange(0, n - half, step)
        e = o + half
        xo, xe = x[o].copy(), x[e].copy()
        x[e] = 0.5 * (xe - xo)
        x[o] = 0.5 * (xo + xe)
    return np.moveaxis(x, 0, axis)


def update_wavelets(model):
    """update_wavelets! (src/Wavelets/update_wavelets.jl:6-32)."""
    f, sp = model.fields, model.solver_params
    wu = haar_forward_1d(haar_forward_1d(np.where(model.u_mask, f["u"], 0.0), sp.levels, 1), sp.levels, 0)
    wv = haar_forward_1d(haar_forward_1d(np.where(model.v_mask, f["v"], 0.0), sp.levels, 1), sp.levels, 0)
    f["wu_mask"][...] = (np.abs(wu) >= sp.wavelet_threshold)
    f["wv_mask"][...] = (np.abs(wv) >= sp.wavelet_threshold)
    f["wu_correction_coarse"] = np.zeros(int(f["wu_mask"].sum()))
    f["wv_correction_coarse"] = np.zeros(int(f["wv_mask"].sum()))


def pre_solve(model):
    update_surface_elevation(model)
    update_geometry_on_uv_grids(model)
    update_height_above_floatation(model)
    update_grounded_fraction_on_huv_grids(model)
    update_accumulation_rate(model)
    update_basal_melt(model)
    update_weertman_c(model)
    update_dsdh(model)


def post_solve_steps(model):
    """update_state.jl:17-19: h-grid velocities, dh/dt, wavelet coarse space."""
    update_velocities_on_h_grid(model)
    update_dhdt(model)
    update_wavelets(model)


def update_state(model):
    """update_state!(model) (src/Models/update_state.jl:7-42)."""
    pre_solve(model)
    update_velocities(model)
    post_solve_steps(model)
    return model


class Simulation:
    """Mirror of WAVI.Simulation (src/Simulations/Simulation.jl:24-52) with its output files but without
    checkpoints or pickup."""

    def __init__(self, model: Model, timestepping_params: TimesteppingParams, output_params: OutputParams = None):
        self.model = model
        self.timestepping_params = timestepping_params
        self.output_params = output_params
        if output_params is not None:
            output_params.set_n_iter_out(timestepping_params.dt, timestepping_params.n_iter_total)
        self.n_iter = 0
        self.time = 0.0
        model.params.dt = timestepping_params.dt  # set_dt_in_model! (Simulation.jl:56-59)


def update_thickness(sim):
    """update_thickness! (src/Simulations/run_simulation.jl:24-42), evolveShelves = true branch."""
    model, dt = sim.model, sim.timestepping_params.dt
    f, m = model.fields, model.h_mask
    if not model.params.evolveShelves:
        raise NotImplementedError("evolveShelves = false is outside the velocity-solve path")
    hup = np.zeros_like(f["h"])
    hup[m] = np.maximum(model.params.minimum_thickness - f["h"][m], dt * f["dhdt"][m])
    hup[model.h_isfixed] = 0.0
    f["h"][m] = f["h"][m] + hup[m]


def timestep(sim):
    update_state(sim.model)
    if sim.timestepping_params.step_thickness:
        update_thickness(sim)
    sim.n_iter += 1
    sim.time += sim.timestepping_params.dt


def _write_due_output(sim):
    """The output steps of run_simulation! after time step sim.n_iter (run_simulation.jl:85-94)."""
    from .io import write_output, write_vel
    op = sim.output_params
    if op is None:
        return
    if sim.n_iter % op.n_iter_out == 0:
        write_output(sim)
    if sim.n_iter == sim.timestepping_params.n_iter_total and op.dump_vel:
        write_vel(op.prefix, sim.model.fields["u"], sim.model.fields["v"])


def run_simulation(sim, callback=None):
    """run_simulation! (src/Simulations/run_simulation.jl:61-100) without checkpoints: the initial output
    when output_start is set, then each time step followed by its due outputs.  With a device-resident
    GPU spec and no callback, the steps between two outputs run as one wavi_run_device call."""
    tp, op = sim.timestepping_params, sim.output_params
    if op is not None and op.output_start and sim.n_iter == 0:
        from .io import write_output
        write_output(sim)
    ps = sim.model.parallel_spec
    on_device = (isinstance(ps, GPUParallelSpec) and ps.device_run and callback is None and tp.step_thickness)
    while sim.n_iter < tp.n_iter_total:
        if on_device:
            n = tp.n_iter_total - sim.n_iter
            if op is not None:
                n = min(n, op.n_iter_out - sim.n_iter % op.n_iter_out)
            _run_on_device(sim, n)
        else:
            timestep(sim)
            if callback is not None:
                callback(sim)
        _write_due_output(sim)
    if sim.output_params is not None:
        from .io import zip_output
        zip_output(sim)  # (zipping_output.jl:162-169; after the last step, run_simulation.jl:96-97)
    return sim


def _assign_field(f, name, host):
    """Put a host copy of a field back into the model in place, so references to the field (such as an
    OutputParams output) stay valid; a field of another shape, or a new one, is replaced."""
    cur = f.get(name)
    if isinstance(cur, np.ndarray) and cur.shape == host.shape and cur.flags.writeable:
        cur[...] = host
    else:
        f[name] = host


def _run_on_device(sim, n):
    """n time steps of update_state! + update_thickness! in one wavi_run_device call: the fields go to the
    device once and come back once."""
    import torch
    model, dt = sim.model, sim.timestepping_params.dt
    if not model.params.evolveShelves:
        raise NotImplementedError("evolveShelves = false is outside the velocity-solve path")
    f = model.fields
    dev = lambda a, t=np.float64: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=t).ravel(order="F"))).cuda()
    t = {k: dev(f[k], np.uint8 if k in ("wu_mask", "wv_mask") else np.float64) for k in gpu.ALL_FIELDS}
    outs = {k: torch.zeros(model.grid.nx * model.grid.ny, dtype=torch.float64, device="cuda")
            for k in ("dhdt", "u_h", "v_h", "u_bed", "v_bed", "u_surf", "v_surf")}
    stats, (nwu, nwv) = _solver_for(model).run_device(model.params, dt, n, dev(f["b"]), dev(model.weertman_c_param),
                                                       dev(model.accumulation_param), dev(model.h_isfixed, np.uint8),
                                                       model.melt_rate, t, outputs=outs)
    for k in gpu.ALL_FIELDS:
        if k in ("wu_correction_coarse", "wv_correction_coarse"):
            continue
        _assign_field(f, k, t[k].cpu().numpy().reshape(np.asarray(f[k]).shape, order="F"))
    f["wu_correction_coarse"] = np.zeros(nwu)  # update_wavelets! restarts the coarse cache
    f["wv_correction_coarse"] = np.zeros(nwv)
    shape = (model.grid.nx, model.grid.ny)
    _assign_field(f, "dhdt", outs["dhdt"].cpu().numpy().reshape(shape, order="F"))
    for key, name in (("u_h", "uh"), ("v_h", "vh"), ("u_bed", "ub"), ("v_bed", "vb"), ("u_surf", "us"), ("v_surf", "vs")):
        if name in f:
            _assign_field(f, name, outs[key].cpu().numpy().reshape(shape, order="F"))
    model.last_stats = stats
    sim.n_iter += n
    sim.time += n * dt
    return sim
