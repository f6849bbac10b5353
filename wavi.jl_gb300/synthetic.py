"""Seeded synthetic inputs for the benchmark and parity workloads.

There is no external benchmark data for this path: the synthetic channel follows the MISMIP+ geometry
the reference ships (``mismip_plus_bed``, src/utilities.jl:401-409, used by test_version_updates.jl and
example_drivers/MISMIP_PLUS) with seeded roughness, thickness noise, and, for the large domain, a
log-normal drag field and a vertical temperature profile.

  channel_c1   80 x 10 at 8 km, nσ = 4                (time-stepping case)
  channel_c2   640 x 80 at 1 km, nσ = 4               (single converged solve; the benchmark workload)
  channel_c3   2560 x 320 at 250 m, nσ = 8            (large single domain)
  ensemble     ragged members, dx = dy = 2 km, nσ = 4
"""
import numpy as np

from .config import Grid, InitialConditions, Params, SolverParams


def mismip_plus_bed(x, y):
    """MISMIP+ bed elevation (src/utilities.jl:401-409), vectorised."""
    xbar = 300000.0
    b0, b2, b4, b6 = -150.0, -728.8, 343.91, -50.75
    wc, fc, dc = 24000.0, 4000.0, 500.0
    xs = x / xbar
    bx = b0 + b2 * xs ** 2 + b4 * xs ** 4 + b6 * xs ** 6
    by = dc * ((1 + np.exp(-2 * (y - wc) / fc)) ** (-1) + (1 + np.exp(2 * (y + wc) / fc)) ** (-1))
    return np.maximum(bx + by, -720.0)


def channel_bed(grid, seed=0, roughness=20.0, xscale=1.0, yscale=1.0):
    """MISMIP+ channel on the grid's h points plus N(0, roughness) per cell, re-clipped at -720 m."""
    rng = np.random.default_rng(seed)
    b = mismip_plus_bed(grid.xxh * xscale, grid.yyh * yscale)
    b = b + roughness * rng.standard_normal(b.shape)
    return np.asfortranarray(np.maximum(b, -720.0))


def noisy_thickness(shape, seed, mean=300.0, rel=0.05):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(mean * (1.0 + rng.uniform(-rel, rel, size=shape)))




def gaussian_filter_periodic(z, sigma_cells):
    """Gaussian smoothing by FFT (periodic), renormalised to unit variance."""
    nx, ny = z.shape
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.fftfreq(ny)[None, :]
    g = np.exp(-2.0 * (np.pi ** 2) * (sigma_cells ** 2) * (kx ** 2 + ky ** 2))
    out = np.real(np.fft.ifft2(np.fft.fft2(z) * g))
    out = (out - out.mean()) / out.std()
    return out


def _grid(nx, ny, dx, ns):
    return Grid(nx=nx, ny=ny, nσ=ns, dx=dx, dy=dx, x0=0.0, y0=-40000.0 * (ny * dx) / 80000.0,
                u_iszero=["north"], v_iszero=["west", "east"])


def channel_case(nx, ny, dx, ns, seed_bed=0, seed_h=1, tol_picard=1e-5, maxiter_picard=30, C=1.0e4,
                 temperature=None, accumulation=0.3):
    """A channel configuration: (grid, bed, params, solver_params, initial_conditions).

    Physics as the benchmark configurations state: Glen n = 3 with A = 2e-17 Pa^-3 yr^-1 (glen_a_ref at
    the reference temperature), Weertman m = 3, C = 1e4 (or a per-cell field), accumulation 0.3 m/yr.
    """
    g = _grid(nx, ny, dx, ns)
    bed = refined_channel_bed(g, seed=seed_bed)
    p = Params(accumulation_rate=accumulation, glen_a_ref=2.0e-17, weertman_c=C, default_temperature=263.15)
    sp = SolverParams(tol_picard=tol_picard, maxiter_picard=maxiter_picard)
    ic = InitialConditions(initial_thickness=np.asfortranarray(300.0 * (1.0 + template_field((nx, ny), seed_h, "uniform"))),
                           initial_temperature=temperature)
    return g, bed, p, sp, ic


TEMPLATE = (80, 10)  # the 8 km channel grid on which every seeded field is drawn


def template_field(shape, seed, kind, amplitude=0.05):
    """A seeded field drawn on the 80 x 10 (8 km) template grid — U(-amplitude, amplitude) ('uniform') or
    N(0, amplitude) ('normal') per template cell — and interpolated bilinearly to the cell centres of an
    nx x ny grid covering the same 640 x 80 km.  On the template grid itself it is the raw draw, so the
    8 km case and its refinements share one geometry."""
    rng = np.random.default_rng(seed)
    z = rng.uniform(-amplitude, amplitude, size=TEMPLATE) if kind == "uniform" else amplitude * rng.standard_normal(TEMPLATE)
    if tuple(shape) == TEMPLATE:
        return np.asfortranarray(z)
    return _bilinear(z, shape)


def _bilinear(z, shape):
    nx, ny = shape
    cx, cy = z.shape
    xs = (np.arange(nx) + 0.5) * cx / nx - 0.5
    ys = (np.arange(ny) + 0.5) * cy / ny - 0.5
    x0 = np.clip(np.floor(xs).astype(int), 0, cx - 1)
    y0 = np.clip(np.floor(ys).astype(int), 0, cy - 1)
    x1 = np.clip(x0 + 1, 0, cx - 1)
    y1 = np.clip(y0 + 1, 0, cy - 1)
    fx = np.clip(xs - x0, 0.0, 1.0)[:, None]
    fy = np.clip(ys - y0, 0.0, 1.0)[None, :]
    out = ((1 - fx) * (1 - fy) * z[x0][:, y0] + fx * (1 - fy) * z[x1][:, y0] +
           (1 - fx) * fy * z[x0][:, y1] + fx * fy * z[x1][:, y1])
    return np.asfortranarray(out)


def refined_channel_bed(grid, seed=0, roughness=20.0):
    """The MISMIP+ channel on the grid's h points plus 20 m Gaussian roughness drawn on the 8 km
    template (seed 0) and refined, re-clipped at -720 m."""
    b = mismip_plus_bed(grid.xxh * (640000.0 / (grid.nx * grid.dx)), grid.yyh * (80000.0 / (grid.ny * grid.dy)))
    b = b + template_field((grid.nx, grid.ny), seed, "normal", amplitude=roughness)
    return np.asfortranarray(np.maximum(b, -720.0))


def channel_c1(**kw):
    return channel_case(80, 10, 8000.0, 4, **kw)


def channel_c2(**kw):
    return channel_case(640, 80, 1000.0, 4, **kw)


def channel_c3(**kw):
    """2560 x 320 at 250 m, nσ = 8; log-normal C (median 1e4, σ_log 0.5, 20 km correlation, seed 3);
    temperature linear in σ from 268 K at the bed to 243 K at the surface."""
    nx, ny, dx, ns = 2560, 320, 250.0, 8
    rng = np.random.default_rng(3)
    z = gaussian_filter_periodic(rng.standard_normal((nx, ny)), 20000.0 / dx)
    C = np.asfortranarray(np.exp(np.log(1.0e4) + 0.5 * z))
    sigma = np.linspace(0.0, 1.0, ns)
    T = 243.0 + (268.0 - 243.0) * (1.0 - sigma)  # σ = 0 at the bed (ζ = 1), σ = 1 at the surface
    temp = np.asfortranarray(np.broadcast_to(T[None, None, :], (nx, ny, ns)).copy())
    return channel_case(nx, ny, dx, ns, C=C, temperature=temp, **kw)


def ensemble_members(n=256, seed=6, tol_picard=1e-6, maxiter_picard=100):
    """The ragged ensemble: n independent channel domains at dx = dy = 2 km, nσ = 4, with nx ~ U{64..512},
    ny ~ U{16..128}, C ~ log-U(3e3, 3e4) and accumulation ~ U(0.1, 0.5) drawn from `seed`.  Each member
    is the MISMIP+ channel scaled to its own extent with its own roughness (seed 1000 + k) and thickness
    noise (seed 2000 + k), both drawn on the 8 km template and refined, as for the 640 x 80 case.
    Returns a list of (grid, bed, params, solver_params, initial_conditions)."""
    rng = np.random.default_rng(seed)
    nxs = rng.integers(64, 513, size=n)
    nys = rng.integers(16, 129, size=n)
    cs = np.exp(rng.uniform(np.log(3.0e3), np.log(3.0e4), size=n))
    accs = rng.uniform(0.1, 0.5, size=n)
    out = []
    for k in range(n):
        nx, ny = int(nxs[k]), int(nys[k])
        g = _grid(nx, ny, 2000.0, 4)
        bed = refined_channel_bed(g, seed=1000 + k)
        p = Params(accumulation_rate=float(accs[k]), glen_a_ref=2.0e-17, weertman_c=float(cs[k]),
                   default_temperature=263.15)
        sp = SolverParams(tol_picard=tol_picard, maxiter_picard=maxiter_picard)
        ic = InitialConditions(initial_thickness=np.asfortranarray(
            300.0 * (1.0 + template_field((nx, ny), 2000 + k, "uniform"))))
        out.append((g, bed, p, sp, ic))
    return out


def small_case(nx=24, ny=12, dx=4000.0, ns=4, seed=0, mask="full", fixed=False, **kw):
    """Small ragged test cases: masks 'full', 'disc' (a circular ice mask, calving fronts on all sides),
    optional Dirichlet lines (u_isfixed / v_isfixed) as in the reference's iceberg test."""
    rng = np.random.default_rng(seed)
    x0, y0 = 0.0, -0.5 * ny * dx
    h_mask = None
    if mask == "disc":
        xc, yc = 0.5 * nx * dx, 0.0
        xx = x0 + (np.arange(nx)[:, None] + 0.5) * dx
        yy = y0 + (np.arange(ny)[None, :] + 0.5) * dx
        h_mask = np.sqrt((xx - xc) ** 2 + (yy - yc) ** 2) < 0.45 * min(nx, ny) * dx
    u_isfixed = v_isfixed = None
    if fixed:
        u_isfixed = np.zeros((nx + 1, ny), bool)
        u_isfixed[nx // 2, :] = True
        v_isfixed = np.zeros((nx, ny + 1), bool)
        v_isfixed[:, ny // 2] = True
    g = Grid(nx=nx, ny=ny, nσ=ns, dx=dx, dy=dx, x0=x0, y0=y0, h_mask=h_mask,
             u_iszero=None if mask == "disc" else ["north"], v_iszero=None if mask == "disc" else ["west", "east"],
             u_isfixed=u_isfixed, v_isfixed=v_isfixed)
    bed = np.asfortranarray(mismip_plus_bed(g.xxh * (640000.0 / (nx * dx)), g.yyh * (80000.0 / (ny * dx)))
                            + 20.0 * rng.standard_normal((nx, ny)))
    h = np.asfortranarray(300.0 * (1.0 + rng.uniform(-0.05, 0.05, (nx, ny))))
    if h_mask is not None:
        h[~h_mask] = 0.0
    u0 = v0 = None
    if fixed:
        u0 = np.zeros((nx + 1, ny), order="F")
        u0[u_isfixed] = 5.0 - 6e-4 * g.yyu[u_isfixed] * 1e-3
        v0 = np.zeros((nx, ny + 1), order="F")
        v0[v_isfixed] = 3.0 + 6e-4 * g.xxv[v_isfixed] * 1e-3
    p = Params(accumulation_rate=0.3, glen_a_ref=2.0e-17, default_temperature=263.15)
    sp = SolverParams(**kw)
    ic = InitialConditions(initial_thickness=h, initial_u_veloc=u0, initial_v_veloc=v0)
    return g, bed, p, sp, ic


ICEBERG_DRIFT = (5.0, 3.0)           # m/yr in x and y
ICEBERG_ROTATION_PERIOD = 10000.0    # yr


def iceberg_case(maxiter_picard=1):
    """The reference's spinning, drifting iceberg (test/verification_tests/iceberg_test.jl:7-80): a 20 x 20
    grid of 5 km cells centred on the origin, a 200 m thick floating disc of radius 45 km over a 500 m
    deep bed, and the solid-body velocity (drift 5, 3 m/yr, one turn in 10 000 yr) imposed on the u points
    of the line x = 0 and the v points of the line y = 0.  Run to steady state (1000 yr of dt = 0.1, one
    Picard iteration per step) it meets the closed form of iceberg_analytic."""
    nx = ny = 20
    u_isfixed = np.zeros((nx + 1, ny), bool)
    u_isfixed[nx // 2, :] = True
    v_isfixed = np.zeros((nx, ny + 1), bool)
    v_isfixed[:, ny // 2] = True
    kw = dict(nx=nx, ny=ny, nσ=4, x0=-50000.0, y0=-50000.0, dx=5000.0, dy=5000.0, u_isfixed=u_isfixed,
              v_isfixed=v_isfixed)
    xxh = Grid(**kw).xxh
    yyh = Grid(**kw).yyh
    h_mask = np.sqrt(xxh ** 2 + yyh ** 2) < 45000
    g = Grid(h_mask=h_mask, **kw)
    h = np.zeros((nx, ny), order="F")
    h[h_mask] = 200.0
    sbu, sbv = _solid_body(g)
    u0 = np.zeros((nx + 1, ny), order="F")
    v0 = np.zeros((nx, ny + 1), order="F")
    u0[u_isfixed] = sbu[u_isfixed]
    v0[v_isfixed] = sbv[v_isfixed]
    ic = InitialConditions(initial_thickness=h, initial_u_veloc=u0, initial_v_veloc=v0)
    p = Params(accumulation_rate=0.3, default_temperature=265.700709)
    return g, np.full((nx, ny), -500.0, order="F"), p, SolverParams(maxiter_picard=maxiter_picard), ic


def _solid_body(g):
    rate = 2 * np.pi / ICEBERG_ROTATION_PERIOD
    return ICEBERG_DRIFT[0] - rate * g.yyu, ICEBERG_DRIFT[1] + rate * g.xxv


def iceberg_analytic(g, accumulation=0.3, glen_a=2.0e-17, density_ice=918.0, density_ocean=1028.0, gravity=9.81):
    """The iceberg's steady state (iceberg_test.jl:82-84): uniform thickness h0 at which the spreading of a
    floating slab balances the accumulation, and the solid-body velocity plus the radial spreading
    accumulation / (2 h0) times x (u) and y (v).  Returns (h0, u0, v0)."""
    h0 = ((36.0 * accumulation / glen_a) * (1.0 / (gravity * density_ice * (1 - density_ice / density_ocean))) ** 3) ** 0.25
    sbu, sbv = _solid_body(g)
    return h0, g.xxu * accumulation / (2.0 * h0) + sbu, g.yyv * accumulation / (2.0 * h0) + sbv


def relative_error(a, b, mask):
    """‖a − b‖ / ‖b‖ over the points of ``mask`` (iceberg_test.jl:85-90)."""
    b = np.broadcast_to(b, np.shape(a))
    return float(np.linalg.norm(a[mask] - b[mask]) / np.linalg.norm(b[mask]))
