"""Host-side mirror of the reference's configuration API: Grid, Params, SolverParams,
TimesteppingParams and InitialConditions, with the same keyword names, defaults and error behaviour.

  Grid                src/Grid.jl:1-27, constructor :66-201, orientations2bc :211-221
  Params              src/Params.jl:1-25, constructor :59-110
  SolverParams        src/SolverParams.jl:2-13
  TimesteppingParams  src/TimesteppingParams.jl (compute_iterations_and_end_time :81-98)
  InitialConditions   src/InitialConditions.jl:27-34

Arrays follow the reference layout: Fortran (column-major) numpy arrays, x (first index) fastest.
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import abi


def orientations2bc(orientations, M, N):
    """An M x N Bool array with trues on the named edges (src/Grid.jl:211-221).

    As in the reference, "north" is the first row of the first index (x = x0 edge), "south" the last,
    "west" the first column (y = y0 edge) and "east" the last.
    """
    A = np.zeros((M, N), dtype=bool, order="F")
    for o in orientations:
        o = o.lower()
        if o == "north":
            A[0, :] = True
        if o == "south":
            A[-1, :] = True
        if o == "east":
            A[:, -1] = True
        if o == "west":
            A[:, 0] = True
    return A


def _as_bool(a, name):
    try:
        return np.asfortranarray(np.asarray(a).astype(bool))
    except Exception as e:  # pragma: no cover - mirrors the reference's ArgumentError
        raise ValueError(f"{name} must be Boolean (or equivalent)") from e


class Grid:
    """Mirror of WAVI.Grid (src/Grid.jl:66-201)."""

    def __init__(self, nx=80, ny=10, dx=8000.0, dy=8000.0, nσ=4, x0=0.0, y0=-40000.0, h_mask=None,
                 h_isfixed=None, u_iszero=None, v_iszero=None, u_isfixed=None, v_isfixed=None,
                 quadrature_weights=None, σ=None, basin_ID=None, nsigma=None, sigma=None):
        if nsigma is not None:
            nσ = nsigma
        if sigma is not None:
            σ = sigma
        for nm, v in (("nx", nx), ("ny", ny), ("nσ", nσ)):
            if not (isinstance(v, (int, np.integer)) and v > 1):
                raise ValueError(f"number of grid cells ({nm}) must a positive integer larger than one")
        self.nx, self.ny, self.nσ = int(nx), int(ny), int(nσ)
        self.dx, self.dy, self.x0, self.y0 = float(dx), float(dy), float(x0), float(y0)
        if isinstance(u_iszero, (list, tuple)):
            u_iszero = orientations2bc(u_iszero, nx + 1, ny)
        if isinstance(v_iszero, (list, tuple)):
            v_iszero = orientations2bc(v_iszero, nx, ny + 1)
        if isinstance(h_isfixed, (list, tuple)):
            h_isfixed = orientations2bc(h_isfixed, nx, ny)
        if isinstance(u_isfixed, (list, tuple)):
            u_isfixed = orientations2bc(u_isfixed, nx + 1, ny)
        if isinstance(v_isfixed, (list, tuple)):
            v_isfixed = orientations2bc(v_isfixed, nx, ny + 1)
        h_mask = np.ones((nx, ny), bool) if h_mask is None else h_mask
        h_isfixed = np.zeros((nx, ny), bool) if h_isfixed is None else h_isfixed
        u_iszero = np.zeros((nx + 1, ny), bool) if u_iszero is None else u_iszero
        v_iszero = np.zeros((nx, ny + 1), bool) if v_iszero is None else v_iszero
        u_isfixed = np.zeros((nx + 1, ny), bool) if u_isfixed is None else u_isfixed
        v_isfixed = np.zeros((nx, ny + 1), bool) if v_isfixed is None else v_isfixed
        basin_ID = np.ones((nx, ny)) if basin_ID is None else basin_ID
        checks = (("h_mask", h_mask, (nx, ny)), ("h_isfixed", h_isfixed, (nx, ny)),
                  ("u_iszero", u_iszero, (nx + 1, ny)), ("v_iszero", v_iszero, (nx, ny + 1)),
                  ("basin_ID", basin_ID, (nx, ny)), ("u_isfixed", u_isfixed, (nx + 1, ny)),
                  ("v_isfixed", v_isfixed, (nx, ny + 1)))
        for nm, a, shp in checks:
            if np.shape(a) != shp:
                raise ValueError(f"DimensionMismatch: {nm} size must be {shp}")
        self.h_mask = _as_bool(h_mask, "h_mask")
        self.h_isfixed = _as_bool(h_isfixed, "h_isfixed")
        self.u_iszero = _as_bool(u_iszero, "u_iszero")
        self.v_iszero = _as_bool(v_iszero, "v_iszero")
        self.u_isfixed = _as_bool(u_isfixed, "u_isfixed")
        self.v_isfixed = _as_bool(v_isfixed, "v_isfixed")
        self.basin_ID = np.asfortranarray(basin_ID, dtype=np.float64)
        i = np.arange(1, nx + 2)[:, None]
        j = np.arange(1, ny + 2)[None, :]
        self.xxh = np.asfortranarray(np.broadcast_to(x0 + (i[:nx] - 0.5) * dx, (nx, ny)))
        self.yyh = np.asfortranarray(np.broadcast_to(y0 + (j[:, :ny] - 0.5) * dy, (nx, ny)))
        self.xxu = np.asfortranarray(np.broadcast_to(x0 + (i - 1.0) * dx, (nx + 1, ny)))
        self.yyu = np.asfortranarray(np.broadcast_to(y0 + (j[:, :ny] - 0.5) * dy, (nx + 1, ny)))
        self.xxv = np.asfortranarray(np.broadcast_to(x0 + (i[:nx] - 0.5) * dx, (nx, ny + 1)))
        self.yyv = np.asfortranarray(np.broadcast_to(y0 + (j - 1.0) * dy, (nx, ny + 1)))
        self.xxc = np.asfortranarray(np.broadcast_to(x0 + i[:nx - 1] * dx, (nx - 1, ny - 1)))
        self.yyc = np.asfortranarray(np.broadcast_to(y0 + j[:, :ny - 1] * dy, (nx - 1, ny - 1)))
        if σ is None:
            σ = np.linspace(0.0, 1.0, nσ)
        σ = np.asarray(σ, dtype=np.float64)
        if σ.shape != (nσ,):
            raise ValueError("DimensionMismatch: number of sigma levels must match nσ")
        if not (σ[0] == 0.0 and σ[-1] == 1.0):
            raise ValueError("σ must start at 0 and end at 1")
        self.σ = σ
        self.ζ = 1.0 - σ
        if quadrature_weights is None:
            quadrature_weights = 0.5 * np.concatenate(([σ[1] - σ[0]], σ[2:] - σ[:-2], [σ[-1] - σ[-2]]))
        quadrature_weights = np.asarray(quadrature_weights, dtype=np.float64)
        if quadrature_weights.shape != (nσ,):
            raise ValueError("DimensionMismatch: quadrature weights must have size (nσ,)")
        self.quadrature_weights = quadrature_weights

    nsigma = property(lambda self: self.nσ)
    sigma = property(lambda self: self.σ)

    def descriptor(self):
        """A GridDesc (ctypes) whose pointers stay valid while the returned holder is alive."""
        return GridDescHolder(self)


class GridDescHolder:
    """Keeps the contiguous arrays behind a GridDesc alive."""

    def __init__(self, g: Grid):
        self.nx, self.ny, self.nsigma = g.nx, g.ny, g.nσ
        u8 = lambda a: np.asfortranarray(a, dtype=np.uint8)
        self._arrays = {
            "sigma": np.ascontiguousarray(g.σ, dtype=np.float64),
            "qw": np.ascontiguousarray(g.quadrature_weights, dtype=np.float64),
            "h_mask": u8(g.h_mask), "u_iszero": u8(g.u_iszero), "v_iszero": u8(g.v_iszero),
            "u_isfixed": u8(g.u_isfixed), "v_isfixed": u8(g.v_isfixed),
        }
        A = self._arrays
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        up = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint8))
        self.desc = abi.GridDesc(g.nx, g.ny, g.nσ, 0, g.dx, g.dy, dp(A["sigma"]), dp(A["qw"]),
                                 up(A["h_mask"]), up(A["u_iszero"]), up(A["v_iszero"]),
                                 up(A["u_isfixed"]), up(A["v_isfixed"]))


SEC_PER_YEAR = 3600 * 24 * 365.25


@dataclass
class Params:
    """Mirror of WAVI.Params (src/Params.jl:59-110).  accumulation_rate, glen_a_ref and weertman_c may
    be scalars or nx x ny arrays; Model broadcasts scalars (src/Models/Model.jl:60-79)."""
    g: float = 9.81
    density_ice: float = 918.0
    density_ocean: float = 1028.0
    gas_const: float = 8.314
    sec_per_year: float = SEC_PER_YEAR
    default_thickness: float = 100.0
    default_viscosity: float = 1.0e7
    default_temperature: float = 263.15
    default_damage: float = 0.0
    accumulation_rate: object = 0.0
    glen_a_activation_energy: float = 5.8631e+04
    glen_a_ref: object = 4.9e-16 * SEC_PER_YEAR * 1.0e-9
    glen_temperature_ref: float = 263.15
    glen_n: float = 3.0
    glen_reg_strain_rate: float = 1.0e-5
    weertman_c: object = 1.0e4
    weertman_m: float = 3.0
    weertman_reg_speed: float = 1.0e-5
    sea_level_wrt_geoid: float = 0.0
    minimum_thickness: float = 50.0
    evolveShelves: bool = True
    smallHAF: float = 1.0
    dt: float = 1.0  # the reference defaults dt to 1.0 until a Simulation sets it (Params.jl:83)

    def to_c(self) -> abi.Params:
        return abi.Params(self.dt, self.g, self.density_ice, self.density_ocean, self.gas_const,
                          self.glen_a_activation_energy, self.glen_temperature_ref, self.glen_n,
                          self.glen_reg_strain_rate, self.weertman_m, self.weertman_reg_speed,
                          self.sea_level_wrt_geoid, self.minimum_thickness, self.smallHAF,
                          1 if self.evolveShelves else 0, 0)


@dataclass
class SolverParams:
    """Mirror of WAVI.SolverParams (src/SolverParams.jl:2-13)."""
    n_iter_viscosity: int = 2
    tol_picard: float = 1e-5
    maxiter_picard: int = 30
    tol_coarse: float = 1e-5
    maxiter_coarse: int = 1000
    levels: int = 3
    wavelet_threshold: float = 10.0
    nsmooth: int = 5
    smoother_omega: float = 1.0
    stencil_margin: int = 3
    super_implicitness: float = 1.0

    def __post_init__(self):
        if self.n_iter_viscosity != 2:  # SolverParams.jl:3
            raise AssertionError("n_iter_viscosity == 2")

    def to_c(self) -> abi.SolverParams:
        return abi.SolverParams(self.n_iter_viscosity, self.maxiter_picard, self.maxiter_coarse, self.levels,
                                self.nsmooth, self.stencil_margin, self.tol_picard, self.tol_coarse,
                                self.wavelet_threshold, self.smoother_omega, self.super_implicitness)


@dataclass
class TimesteppingParams:
    """Mirror of WAVI.TimesteppingParams (src/TimesteppingParams.jl:43-98), without checkpoint paths."""
    niter0: int = 0
    dt: float = 1.0
    end_time: Optional[float] = None
    n_iter_total: Optional[int] = None
    step_thickness: bool = True

    def __post_init__(self):
        if not (self.dt > 0):
            raise ValueError("timestep dt must be a positive number")
        if self.n_iter_total is not None and self.end_time is not None:
            if not math.isclose(self.end_time, self.n_iter_total * self.dt, rel_tol=1.5e-8):
                raise ValueError("end_time and n_iter_total are incompatible")
        elif self.end_time is not None:
            self.n_iter_total = int(round(self.end_time / self.dt))
        elif self.n_iter_total is not None:
            self.end_time = self.dt * self.n_iter_total
        else:
            raise ValueError("You must pass at least one of end_time or n_iter_total")
        if not (self.n_iter_total > 0):
            raise ValueError("n_iter_total must be a positive integer")


@dataclass
class OutputParams:
    """Mirror of WAVI.OutputParams (src/OutputParams/OutputParams.jl:2-12, constructor :34-70).

    ``outputs`` maps each output name to the array written under it (a reference to a model field, read
    when the output is written, as the reference's named tuple of field references is); ``n_iter_out`` is
    set by the Simulation from the time step (set_n_iter_out!, Simulation.jl:62-66).  zip_format "nc"
    merges the output files into one NetCDF file at the end of run_simulation (io.zip_output)."""
    outputs: dict = field(default_factory=dict)
    output_freq: float = math.inf
    output_format: str = "jld2"
    prefix: str = "outfile"
    output_path: str = "./"
    dump_vel: bool = False
    zip_format: str = "none"
    output_start: bool = False
    n_iter_out: int = -1

    def __post_init__(self):
        import os
        if not (self.output_freq == math.inf or self.output_freq > 0):
            raise ValueError("output frequency must be positive or Inf")
        if not os.path.isdir(self.output_path):
            os.makedirs(self.output_path)
        if not self.output_path.endswith("/"):
            self.output_path = self.output_path + "/"
        if self.output_format not in ("jld2", "mat"):
            raise ValueError("Output format must be `jld2` or `mat`")
        if self.zip_format not in ("none", "nc"):
            self.zip_format = "none"

    def set_n_iter_out(self, dt, n_iter_total):
        """set_n_iter_out! (src/Simulations/Simulation.jl:62-66)."""
        self.n_iter_out = n_iter_total + 1 if self.output_freq == math.inf else int(round(self.output_freq / dt))
        return self


@dataclass
class InitialConditions:
    """Mirror of WAVI.InitialConditions (src/InitialConditions.jl:27-34); None means 'use the default'."""
    initial_thickness: Optional[np.ndarray] = None
    initial_grounded_fraction: Optional[np.ndarray] = None
    initial_u_veloc: Optional[np.ndarray] = None
    initial_v_veloc: Optional[np.ndarray] = None
    initial_viscosity: Optional[np.ndarray] = None
    initial_temperature: Optional[np.ndarray] = None
    initial_damage: Optional[np.ndarray] = None
