"""ctypes binding of the FP64 CPU oracle (oracle/wavi_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()`` to check its result and by
``bench.py`` for the CPU-baseline leg.  The product (the package and libwavi_gpu.so) never imports it.

Parity of the oracle itself is pinned against the reference's golden files (tests/golden/*.npz, made
from test/version_update_test_verification/*.jld2), its known-answer tests (pos_fraction, Kronecker
products, sigma quadrature) and its analytic iceberg steady state (test/verification_tests/iceberg_test.jl).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "wavi_oracle.cpp")
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    """Compile the oracle with g++ (no fused multiply-add contraction, so x86 and Arm agree)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", LIB, SRC]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, dp, u8p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint8)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [vp, vp, vp]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_field.restype = dp
        L.oracle_field.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int64)]
        L.oracle_mask.restype = u8p
        L.oracle_mask.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int64)]
        L.oracle_set_params.argtypes = [vp, vp, vp, C.c_double]
        for n in ("oracle_init_fields", "oracle_pre_solve", "oracle_update_velocities", "oracle_post_solve",
                  "oracle_update_state", "oracle_update_wavelets", "oracle_inner_update"):
            getattr(L, n).argtypes = [vp]
        L.oracle_update_thickness.argtypes = [vp, C.c_double]
        L.oracle_run.argtypes = [vp, C.c_int, C.c_double]
        L.oracle_apply_operator.argtypes = [vp, dp, dp, dp, dp]
        L.oracle_rhs.argtypes = [vp, dp, dp]
        L.oracle_op_diag.argtypes = [vp, dp, dp]
        L.oracle_haar.argtypes = [vp, C.c_int, C.c_int, dp, dp]
        L.oracle_vcycle.restype = C.c_int
        L.oracle_vcycle.argtypes = [vp, dp, dp, dp, dp]
        L.oracle_stats.argtypes = [vp, C.POINTER(C.c_int), dp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.oracle_cg_history.restype = C.c_int
        L.oracle_cg_history.argtypes = [vp, C.POINTER(C.c_int), C.c_int]
        L.oracle_picard_history.restype = C.c_int
        L.oracle_picard_history.argtypes = [vp, dp, dp, C.c_int]
        L.oracle_pos_fraction.argtypes = [C.c_int, C.c_int, dp, u8p, dp, dp, dp]
        L.oracle_kron_apply.argtypes = [C.c_int, C.c_int, dp, C.c_int, C.c_int, dp, dp, dp]
        L.oracle_set_coarse_variant.argtypes = [C.c_int]
        L.oracle_set_chebyshev.argtypes = [C.c_int, C.c_double]
        L.oracle_set_anderson.argtypes = [C.c_int, C.c_double]
        L.oracle_set_coarse_forcing.argtypes = [C.c_int]
        L.oracle_coarse_diag.argtypes = [vp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleModel:
    """A reference-model instance held by the C++ oracle.  Fields are numpy views of its storage."""

    SHAPES = None

    def __init__(self, grid_desc, params, solver_params, melt_m=0.0):
        L = lib()
        self._keep = grid_desc  # the descriptor's arrays must outlive oracle_create
        self.h = L.oracle_create(C.byref(grid_desc.desc), C.byref(params), C.byref(solver_params))
        if not self.h:
            raise ValueError("oracle_create rejected the grid")
        self.nx, self.ny, self.ns = grid_desc.nx, grid_desc.ny, grid_desc.nsigma
        self.params, self.solver_params = params, solver_params
        L.oracle_set_params(self.h, C.byref(params), C.byref(solver_params), melt_m)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    U_NAMES = ("u", "u_mask", "u_inner", "u_isfixed", "wu_mask")
    V_NAMES = ("v", "v_mask", "v_inner", "v_isfixed", "wv_mask")

    def _shape(self, name, n):
        nx, ny, ns = self.nx, self.ny, self.ns
        if name in ("coarse_b", "coarse_x0"):  # the last V-cycle's coarse problem, in the coarse order
            return (n,)
        if name.startswith(("gu_", "wu_")) or name in self.U_NAMES:
            shp = (nx + 1, ny)
        elif name.startswith(("gv_", "wv_")) or name in self.V_NAMES:
            shp = (nx, ny + 1)
        elif name in ("eta", "temperature", "damage", "glen_b"):
            shp = (nx, ny, ns)
        elif name in ("dneg_heta_c", "c_mask"):
            shp = (nx - 1, ny - 1)
        else:
            shp = (nx, ny)
        if int(np.prod(shp)) != n:
            raise ValueError(f"{name}: {n} elements do not fit {shp}")
        return shp

    def field(self, name):
        """Writable numpy view (Fortran order) of a float64 field."""
        n = C.c_int64()
        p = lib().oracle_field(self.h, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        flat = np.ctypeslib.as_array(p, shape=(n.value,))
        return flat.reshape(self._shape(name, n.value), order="F")

    def mask(self, name):
        n = C.c_int64()
        p = lib().oracle_mask(self.h, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        flat = np.ctypeslib.as_array(p, shape=(n.value,))
        return flat.reshape(self._shape(name, n.value), order="F")

    def set(self, name, value):
        f = self.field(name)
        f[...] = value

    def init_fields(self):
        lib().oracle_init_fields(self.h)

    def pre_solve(self):
        lib().oracle_pre_solve(self.h)

    def update_velocities(self):
        lib().oracle_update_velocities(self.h)

    def post_solve(self):
        lib().oracle_post_solve(self.h)

    def update_state(self):
        lib().oracle_update_state(self.h)

    def inner_update(self):
        lib().oracle_inner_update(self.h)

    def update_wavelets(self):
        lib().oracle_update_wavelets(self.h)

    def update_thickness(self, dt):
        lib().oracle_update_thickness(self.h, dt)

    def run(self, nsteps, dt):
        lib().oracle_run(self.h, int(nsteps), float(dt))

    def stats(self):
        p, r, cg, ops = C.c_int(), C.c_double(), C.c_int64(), C.c_int64()
        lib().oracle_stats(self.h, C.byref(p), C.byref(r), C.byref(cg), C.byref(ops))
        cap = 4096
        hist = (C.c_int * cap)()
        n = lib().oracle_cg_history(self.h, hist, cap)
        rel, upd = (C.c_double * cap)(), (C.c_double * cap)()
        npic = lib().oracle_picard_history(self.h, rel, upd, cap)
        return {"picard_iterations": p.value, "rel_residual": r.value, "coarse_cg_iterations": cg.value,
                "op_applications": ops.value, "cg_history": list(hist[:min(n, cap)]),
                "rel_history": list(rel[:min(npic, cap)]), "update_history": list(upd[:min(npic, cap)])}

    def apply_operator(self, u, v):
        u = np.asfortranarray(u, dtype=np.float64)
        v = np.asfortranarray(v, dtype=np.float64)
        fu, fv = np.zeros_like(u), np.zeros_like(v)
        lib().oracle_apply_operator(self.h, _dp(u), _dp(v), _dp(fu), _dp(fv))
        return fu, fv

    def rhs(self):
        bu = np.zeros((self.nx + 1, self.ny), order="F")
        bv = np.zeros((self.nx, self.ny + 1), order="F")
        lib().oracle_rhs(self.h, _dp(bu), _dp(bv))
        return bu, bv

    def op_diag(self):
        du = np.zeros((self.nx + 1, self.ny), order="F")
        dv = np.zeros((self.nx, self.ny + 1), order="F")
        lib().oracle_op_diag(self.h, _dp(du), _dp(dv))
        return du, dv

    def haar(self, grid, which, x):
        """grid 0 = u, 1 = v; which 0 = idwt, 1 = idwtᵀ, 2 = dwt."""
        x = np.asfortranarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        lib().oracle_haar(self.h, grid, which, _dp(x), _dp(y))
        return y

    def vcycle(self, ru, rv):
        ru = np.asfortranarray(ru, dtype=np.float64)
        rv = np.asfortranarray(rv, dtype=np.float64)
        cu, cv = np.zeros_like(ru), np.zeros_like(rv)
        it = lib().oracle_vcycle(self.h, _dp(ru), _dp(rv), _dp(cu), _dp(cv))
        return cu, cv, it

    def coarse_diag(self):
        """diag(R A P) on the full wavelet grids (zero off the coarse space)."""
        du = np.zeros((self.nx + 1, self.ny), order="F")
        dv = np.zeros((self.nx, self.ny + 1), order="F")
        lib().oracle_coarse_diag(self.h, _dp(du), _dp(dv))
        return du, dv


COARSE_VARIANTS = {"cg": 0, "srcg": 2, "srcg_jacobi": 3, "srcg_chebyshev": 4, "pipelined_chebyshev": 5}


def set_coarse_variant(name):
    """Coarse solve of every later oracle V-cycle: the reference's cg! ("cg", the default) or a restatement
    of one of the GPU library's opt-in coarse solvers."""
    lib().oracle_set_coarse_variant(COARSE_VARIANTS[name])


CHEB_DEFAULT = (3, 120.0)


def set_chebyshev(steps=CHEB_DEFAULT[0], ratio=CHEB_DEFAULT[1]):
    """The Chebyshev preconditioner of the "srcg_chebyshev" and "pipelined_chebyshev" variants: steps per
    application (odd) and the ratio b/a of its interval [a, b].  The defaults are the GPU library's."""
    lib().oracle_set_chebyshev(int(steps), float(ratio))


ANDERSON_DEFAULT = (3, 0.3)


def set_anderson(depth=0, start_rel=ANDERSON_DEFAULT[1]):
    """Anderson acceleration of every later oracle solve's Picard loop: depth 0 (the reference's plain
    iteration, the default) or 1..5 columns, from the first Picard iteration whose relative residual is
    below start_rel.  Restates the GPU library's opt-in WAVI_PICARD_ANDERSON."""
    lib().oracle_set_anderson(int(depth), float(start_rel))


def set_coarse_forcing(on=False):
    """The coarse CG's relative tolerance in every later V-cycle: the reference's tol_coarse (False, the
    default) or max(tol_coarse, min(0.1, 0.1 x the Picard relative residual)) (True).  Restates the GPU
    library's opt-in WAVI_FORCING_ADAPTIVE."""
    lib().oracle_set_coarse_forcing(1 if on else 0)


def pos_fraction(z, mask=None):
    z = np.asfortranarray(z, dtype=np.float64)
    m, n = z.shape
    mk = np.asfortranarray(np.ones((m, n), np.uint8) if mask is None else np.asarray(mask, np.uint8))
    af = np.zeros((m, n), order="F")
    afu = np.zeros((m + 1, n), order="F")
    afv = np.zeros((m, n + 1), order="F")
    lib().oracle_pos_fraction(m, n, _dp(z), mk.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(af), _dp(afu), _dp(afv))
    return af, afu, afv


def kron_apply(A, B, x):
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(A.shape[0] * B.shape[0])
    lib().oracle_kron_apply(A.shape[0], A.shape[1], _dp(A), B.shape[0], B.shape[1], _dp(B), _dp(x), _dp(y))
    return y


def build_model(grid, bed, params, solver_params, initial_conditions=None, melt_m=0.0):
    """Restates Model(...) (src/Models/Model.jl:34-93) with check_initial_conditions
    (src/Models/model_utilities.jl:7-60) and setup_fields (src/Fields/Fields.jl:26-115) for the oracle.

    ``grid``, ``params``, ``solver_params`` and ``initial_conditions`` are the host package's config
    objects (plain data); ``bed`` is an nx x ny array or a function of (x, y).
    """
    nx, ny, ns = grid.nx, grid.ny, grid.nσ
    ic = initial_conditions
    desc = grid.descriptor()
    m = OracleModel(desc, params.to_c(), solver_params.to_c(), melt_m)

    def pick(val, default):
        return default if val is None else np.asarray(val, dtype=np.float64)

    bed_arr = np.vectorize(bed)(grid.xxh, grid.yyh) if callable(bed) else np.asarray(bed, np.float64)
    m.set("b", bed_arr)
    m.set("h", pick(ic and ic.initial_thickness, params.default_thickness * np.ones((nx, ny))))
    m.set("grounded_fraction", pick(ic and ic.initial_grounded_fraction, np.ones((nx, ny))))
    m.set("u", pick(ic and ic.initial_u_veloc, np.zeros((nx + 1, ny))))
    m.set("v", pick(ic and ic.initial_v_veloc, np.zeros((nx, ny + 1))))
    m.set("eta", pick(ic and ic.initial_viscosity, params.default_viscosity * np.ones((nx, ny, ns))))
    m.set("temperature", pick(ic and ic.initial_temperature, params.default_temperature * np.ones((nx, ny, ns))))
    m.set("damage", pick(ic and ic.initial_damage, params.default_damage * np.ones((nx, ny, ns))))
    m.set("glen_a_ref", np.broadcast_to(np.asarray(params.glen_a_ref, np.float64), (nx, ny)))
    m.set("weertman_c_param", np.broadcast_to(np.asarray(params.weertman_c, np.float64), (nx, ny)))
    m.set("accumulation_param", np.broadcast_to(np.asarray(params.accumulation_rate, np.float64), (nx, ny)))
    m.init_fields()
    return m
