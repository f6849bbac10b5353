"""ctypes mirror of include/wavi_gpu.h and the loader of libwavi_gpu.so.

The structs here are byte-for-byte the C structs of the header; a test checks their sizes and field
offsets against the compiled library (``wavi_abi_layout``).  Loading fails loudly: there is no CPU
fallback for the velocity solve.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwavi_gpu.so")

WAVI_ABI_VERSION = 5

STATUS = {
    0: "WAVI_OK", -1: "WAVI_ERR_ARGUMENT", -2: "WAVI_ERR_CUDA", -3: "WAVI_ERR_NONFINITE",
    -4: "WAVI_ERR_NOT_CONVERGED", -5: "WAVI_ERR_COARSE_CAP", -6: "WAVI_ERR_WATCHDOG",
    -7: "WAVI_ERR_NO_DEVICE", -8: "WAVI_ERR_ALLOC",
}
SOFT_STATUS = (-4, -5)  # results are written; mirrors the reference's silent stop at maxiter

PRECISION_FP64 = 0
PRECISION_MIXED = 1

COARSE_SOLVERS = {"auto": 0, "cg": 1, "srcg": 2, "srcg_jacobi": 3, "srcg_chebyshev": 4, "pipelined_chebyshev": 5}  # wavi_coarse_solver
COARSE_SOLVER_NAMES = {v: k for k, v in COARSE_SOLVERS.items()}
COARSE_SUMS = {"default": 0, "float_float": 1, "fp64": 2, "fp64_solve": 3}  # wavi_coarse_sums
VISCOSITY = {"default": 0, "fp32": 1, "fp64": 2}  # wavi_viscosity
PICARD_ACCEL = {"auto": 0, "plain": 1, "anderson": 2}  # wavi_picard_accel
PICARD_ACCEL_NAMES = {v: k for k, v in PICARD_ACCEL.items()}
COARSE_FORCING = {"auto": 0, "fixed": 1, "adaptive": 2}  # wavi_coarse_forcing
COARSE_FORCING_NAMES = {v: k for k, v in COARSE_FORCING.items()}
ADJOINT_PRECOND = {"auto": 0, "fp64": 1, "fp32": 2}  # wavi_adjoint_precond

_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


class GridDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nsigma", C.c_int32), ("reserved0", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double),
        ("sigma", _dp), ("quadrature_weights", _dp),
        ("h_mask", _u8p), ("u_iszero", _u8p), ("v_iszero", _u8p), ("u_isfixed", _u8p), ("v_isfixed", _u8p),
    ]


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dt", "g", "density_ice", "density_ocean", "gas_const",
        "glen_a_activation_energy", "glen_temperature_ref", "glen_n", "glen_reg_strain_rate",
        "weertman_m", "weertman_reg_speed", "sea_level_wrt_geoid", "minimum_thickness", "small_haf")] + [
        ("evolve_shelves", C.c_int32), ("reserved0", C.c_int32)]


class SolverParams(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "n_iter_viscosity", "maxiter_picard", "maxiter_coarse", "levels", "nsmooth", "stencil_margin")] + [
        (n, C.c_double) for n in ("tol_picard", "tol_coarse", "wavelet_threshold", "smoother_omega",
                                  "super_implicitness")]


class Options(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("use_graphs", C.c_int32),
                ("picard_test", C.c_int32), ("coarse_kernel", C.c_int32), ("coarse_solver", C.c_int32),
                ("stencil_kernel", C.c_int32), ("cheb_steps", C.c_int32), ("coarse_sums", C.c_int32),
                ("viscosity", C.c_int32), ("picard_accel", C.c_int32), ("anderson_depth", C.c_int32),
                ("coarse_forcing", C.c_int32), ("adjoint_precond", C.c_int32)]


FIELD_INPUTS = ("h", "s", "dsdh", "grounded_fraction", "weertman_c", "accumulation", "basal_melt",
                "gu_h", "gu_s", "gu_grounded_fraction", "gv_h", "gv_s", "gv_grounded_fraction", "glen_b")
FIELD_STATE = ("u", "v", "eta", "beta", "quad_f2")
FIELD_OUTPUTS = ("shelf_strain_rate", "av_speed", "bed_speed", "tau_bed", "eta_av", "quad_f1", "beta_eff",
                 "gu_beta_eff", "gv_beta_eff", "gu_residual", "gv_residual")


class Fields(C.Structure):
    _fields_ = ([(n, _dp) for n in FIELD_INPUTS] + [(n, _dp) for n in FIELD_STATE] +
                [("wu_mask", _u8p), ("wv_mask", _u8p),
                 ("wu_correction_coarse", _dp), ("wv_correction_coarse", _dp)] +
                [(n, _dp) for n in FIELD_OUTPUTS])


class Stats(C.Structure):
    _fields_ = [("status", C.c_int32), ("picard_iterations", C.c_int32),
                ("coarse_cg_iterations", C.c_int32), ("op_applications", C.c_int32),
                ("rel_residual", C.c_double), ("rel_update", C.c_double),
                ("algorithmic_bytes", C.c_double), ("elapsed_ms", C.c_double),
                ("kernel_launches", C.c_int32), ("host_syncs", C.c_int32),
                ("coarse_ms", C.c_double), ("coarse_solver", C.c_int32), ("coarse_launches", C.c_int32),
                ("coarse_kernel", C.c_int32), ("cheb_steps", C.c_int32), ("anderson_steps", C.c_int32),
                ("picard_accel", C.c_int32), ("coarse_forcing", C.c_int32), ("reserved1", C.c_int32)]


class OperatorDesc(C.Structure):
    """wavi_operator_desc: device coefficient arrays of the linearised operator (wavi_residual_noalloc)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("dx", C.c_double), ("dy", C.c_double),
                ("heta_h", C.c_void_p), ("heta_c", C.c_void_p), ("dimp", C.c_void_p), ("beta_m", C.c_void_p),
                ("h_m", C.c_void_p), ("inner", C.c_void_p)]


class StepInputs(C.Structure):
    _fields_ = [("bed", C.c_void_p), ("weertman_c", C.c_void_p), ("accumulation", C.c_void_p),
                ("h_isfixed", C.c_void_p), ("basal_melt_rate", C.c_double), ("reserved0", C.c_double)]


class StepOutputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("dhdt", "u_h", "v_h", "u_bed", "v_bed", "u_surf", "v_surf")] + [
        ("n_wu", C.c_int32), ("n_wv", C.c_int32), ("steps", C.c_int32), ("reserved0", C.c_int32)]


class AdjointStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("rel_residual", C.c_double),
                ("elapsed_ms", C.c_double)]


NOALLOC_MAX_TILES = 16384


class WaviError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def load_library(path=None):
    """Load libwavi_gpu.so (built in-tree by build.build_library).  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise WaviError(-7, f"{p} is not built; run __graft_entry__.build() (nvcc, sm_103a)")
    lib = C.CDLL(p)
    vp = C.c_void_p
    sig = {
        "wavi_abi_version": (C.c_int, []),
        "wavi_abi_struct_sizes": (C.c_int, [C.POINTER(C.c_int32), C.c_int]),
        "wavi_device_count": (C.c_int, []),
        "wavi_ctx_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(SolverParams), C.POINTER(Options),
                                      C.POINTER(vp)]),
        "wavi_ctx_destroy": (C.c_int, [vp]),
        "wavi_ctx_stream": (vp, [vp]),
        "wavi_last_error": (C.c_char_p, [vp]),
        "wavi_solve_velocities": (C.c_int, [vp, C.POINTER(Params), C.POINTER(Fields), C.POINTER(Stats)]),
        "wavi_solve_velocities_device": (C.c_int, [vp, C.POINTER(Params), C.POINTER(Fields),
                                                   C.POINTER(Stats)]),
        "wavi_relinearise_device": (C.c_int, [vp, C.POINTER(Params), C.POINTER(Fields)]),
        "wavi_apply_operator_device": (C.c_int, [vp, C.c_int, vp, vp]),
        "wavi_op_diagonal_device": (C.c_int, [vp, C.c_int, vp]),
        "wavi_coarse_diagonal_device": (C.c_int, [vp, C.c_int, vp]),
        "wavi_time_operator_device": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, C.POINTER(C.c_double)]),
        "wavi_time_relinearise_device": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "wavi_haar_device": (C.c_int, [vp, C.c_int, vp, vp, vp]),
        "wavi_update_wavelets_device": (C.c_int, [vp, vp, vp]),
        "wavi_residual_noalloc": (C.c_int, [C.POINTER(OperatorDesc), vp, vp, vp, vp, vp]),
        "wavi_selftest_watchdog": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "wavi_selftest_conversions": (C.c_int, [vp, C.c_longlong, C.POINTER(C.c_longlong)]),
        "wavi_adjoint_device": (C.c_int, [vp, C.POINTER(Params), vp, vp, vp, vp, C.c_double, C.c_int,
                                          C.POINTER(AdjointStats)]),
        "wavi_tangent_device": (C.c_int, [vp, C.POINTER(Params), vp, vp, vp, vp, C.c_double, C.c_int,
                                          C.POINTER(AdjointStats)]),
        "wavi_run_device": (C.c_int, [vp, C.POINTER(Params), C.c_double, C.c_int, C.POINTER(StepInputs),
                                      C.POINTER(Fields), C.POINTER(StepOutputs), C.POINTER(Stats)]),
        "wavi_ensemble_create": (C.c_int, [C.c_int, C.POINTER(GridDesc), C.POINTER(SolverParams), C.POINTER(Options),
                                           C.c_int, C.POINTER(vp)]),
        "wavi_ensemble_solve_device": (C.c_int, [vp, C.POINTER(Params), C.POINTER(Fields), C.POINTER(Stats)]),
        "wavi_ensemble_destroy": (C.c_int, [vp]),
        "wavi_ensemble_last_error": (C.c_char_p, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.wavi_abi_version() != WAVI_ABI_VERSION:
        raise WaviError(-1, "libwavi_gpu.so ABI version does not match wavi_gpu.h")
    if path is None:
        _lib = lib
    return lib


def header_symbols():
    """Names of the functions declared in include/*.h (checked against the library's exports)."""
    import re
    root = os.path.dirname(HERE)
    names = []
    inc = os.path.join(root, "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            txt = open(os.path.join(inc, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b(wavi_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))
