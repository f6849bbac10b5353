"""Python binding of libwavi_gpu.so's velocity solve (include/wavi_gpu.h).

``VelocitySolver`` owns one wavi_ctx (one CUDA stream, all device buffers) for one grid.  ``solve``
takes host numpy arrays (the e2e path: copies in and out inside the call); ``solve_device`` takes
device tensors (anything with ``data_ptr()``), the path used when the fields already live in HBM.

Field names are those of ``wavi_fields``; arrays are float64, Fortran order, reference shapes.
There is no CPU fallback: construction raises if the library or a GPU is missing.
"""
import ctypes as C
import sys

import numpy as np

from . import abi

PRECISIONS = {"fp64": abi.PRECISION_FP64, "mixed": abi.PRECISION_MIXED}
COARSE_KERNEL_NAMES = {1: "persistent", 2: "iterations", 3: "persistent_global"}  # wavi_stats.coarse_kernel


def _shape_of(name, nx, ny, ns):
    if name in ("u", "gu_h", "gu_s", "gu_grounded_fraction", "gu_beta_eff", "gu_residual", "wu_mask"):
        return (nx + 1, ny)
    if name in ("v", "gv_h", "gv_s", "gv_grounded_fraction", "gv_beta_eff", "gv_residual", "wv_mask"):
        return (nx, ny + 1)
    if name in ("glen_b", "eta"):
        return (nx, ny, ns)
    if name in ("wu_correction_coarse", "wv_correction_coarse"):
        return None
    return (nx, ny)


ALL_FIELDS = abi.FIELD_INPUTS + abi.FIELD_STATE + ("wu_mask", "wv_mask", "wu_correction_coarse",
                                                   "wv_correction_coarse") + abi.FIELD_OUTPUTS


class VelocitySolver:
    """One GPU velocity-solve context (``wavi_ctx``) for a fixed grid and solver parameters."""

    COARSE_KERNELS = {"auto": 0, "persistent": 1, "iterations": 2, "persistent_global": 3}
    STENCIL_KERNELS = {"auto": 0, "tiled": 1, "streaming": 2}

    def __init__(self, grid, solver_params, precision="fp64", device=0, use_graphs=True, picard_test=0,
                 coarse_kernel="auto", coarse_solver="auto", stencil_kernel="auto", cheb_steps=0,
                 coarse_sums="default", viscosity="default", picard_accel="auto", anderson_depth=0,
                 coarse_forcing="auto", adjoint_precond="auto"):
        self.lib = abi.load_library()
        self.grid = grid
        self.nx, self.ny, self.ns = grid.nx, grid.ny, grid.nσ
        self.solver_params = solver_params
        self.precision = precision
        self._desc = grid.descriptor()
        self._sp = solver_params.to_c()
        self._opt = abi.Options(int(device), PRECISIONS[precision], 1 if use_graphs else 0, int(picard_test),
                                self.COARSE_KERNELS[coarse_kernel], abi.COARSE_SOLVERS[coarse_solver],
                                self.STENCIL_KERNELS[stencil_kernel], int(cheb_steps),
                                abi.COARSE_SUMS[coarse_sums], abi.VISCOSITY[viscosity],
                                abi.PICARD_ACCEL[picard_accel], int(anderson_depth),
                                abi.COARSE_FORCING[coarse_forcing], abi.ADJOINT_PRECOND[adjoint_precond])
        ctx = C.c_void_p()
        st = self.lib.wavi_ctx_create(C.byref(self._desc.desc), C.byref(self._sp), C.byref(self._opt), C.byref(ctx))
        if st != 0:
            raise abi.WaviError(st, self.lib.wavi_last_error(None).decode())
        self.ctx = ctx

    def close(self):
        if getattr(self, "ctx", None) and self.ctx.value:
            self.lib.wavi_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    __del__ = close

    def stream(self):
        """The context's cudaStream_t as an integer handle (for torch.cuda.ExternalStream)."""
        return self.lib.wavi_ctx_stream(self.ctx) or 0

    def _err(self, st):
        return abi.WaviError(st, self.lib.wavi_last_error(self.ctx).decode())

    def _after_caller(self):
        """Order the context's stream (a non-blocking stream of its own) after the work already queued on
        torch's current CUDA stream, so that device tensors a caller has just written with torch are
        complete before the library reads them and not overwritten after it writes them.  Nothing to do
        when torch is not in use (other callers order their streams themselves, wavi_ctx_stream)."""
        torch = sys.modules.get("torch")
        if torch is None or not torch.cuda.is_available():
            return
        cur = torch.cuda.current_stream()
        if cur.cuda_stream != self.stream():
            torch.cuda.ExternalStream(self.stream()).wait_stream(cur)

    # -- host arrays -------------------------------------------------------------------------------
    def _host_fields(self, fields):
        f = abi.Fields()
        keep = []
        for name in ALL_FIELDS:
            a = fields[name]
            shp = _shape_of(name, self.nx, self.ny, self.ns)
            if name in ("wu_mask", "wv_mask"):
                if a.dtype != np.uint8 and a.dtype != np.bool_:
                    raise TypeError(f"{name} must be bool/uint8")
                arr = np.asfortranarray(a).view(np.uint8) if a.dtype == np.bool_ else np.asfortranarray(a)
                ptr = arr.ctypes.data_as(C.POINTER(C.c_uint8))
            else:
                if a.dtype != np.float64:
                    raise TypeError(f"{name} must be float64")
                if shp is not None and a.shape != shp:
                    raise ValueError(f"{name}: shape {a.shape} != {shp}")
                if not a.flags.f_contiguous:
                    raise ValueError(f"{name} must be Fortran-contiguous (it is written in place)")
                arr = a
                ptr = arr.ctypes.data_as(C.POINTER(C.c_double))
            keep.append(arr)
            setattr(f, name, ptr)
        n_wu, n_wv = int(np.count_nonzero(fields["wu_mask"])), int(np.count_nonzero(fields["wv_mask"]))
        if fields["wu_correction_coarse"].size != n_wu or fields["wv_correction_coarse"].size != n_wv:
            raise ValueError("coarse corrections must have count(wavelet mask) entries")
        return f, keep

    def solve(self, params, fields):
        """update_velocities! on host arrays (modified in place).  Returns the stats dict."""
        f, keep = self._host_fields(fields)
        stats = abi.Stats()
        st = self.lib.wavi_solve_velocities(self.ctx, C.byref(params.to_c()), C.byref(f), C.byref(stats))
        if st != 0:
            raise self._err(st)
        return stats_dict(stats)

    # -- device tensors ----------------------------------------------------------------------------
    def _device_fields(self, tensors):
        return device_fields(tensors)

    def solve_device(self, params, tensors):
        """update_velocities! on device tensors (dict of name -> tensor with data_ptr()), in place."""
        f = self._device_fields(tensors)
        stats = abi.Stats()
        self._after_caller()
        st = self.lib.wavi_solve_velocities_device(self.ctx, C.byref(params.to_c()), C.byref(f), C.byref(stats))
        if st != 0:
            raise self._err(st)
        return stats_dict(stats)

    def relinearise_device(self, params, tensors):
        f = self._device_fields(tensors)
        self._after_caller()
        st = self.lib.wavi_relinearise_device(self.ctx, C.byref(params.to_c()), C.byref(f))
        if st != 0:
            raise self._err(st)

    def apply_operator_device(self, in_uv, out_uv, precision="fp64"):
        self._after_caller()
        st = self.lib.wavi_apply_operator_device(self.ctx, PRECISIONS[precision], C.c_void_p(in_uv.data_ptr()),
                                                 C.c_void_p(out_uv.data_ptr()))
        if st != 0:
            raise self._err(st)

    def time_operator_device(self, in_uv, out_uv, precision="fp64", repeats=200):
        """Mean duration (s) of one operator launch over `repeats` back-to-back launches (CUDA events)."""
        ms = C.c_double()
        self._after_caller()
        st = self.lib.wavi_time_operator_device(self.ctx, PRECISIONS[precision], C.c_void_p(in_uv.data_ptr()),
                                                C.c_void_p(out_uv.data_ptr()), int(repeats), C.byref(ms))
        if st != 0:
            raise self._err(st)
        return ms.value / 1e3

    def time_relinearise_device(self, repeats=20):
        """Mean durations (s) of one launch of the relinearisation's h-grid and u/v-grid kernels over
        `repeats` back-to-back launches each, on the fields of the last solve or relinearisation."""
        mh, muv = C.c_double(), C.c_double()
        self._after_caller()
        st = self.lib.wavi_time_relinearise_device(self.ctx, int(repeats), C.byref(mh), C.byref(muv))
        if st != 0:
            raise self._err(st)
        return mh.value / 1e3, muv.value / 1e3

    def op_diagonal_device(self, out_uv, precision="fp64"):
        self._after_caller()
        st = self.lib.wavi_op_diagonal_device(self.ctx, PRECISIONS[precision], C.c_void_p(out_uv.data_ptr()))
        if st != 0:
            raise self._err(st)

    # -- device time stepping --------------------------------------------------------------------
    def run_device(self, params, dt, nsteps, bed, weertman_c, accumulation, h_isfixed, melt_rate, tensors,
                   outputs=None):
        """nsteps of update_state! + update_thickness! on the device (wavi_run_device).  bed, weertman_c,
        accumulation (float64) and h_isfixed (uint8) are device tensors of nx*ny; tensors holds the model
        fields (modified in place: the state after the last step); outputs optionally maps dhdt, u_h, v_h,
        u_bed, v_bed, u_surf, v_surf to device tensors.  Returns (stats dict, (n_wu, n_wv))."""
        ins = abi.StepInputs(bed.data_ptr(), weertman_c.data_ptr(), accumulation.data_ptr(), h_isfixed.data_ptr(),
                             float(melt_rate), 0.0)
        outs = abi.StepOutputs()
        for k, t in (outputs or {}).items():
            setattr(outs, k, t.data_ptr())
        f = device_fields(tensors)
        stats = abi.Stats()
        self._after_caller()
        st = self.lib.wavi_run_device(self.ctx, C.byref(params.to_c()), float(dt), int(nsteps), C.byref(ins),
                                      C.byref(f), C.byref(outs), C.byref(stats))
        if st != 0:
            raise self._err(st)
        return stats_dict(stats), (outs.n_wu, outs.n_wv)

    # -- adjoint ---------------------------------------------------------------------------------
    def adjoint_device(self, params, dJ_du, dJ_dv, grad_logC, grad_logA, tol=1e-10, maxiter=400):
        """Gradient of J w.r.t. per-cell log C and log A at the last solve's fixed point, from dJ/du, dJ/dv
        (device tensors in reference shapes, flattened column-major); writes grad_logC, grad_logA (nx*ny)."""
        st = abi.AdjointStats()
        self._after_caller()
        r = self.lib.wavi_adjoint_device(self.ctx, C.byref(params.to_c()), C.c_void_p(dJ_du.data_ptr()),
                                         C.c_void_p(dJ_dv.data_ptr()), C.c_void_p(grad_logC.data_ptr()),
                                         C.c_void_p(grad_logA.data_ptr()), float(tol), int(maxiter), C.byref(st))
        if r != 0:
            raise self._err(r)
        return {"status": st.status, "iterations": st.iterations, "rel_residual": st.rel_residual,
                "elapsed_ms": st.elapsed_ms}

    def tangent_device(self, params, dlogC, dlogA, du, dv, tol=1e-10, maxiter=400):
        """(du, dv) = d(u, v)/d(log C, log A) · (dlogC, dlogA) at the last solve's fixed point."""
        st = abi.AdjointStats()
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
        self._after_caller()
        r = self.lib.wavi_tangent_device(self.ctx, C.byref(params.to_c()), ptr(dlogC), ptr(dlogA), ptr(du), ptr(dv),
                                         float(tol), int(maxiter), C.byref(st))
        if r != 0:
            raise self._err(r)
        return {"status": st.status, "iterations": st.iterations, "rel_residual": st.rel_residual,
                "elapsed_ms": st.elapsed_ms}

    def coarse_diagonal_device(self, out_uv, precision="fp64"):
        """diag(R A P) for the current coefficients and wavelet mask, on the full wavelet grids."""
        self._after_caller()
        st = self.lib.wavi_coarse_diagonal_device(self.ctx, PRECISIONS[precision], C.c_void_p(out_uv.data_ptr()))
        if st != 0:
            raise self._err(st)

    def selftest_conversions(self, n=1 << 26):
        """Compare the library's integer binary64 <-> binary32 conversions with the hardware ones over n
        hashed patterns of each width (wavi_selftest_conversions).  Returns the number of mismatches."""
        bad = C.c_longlong()
        st = self.lib.wavi_selftest_conversions(self.ctx, int(n), C.byref(bad))
        if st != 0:
            raise self._err(st)
        return bad.value

    def selftest_watchdog(self):
        """Run the bounded-wait self-test (wavi_selftest_watchdog): True if the wait gave up as designed."""
        fired = C.c_int(0)
        st = self.lib.wavi_selftest_watchdog(self.ctx, C.byref(fired))
        if st != 0:
            raise self._err(st)
        return bool(fired.value)

    def update_wavelets_device(self, in_uv, wmask_out):
        """update_wavelets! with the device time step's kernels: the context's wavelet mask from the float64
        velocities in_uv ([u | v]), copied to the uint8 device tensor wmask_out."""
        self._after_caller()
        st = self.lib.wavi_update_wavelets_device(self.ctx, C.c_void_p(in_uv.data_ptr()), C.c_void_p(wmask_out.data_ptr()))
        if st != 0:
            raise self._err(st)

    def haar_device(self, kind, in_uv, out_uv, mask_uv=None):
        m = C.c_void_p(mask_uv.data_ptr()) if mask_uv is not None else None
        self._after_caller()
        st = self.lib.wavi_haar_device(self.ctx, int(kind), C.c_void_p(in_uv.data_ptr()), C.c_void_p(out_uv.data_ptr()), m)
        if st != 0:
            raise self._err(st)


def device_fields(tensors):
    """wavi_fields of device pointers from a dict of name -> tensor (anything with data_ptr())."""
    f = abi.Fields()
    for name in ALL_FIELDS:
        ptr = tensors[name].data_ptr()
        if name in ("wu_mask", "wv_mask"):
            setattr(f, name, C.cast(C.c_void_p(ptr), C.POINTER(C.c_uint8)))
        else:
            setattr(f, name, C.cast(C.c_void_p(ptr), C.POINTER(C.c_double)))
    return f


def stats_dict(s):
    return {"status": s.status, "status_name": abi.STATUS.get(s.status, str(s.status)),
            "picard_iterations": s.picard_iterations, "coarse_cg_iterations": s.coarse_cg_iterations,
            "op_applications": s.op_applications, "rel_residual": s.rel_residual, "rel_update": s.rel_update,
            "algorithmic_bytes": s.algorithmic_bytes, "elapsed_ms": s.elapsed_ms,
            "kernel_launches": s.kernel_launches, "host_syncs": s.host_syncs, "coarse_ms": s.coarse_ms,
            "coarse_solver": abi.COARSE_SOLVER_NAMES.get(s.coarse_solver, s.coarse_solver),
            "coarse_launches": s.coarse_launches,
            "coarse_kernel": COARSE_KERNEL_NAMES.get(s.coarse_kernel, s.coarse_kernel), "cheb_steps": s.cheb_steps,
            "anderson_steps": s.anderson_steps,
            "picard_accel": abi.PICARD_ACCEL_NAMES.get(s.picard_accel, s.picard_accel),
            "coarse_forcing": abi.COARSE_FORCING_NAMES.get(s.coarse_forcing, s.coarse_forcing)}
