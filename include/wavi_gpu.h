/*
 * wavi_gpu.h — C ABI of libwavi_gpu.so, the GB300 (sm_103a) backend for WAVI.jl's velocity solve.
 *
 * The library replaces one call of the reference: `update_velocities!(model)`
 * (src/Models/update_velocities.jl:11-29), the Picard loop around the matrix-free momentum operator
 * (src/utilities.jl:13-149) with the Haar-wavelet multigrid V-cycle and coarse conjugate-gradient solve
 * (src/Wavelets/update_preconditioners.jl:7-83, :153-216).  The reference reaches that call from
 * `update_model_velocities!` (src/Models/update_state.jl:154-157) and dispatches on the model's
 * parallel-spec type parameter (src/WAVI.jl:17-18, src/Models/Model.jl:1-8), so a Julia host binds these
 * entry points from a new `GPUParallelSpec <: AbstractParallelSpec` method of `update_velocities!`.
 *
 * Conventions
 *  - Every 2-D array is column-major with x (the first Julia index) fastest, exactly as the reference
 *    stores it: h grid nx*ny, u grid (nx+1)*ny, v grid nx*(ny+1), c grid (nx-1)*(ny-1),
 *    3-D sigma fields nx*ny*nsigma (src/Fields/*.jl).
 *  - Masks are one byte per point (Julia Array{Bool} layout): 0 = false, anything else = true.
 *  - Floating-point arrays are IEEE float64 on the host side of the boundary.
 *  - Every entry point returns 0 on success or a negative wavi_status; the message of the last failure
 *    of a context is available from wavi_last_error().  No entry point aborts, throws or traps.
 *  - A context owns one CUDA stream and its device buffers; it is not re-entrant, but distinct
 *    contexts may be used from distinct host threads at the same time.
 */
#ifndef WAVI_GPU_H
#define WAVI_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WAVI_ABI_VERSION 5

typedef enum wavi_status {
  WAVI_OK = 0,
  WAVI_ERR_ARGUMENT = -1,          /* bad sizes, null pointers, inconsistent masks */
  WAVI_ERR_CUDA = -2,              /* a CUDA runtime call failed (message holds cudaGetErrorString) */
  WAVI_ERR_NONFINITE = -3,         /* NaN/Inf met in a residual norm or a CG scalar */
  WAVI_ERR_NOT_CONVERGED = -4,     /* soft: Picard stopped at maxiter_picard; outputs are written */
  WAVI_ERR_COARSE_CAP = -5,        /* soft: the coarse CG stopped at maxiter_coarse; outputs are written */
  WAVI_ERR_WATCHDOG = -6,          /* a bounded device-side wait gave up */
  WAVI_ERR_NO_DEVICE = -7,         /* no usable CUDA device / extension not built for it */
  WAVI_ERR_ALLOC = -8              /* device or pinned allocation failed */
} wavi_status;

/* Precision modes of a context. */
typedef enum wavi_precision {
  WAVI_PRECISION_FP64 = 0,         /* the reference algorithm in float64 throughout (parity mode) */
  WAVI_PRECISION_MIXED = 1         /* float32 viscosity sweeps (per wavi_viscosity), operator coefficients
                                      and V-cycle (smoother, Haar transforms, coarse CG; its sums per
                                      wavi_coarse_sums); float64 right-hand side, Picard residual,
                                      convergence test and coarse-correction cache */
} wavi_precision;

/* Grid geometry and the masks that fix the problem's sparsity (src/Grid.jl:1-27, :66-201;
 * masks derived as in src/Fields/Fields.jl:26-35). */
typedef struct wavi_grid_desc {
  int32_t nx, ny, nsigma;
  int32_t reserved0;
  double dx, dy;
  const double* sigma;               /* nsigma, sigma[0] = 0, sigma[nsigma-1] = 1 */
  const double* quadrature_weights;  /* nsigma */
  const uint8_t* h_mask;             /* nx*ny */
  const uint8_t* u_iszero;           /* (nx+1)*ny */
  const uint8_t* v_iszero;           /* nx*(ny+1) */
  const uint8_t* u_isfixed;          /* (nx+1)*ny */
  const uint8_t* v_isfixed;          /* nx*(ny+1) */
} wavi_grid_desc;

/* Scalar physical parameters (src/Params.jl:1-25, defaults :59-110).  Array-valued members of the
 * reference's Params (accumulation_rate, glen_a_ref, weertman_c) travel as per-cell fields. */
typedef struct wavi_params {
  double dt, g, density_ice, density_ocean, gas_const;
  double glen_a_activation_energy, glen_temperature_ref, glen_n, glen_reg_strain_rate;
  double weertman_m, weertman_reg_speed, sea_level_wrt_geoid, minimum_thickness, small_haf;
  int32_t evolve_shelves;
  int32_t reserved0;
} wavi_params;

/* Solver parameters (src/SolverParams.jl:2-13). */
typedef struct wavi_solver_params {
  int32_t n_iter_viscosity;          /* the reference asserts == 2 */
  int32_t maxiter_picard;
  int32_t maxiter_coarse;
  int32_t levels;                    /* Haar levels; the transform acts on blocks of 2^(levels+1) */
  int32_t nsmooth;
  int32_t stencil_margin;
  double tol_picard, tol_coarse, wavelet_threshold, smoother_omega, super_implicitness;
} wavi_solver_params;

/* Options of a context (no counterpart in the reference: backend choices). */
typedef struct wavi_options {
  int32_t device;                    /* CUDA ordinal */
  int32_t precision;                 /* wavi_precision */
  int32_t use_graphs;                /* 1: capture each Picard iteration in a CUDA graph */
  int32_t picard_test;               /* 0: reference residual test ||b-Au||/||b|| < tol_picard;
                                        1: additionally require ||du||/||u|| <= tol_picard */
  int32_t coarse_kernel;             /* coarse CG: 0 = one persistent kernel per V-cycle (CG vectors in
                                        registers when the grid's tiles fit the device's resident CTAs,
                                        else in global memory); 1 = persistent (error if it cannot run);
                                        2 = per-iteration kernels; 3 = persistent, global-memory vectors */
  int32_t coarse_solver;             /* wavi_coarse_solver */
  int32_t stencil_kernel;            /* operator and smoother sweeps: 0 = by grid size (row-streaming from
                                        2^19 points of the (nx+1) x (ny+1) index space), 1 = shared-memory
                                        tiles, 2 = row-streaming */
  int32_t cheb_steps;                /* Chebyshev steps per preconditioner application of the Chebyshev
                                        coarse solvers: 0 = the default (5 in the register-resident
                                        single-reduction kernel, 3 in the global-memory and pipelined
                                        kernels); else odd, 1..15 */
  int32_t coarse_sums;               /* wavi_coarse_sums: how a mixed-precision coarse CG accumulates its
                                        dot products (FP64 contexts always sum in FP64) */
  int32_t viscosity;                 /* wavi_viscosity: precision of a mixed context's σ-level viscosity
                                        sweeps (FP64 contexts always sweep in FP64) */
  int32_t picard_accel;              /* wavi_picard_accel: the reference's Picard iteration, or Anderson
                                        acceleration of it (the mixed default) */
  int32_t anderson_depth;            /* columns of the Anderson acceleration: 0 = the default (3), else
                                        1..5 (ignored without WAVI_PICARD_ANDERSON) */
  int32_t coarse_forcing;            /* wavi_coarse_forcing: the coarse CG's tolerance, the reference's fixed
                                        tol_coarse or one that follows the Picard residual (the mixed
                                        default) */
  int32_t adjoint_precond;           /* wavi_adjoint_precond: precision of the V-cycle that preconditions the
                                        adjoint's and tangent linear's FGMRES */
} wavi_options;

/* Precision of the preconditioner V-cycle inside wavi_adjoint_device / wavi_tangent_device.  FGMRES is
 * flexible and keeps its residual and Krylov basis in FP64, so an FP32 V-cycle (on the FP32-rounded
 * coefficients of the linearisation) changes its iteration count, not the accuracy it stops at. */
typedef enum wavi_adjoint_precond {
  WAVI_ADJ_PRECOND_AUTO = 0,         /* FP32 where its coarse kernel fits the context's cooperative grid
                                        (16 x 16 coarse tiles), else FP64 */
  WAVI_ADJ_PRECOND_FP64 = 1,         /* the solve's own FP64 V-cycle */
  WAVI_ADJ_PRECOND_FP32 = 2          /* FP32 (an error where it cannot run) */
} wavi_adjoint_precond;

/* Relative tolerance of each V-cycle's coarse CG (abstol = tolerance x |b_c|, update_preconditioners.jl:73).
 * The reference's is tol_coarse in every Picard iteration.  The adaptive rule (not in the reference; the
 * forcing terms of inexact Newton methods, Eisenstat & Walker 1996) uses max(tol_coarse, min(0.1, 0.1 rel)),
 * rel the Picard iteration's relative residual: far from the fixed point the relinearisation, not the
 * linear solve, limits the next iterate, so the coarse CG stops sooner there; once rel <= 10 tol_coarse the
 * tolerance is the reference's.  Only in solves of maxiter_picard > 1.  On the channel and disc test cases
 * it saves 35-45 % of the coarse iterations at the same Picard count and accuracy. */
typedef enum wavi_coarse_forcing {
  WAVI_FORCING_AUTO = 0,             /* FP64: FIXED (the reference algorithm); mixed: ADAPTIVE */
  WAVI_FORCING_FIXED = 1,            /* tol_coarse */
  WAVI_FORCING_ADAPTIVE = 2          /* max(tol_coarse, min(0.1, 0.1 x the Picard relative residual)) in
                                        solves of maxiter_picard > 1; tol_coarse with maxiter_picard = 1 */
} wavi_coarse_forcing;

/* Acceleration of the Picard loop (update_velocities.jl:11-29).  The reference takes each relinearised
 * V-cycle correction as it is: a fixed-point iteration x -> g(x) = x + V(x)(b(x) - A(x) x) that converges
 * linearly.  Anderson acceleration (Walker & Ni 2011; not in the reference; the default of mixed contexts,
 * opt-in in FP64 ones, which run the reference algorithm) combines the last anderson_depth + 1 iterates by
 * least squares on their corrections, from the first Picard iteration whose relative residual is below
 * 0.3 (the iterations before it, from u = 0, are far from the fixed point).  The stopping rule is the reference's, applied to the accelerated iterates, so a converged
 * solve meets the same criterion; it reaches it in fewer Picard iterations (35-40 % fewer on the channel
 * and disc test cases) and, because the accelerated iterates converge faster than linearly, closer to
 * the fixed point (on the 8 km channel 1.1e-7 from the fully converged solution, where the reference's
 * iteration stops 1.8e-6 from it). */
typedef enum wavi_picard_accel {
  WAVI_PICARD_AUTO = 0,              /* FP64: PLAIN (the reference algorithm); mixed: ANDERSON */
  WAVI_PICARD_PLAIN = 1,             /* the reference's iteration */
  WAVI_PICARD_ANDERSON = 2           /* Anderson acceleration, anderson_depth columns */
} wavi_picard_accel;

/* Precision of the relinearisation's viscosity sweeps (update_velocities.jl:264-283) in a mixed context.
 * FP32 sweeps (the default) keep the mixed solve within ~1e-7 of the FP64 reference solve; FP64 sweeps cost
 * more (FP64 pow per σ level and cell) and bring it to ~1e-9 (on the 640 x 80 benchmark: 1.44e-7 against
 * 2.85e-9, at 51.6 against 55.5 ms per solve). */
typedef enum wavi_viscosity {
  WAVI_VISCOSITY_DEFAULT = 0,        /* WAVI_VISCOSITY_FP32 */
  WAVI_VISCOSITY_FP32 = 1,           /* FP32 sweeps (η, B, the stress term in float) */
  WAVI_VISCOSITY_FP64 = 2            /* FP64 sweeps; the V-cycle's coefficients are then rounded to FP32 */
} wavi_viscosity;

/* Accumulation of the mixed-precision coarse CG's dot products and CG scalars. */
typedef enum wavi_coarse_sums {
  WAVI_SUMS_DEFAULT = 0,             /* WAVI_SUMS_FLOAT_FLOAT */
  WAVI_SUMS_FLOAT_FLOAT = 1,         /* FP32 products, warp and CTA sums; float-float (~48-bit) grid sums
                                        and CG scalars */
  WAVI_SUMS_FP64 = 2,                /* every product and sum of the reductions, and the CG scalars, in FP64
                                        from the FP32 vectors; the single-reduction solvers on the
                                        register-resident 16 x 16 kernel only */
  WAVI_SUMS_FP64_SOLVE = 3           /* the whole coarse CG in FP64 — vectors, the coarse operator on the FP64
                                        coefficients, sums and scalars (the kernels of FP64 contexts) —
                                        inside the FP32 V-cycle, which hands it the restricted residual and
                                        takes back its solution; persistent coarse kernels, not the
                                        pipelined solver */
} wavi_coarse_sums;

/* Coarse solve of each V-cycle (R A P x = b_c, update_preconditioners.jl:54-83).  The reference calls
 * IterativeSolvers cg!; the single-reduction variants (not in the reference; Chronopoulos & Gear 1989)
 * compute both inner products of an iteration in one grid reduction, keep cg!'s stopping rule on the
 * unpreconditioned residual, and need the persistent coarse kernel. */
typedef enum wavi_coarse_solver {
  WAVI_COARSE_AUTO = 0,              /* FP64: cg!; mixed: SRCG_CHEBYSHEV (cg! with per-iteration kernels) */
  WAVI_COARSE_CG = 1,                /* the reference's cg! recurrence */
  WAVI_COARSE_SRCG = 2,              /* single-reduction CG, no preconditioner (same iterates as cg!) */
  WAVI_COARSE_SRCG_JACOBI = 3,       /* single-reduction CG preconditioned by diag(R A P) */
  WAVI_COARSE_SRCG_CHEBYSHEV = 4,    /* single-reduction CG preconditioned by cheb_steps (default 5 or 3)
                                        Chebyshev-accelerated Jacobi steps on [b/120, b],
                                        b = 1.15 lambda_max(diag(R A P)^-1 R A P) from power steps each
                                        V-cycle (12 in a solve's first, then 4, warm-started);
                                        persistent kernel (register-resident, or global-memory vectors
                                        on grids too large for that) */
  WAVI_COARSE_PIPELINED_CHEBYSHEV = 5 /* opt-in, never chosen by AUTO: pipelined CG (Ghysels & Vanroose
                                        2014) with the preconditioner of SRCG_CHEBYSHEV, whose grid
                                        reduction overlaps the iteration's preconditioner and operator;
                                        restarted from the true residual after every hundredfold fall of
                                        |r|; mixed precision, 16 x 16 tiles (levels <= 3), register-
                                        resident kernel */
} wavi_coarse_solver;

/* The model fields the velocity solve reads and writes (src/Models/update_velocities.jl:202-383,
 * src/Fields/HGrid.jl:1-38, UGrid.jl:1-29, VGrid.jl:1-29, SigmaGrid.jl, Wavelets/UWavelets.jl:2-15).
 * Pointers are host pointers for wavi_solve_velocities() and device pointers for
 * wavi_solve_velocities_device(). */
typedef struct wavi_fields {
  /* inputs, h grid */
  const double* h;                   /* gh.h */
  const double* s;                   /* gh.s */
  const double* dsdh;                /* gh.dsdh */
  const double* grounded_fraction;   /* gh.grounded_fraction */
  const double* weertman_c;          /* gh.weertman_c (= C * grounded fraction, update_state.jl:129-134) */
  const double* accumulation;        /* gh.accumulation */
  const double* basal_melt;          /* gh.basal_melt */
  /* inputs, u and v grids */
  const double* gu_h; const double* gu_s; const double* gu_grounded_fraction;
  const double* gv_h; const double* gv_s; const double* gv_grounded_fraction;
  /* input, 3-D */
  const double* glen_b;              /* g3d.glen_b, nx*ny*nsigma */
  /* Picard state, read and written */
  double* u;                         /* gu.u */
  double* v;                         /* gv.v */
  double* eta;                       /* g3d.η, nx*ny*nsigma */
  double* beta;                      /* gh.β */
  double* quad_f2;                   /* gh.quad_f2 */
  /* adaptive coarse space (wu.mask, wv.mask) and its cached coarse correction, compact in mask order */
  const uint8_t* wu_mask;            /* (nx+1)*ny */
  const uint8_t* wv_mask;            /* nx*(ny+1) */
  double* wu_correction_coarse;      /* count(wu_mask) */
  double* wv_correction_coarse;      /* count(wv_mask) */
  /* outputs (written where the reference writes them) */
  double* shelf_strain_rate; double* av_speed; double* bed_speed; double* tau_bed;
  double* eta_av; double* quad_f1; double* beta_eff;
  double* gu_beta_eff; double* gv_beta_eff;
  double* gu_residual; double* gv_residual;
} wavi_fields;

/* Per-solve statistics (the reference prints the residual and Picard count, update_velocities.jl:25). */
typedef struct wavi_stats {
  int32_t status;
  int32_t picard_iterations;
  int32_t coarse_cg_iterations;      /* summed over the solve's V-cycles */
  int32_t op_applications;           /* fine-operator applications, all precisions */
  double rel_residual;               /* last ||b - A u|| / ||b|| (float64) */
  double rel_update;                 /* last ||du|| / ||u|| */
  double algorithmic_bytes;          /* sum over launches of each kernel's algorithmic bytes */
  double elapsed_ms;                 /* device time of the solve (CUDA events) */
  int32_t kernel_launches;           /* kernels this library launched during the solve */
  int32_t host_syncs;                /* host round trips (convergence tests, CG batches) */
  double coarse_ms;                  /* device time of the persistent coarse-CG launches (CUDA events;
                                        host-driven solves, use_graphs = 0, only; else -1) */
  int32_t coarse_solver;             /* the wavi_coarse_solver the solve used (never AUTO) */
  int32_t coarse_launches;           /* persistent coarse-CG launches timed in coarse_ms */
  int32_t coarse_kernel;             /* the coarse-CG kernel the solve ran: 1 = persistent, vectors in
                                        registers; 2 = per-iteration kernels; 3 = persistent, vectors in
                                        global memory (the wavi_options.coarse_kernel codes) */
  int32_t cheb_steps;                /* Chebyshev steps per preconditioner application (0: the coarse
                                        solver has no Chebyshev preconditioner) */
  int32_t anderson_steps;            /* Picard iterations moved by the Anderson acceleration (0 without) */
  int32_t picard_accel;              /* the Picard iteration the solve ran (WAVI_PICARD_PLAIN or _ANDERSON) */
  int32_t coarse_forcing;            /* the coarse tolerance rule it ran (WAVI_FORCING_FIXED or _ADAPTIVE) */
  int32_t reserved1;
} wavi_stats;

typedef struct wavi_ctx wavi_ctx;

/* ABI version compiled into the library (== WAVI_ABI_VERSION of its header). */
int wavi_abi_version(void);

/* sizeof of wavi_grid_desc, wavi_params, wavi_solver_params, wavi_options, wavi_fields, wavi_stats as
 * compiled into the library, written to out[0..min(n,6)); returns 6.  Lets a binding (Julia struct,
 * ctypes) check its layout without a GPU.  No counterpart in the reference (a binding check). */
int wavi_abi_struct_sizes(int32_t* out, int n);

/* Number of CUDA devices, or a negative wavi_status. */
int wavi_device_count(void);

/* Create a context for one grid: validates the masks, derives the u/v/c masks
 * (src/Fields/Fields.jl:28-35, utilities.jl:475-507) and allocates every device buffer once. */
int wavi_ctx_create(const wavi_grid_desc* grid, const wavi_solver_params* solver,
                    const wavi_options* options, wavi_ctx** out);

/* The cudaStream_t (as void*) on which the context launches everything, so a caller can order its own
 * work or CUDA events against the solve.  No counterpart in the reference (a backend detail). */
void* wavi_ctx_stream(const wavi_ctx* ctx);

/* Release a context and its device memory.  Null is accepted. */
int wavi_ctx_destroy(wavi_ctx* ctx);

/* Message of the last failing call on this context (or of the last failing wavi_ctx_create when
 * ctx is null).  The string stays valid until the next call on the same context. */
const char* wavi_last_error(const wavi_ctx* ctx);

/* One velocity solve with host buffers: copies the inputs and Picard state to the device, runs
 * update_velocities! (update_velocities.jl:11-29) and copies the state and outputs back.
 * Replaces update_velocities.jl:11-29 as called from update_state.jl:154-157.
 * Returns 0 whenever the solve ran to its end, with stats->status = WAVI_OK, or the soft
 * WAVI_ERR_NOT_CONVERGED when maxiter_picard stopped it (every output written, as the reference stops
 * silently); a negative return is a hard error.  Bindings should nevertheless treat a return of
 * WAVI_ERR_NOT_CONVERGED or WAVI_ERR_COARSE_CAP as soft. */
int wavi_solve_velocities(wavi_ctx* ctx, const wavi_params* params, wavi_fields* fields,
                          wavi_stats* stats);

/* The same solve on device-resident buffers (every pointer in fields is a device pointer on the
 * context's device).  Runs on the context's stream and synchronises it before returning. */
int wavi_solve_velocities_device(wavi_ctx* ctx, const wavi_params* params, wavi_fields* fields,
                                 wavi_stats* stats);

/* Run inner_update! (update_velocities.jl:32-45) once on device fields, leaving the operator
 * coefficients in the context and writing the relinearised fields back.  Test and benchmark hook. */
int wavi_relinearise_device(wavi_ctx* ctx, const wavi_params* params, wavi_fields* fields);

/* One application of the momentum operator (op_fun!, utilities.jl:61-145, with vecSampled=false) with
 * the coefficients of the last relinearisation.  in_uv / out_uv are device vectors [u (nx+1)*ny | v
 * nx*(ny+1)] of float64 (precision WAVI_PRECISION_FP64) or float32 (WAVI_PRECISION_MIXED, mixed
 * contexts only); out_uv is the operator sampled at the interior points and zero elsewhere.
 * Test and benchmark hook. */
int wavi_apply_operator_device(wavi_ctx* ctx, int precision, const void* in_uv, void* out_uv);

/* Benchmark hook: `repeats` back-to-back launches of the operator kernel (as wavi_apply_operator_device)
 * on the context's stream, timed with CUDA events on that stream; *avg_ms receives the mean duration of
 * one launch.  No counterpart in the reference. */
int wavi_time_operator_device(wavi_ctx* ctx, int precision, const void* in_uv, void* out_uv, int repeats,
                              double* avg_ms);

/* Benchmark hook: `repeats` back-to-back launches of the relinearisation's h-grid kernel (the strain rate,
 * speeds, Weertman β and τ_b, the σ-level viscosity sweeps and quadratures of update_velocities.jl:202-339,
 * :374-383), then as many of its u/v-grid kernel (:348-366, :378), on the fields of the context's last
 * solve or relinearisation (the launches keep iterating the viscosity in place), timed with CUDA events on
 * the context's stream; *avg_ms_h and *avg_ms_uv receive the mean duration of one launch of each.  No
 * counterpart in the reference. */
int wavi_time_relinearise_device(wavi_ctx* ctx, int repeats, double* avg_ms_h, double* avg_ms_uv);

/* Diagonal of the operator at the interior points (what get_op_diag probes, update_preconditioners.jl
 * :92-109), same vector layout and precision rules as wavi_apply_operator_device.  Test hook. */
int wavi_op_diagonal_device(wavi_ctx* ctx, int precision, void* diag_uv);

/* diag(R A P) of the coarse operator (restriction R = wavelet-masked Haar analysis of the interior,
 * prolongation P = its transpose; update_preconditioners.jl:176-193) for the current coefficients and
 * the wavelet mask of the last solve, on the full wavelet grids (zero off the coarse space); the Jacobi
 * preconditioner of WAVI_COARSE_SRCG_JACOBI.  No reference counterpart: the reference's coarse
 * solve is unpreconditioned.  precision as wavi_apply_operator_device. */
int wavi_coarse_diagonal_device(wavi_ctx* ctx, int precision, void* diag_uv);

/* Haar transforms on float64 device vectors of the [u | v] layout (update_wavelets.jl:38-89):
 * kind 0 = mask ⊙ idwt(in) (prolongation, default mask = interior), kind 1 = mask ⊙ idwtᵀ(in)
 * (restriction, default mask = the last uploaded wavelet mask), kind 2 = dwt(mask ⊙ in) (the forward
 * transform of update_wavelets!, default mask = the u/v model masks).  mask_uv may be null.  Test hook. */
int wavi_haar_device(wavi_ctx* ctx, int kind, const double* in_uv, double* out_uv, const uint8_t* mask_uv);

/* update_wavelets! (Wavelets/update_wavelets.jl:6-32) with the kernels of wavi_run_device's time step:
 * the context's wavelet mask becomes |dwt(mask ⊙ in_uv)| >= wavelet_threshold (mask = the u/v model
 * masks), its coarse-correction cache is cleared, and the new mask ([u | v] layout, one byte per point)
 * is copied to the device buffer wmask_out.  in_uv: float64 device vector [u | v].  Test hook. */
int wavi_update_wavelets_device(wavi_ctx* ctx, const double* in_uv, uint8_t* wmask_out);

/* ---------------------------------------------------------------------------------------------------
 * Allocation-free entry point.  No counterpart in the reference: it exists for callers of this library
 * that cannot call cudaMalloc — a host framework that owns the device heap through its own pool
 * allocator, code running under stream capture or inside a callback where allocating is forbidden, or a
 * service whose device-memory budget is fixed at start-up.  Such a caller already holds the operator's
 * coefficients and vectors in its own device buffers.
 * ------------------------------------------------------------------------------------------------- */

/* The linearised momentum operator's coefficients as device arrays (the crops of
 * update_rheological_operators! folded in): heta_h = h_mask*h*ηav (nx*ny), heta_c = c_mask*cent_xy(h*ηav)
 * ((nx-1)*(ny-1)), dimp = h_mask*(-ρ_i g θ dt dsdh) (nx*ny), beta_m = mask*βeff and h_m = mask*h on
 * [u | v] (the u and v grids concatenated), inner = the interior mask on [u | v] (one byte per point). */
typedef struct wavi_operator_desc {
  int32_t nx, ny;
  double dx, dy;
  const double* heta_h;
  const double* heta_c;
  const double* dimp;
  const double* beta_m;
  const double* h_m;
  const uint8_t* inner;
} wavi_operator_desc;

/* Largest grid wavi_residual_noalloc accepts: (nx+1)*(ny+1) split into tiles of 32 x 8 points must
 * need at most this many tiles (about 4.19 million points, e.g. 2560 x 320 fits). */
#define WAVI_NOALLOC_MAX_TILES 16384

/* r = b - A x (float64) and rr_out[0] = ||r||^2, allocating nothing.  x_uv, b_uv, r_uv are device
 * vectors [u (nx+1)*ny | v nx*(ny+1)]; r is zero off the interior; rr_out is a device pointer.  The work
 * is queued on `stream` (a cudaStream_t, null for the legacy default stream) and not waited for.
 * The reduction scratch is a fixed static device array of 2*WAVI_NOALLOC_MAX_TILES+32 doubles
 * (about 256 KiB) that every device loading the library keeps until the process exits; grids beyond
 * WAVI_NOALLOC_MAX_TILES tiles are rejected with WAVI_ERR_ARGUMENT and a message in
 * wavi_last_error(NULL).  The first call on each device looks up that array's device address (with the
 * device current) and caches it for the life of the process: make that first call before any stream
 * capture, and do not call this entry point after cudaDeviceReset() on that device (the reset unloads the
 * module that holds the array, so the cached address is stale).  Every call shares the
 * one array (its counter is cleared at the start of each call), so calls that overlap on the GPU — on
 * different streams, or from different host threads — race and must be ordered by the caller. */
int wavi_residual_noalloc(const wavi_operator_desc* op, const double* x_uv, const double* b_uv, double* r_uv,
                          double* rr_out, void* stream);

/* ---- Adjoint and tangent linear of the converged solve ------------------------------------------
 * Gradients with respect to per-cell log C (Weertman drag coefficient, update_state.jl:129-134) and
 * log A (rate factor, all σ levels; B = A^(-1/n), utilities.jl:462-466) of a misfit J(u, v), by implicit
 * differentiation of the Picard fixed point of the last solve on this context (update_velocities.jl
 * :11-29 at convergence: A(coef) x = b together with the per-cell viscosity and drag fixed points
 * :227-339): one linear solve with the transposed linearised operator J_Fᵀ (viscosity and drag
 * derivatives included), by FGMRES preconditioned with one V-cycle of the solve's preconditioner (in
 * FP32 or FP64, wavi_options.adjoint_precond; FGMRES itself is FP64).  The reference has no adjoint.  Preconditions: a float64 context, no u/v_isfixed points, a preceding solve
 * converged tightly (the linearisation is exact at the fixed point).  Device pointers: dJ_du (nx+1)*ny,
 * dJ_dv nx*(ny+1) in, dJ_dlogC and dJ_dlogA nx*ny out.  The solve's state is left unchanged. */
typedef struct wavi_adjoint_stats {
  int32_t status;                    /* 0, or WAVI_ERR_NOT_CONVERGED if the linear solve hit maxiter */
  int32_t iterations;                /* FGMRES iterations (one preconditioned operator application each) */
  double rel_residual;               /* final ||b - K x|| / ||b|| of the linear solve */
  double elapsed_ms;                 /* host wall time of the call */
} wavi_adjoint_stats;
int wavi_adjoint_device(wavi_ctx* ctx, const wavi_params* params, const double* dJ_du, const double* dJ_dv,
                        double* dJ_dlogC, double* dJ_dlogA, double tol, int maxiter, wavi_adjoint_stats* stats);
/* The tangent linear: (du, dv) = d(u, v)/dθ · (dlogC, dlogA) (either direction may be NULL), from
 * J_F (du, dv) = -∂F/∂θ · dθ.  Same preconditions; the pair satisfies <J v, w> = <v, Jᵀ w>. */
int wavi_tangent_device(wavi_ctx* ctx, const wavi_params* params, const double* dlogC, const double* dlogA,
                        double* du, double* dv, double tol, int maxiter, wavi_adjoint_stats* stats);

/* ---- Device time stepping -------------------------------------------------------------------------
 * nsteps time steps of dt with the model kept on the device (run_simulation.jl:6-42): per step,
 * update_state! (update_state.jl:7-21: surface elevation, geometry on the u/v grids, height above
 * floatation, grounded fraction by pos_fraction (utilities.jl:255-396), accumulation, uniform basal melt,
 * C·grounded fraction, ds/dh; the velocity solve; velocities on the h grid, dh/dt, update_wavelets!) and
 * then update_thickness! with evolve_shelves.  fields (device pointers) holds the model state at the start;
 * on return every field of it holds the state after the last step, including those wavi_fields marks as
 * inputs (update_state! overwrites them in the reference as well) and the wavelet masks.  The coarse-
 * correction cache restarts at zero after every update_wavelets!, so the run leaves
 * wu/wv_correction_coarse untouched: after it the caller's caches are zero vectors of lengths
 * outputs->n_wu, n_wv.  stats sums the steps' counts and keeps the last step's status and residuals. */
typedef struct wavi_step_inputs {
  const double* bed;                 /* nx*ny bed elevation */
  const double* weertman_c;          /* nx*ny Weertman C before the grounded-fraction factor (Params) */
  const double* accumulation;        /* nx*ny accumulation rate (Params) */
  const uint8_t* h_isfixed;          /* nx*ny cells whose thickness does not evolve */
  double basal_melt_rate;            /* uniform basal melt rate (UniformMeltRate) */
  double reserved0;
} wavi_step_inputs;
typedef struct wavi_step_outputs {
  double* dhdt;                      /* nx*ny, or NULL; the other arrays likewise */
  double *u_h, *v_h, *u_bed, *v_bed, *u_surf, *v_surf;  /* velocities on the h grid (:164-178) */
  int32_t n_wu, n_wv;                /* coarse-space sizes after the last update_wavelets! */
  int32_t steps;
  int32_t reserved0;
} wavi_step_outputs;
int wavi_run_device(wavi_ctx* ctx, const wavi_params* params, double dt, int nsteps, const wavi_step_inputs* inputs,
                    wavi_fields* fields, wavi_step_outputs* outputs, wavi_stats* stats);

/* ---- Ensembles ---------------------------------------------------------------------------------
 * n independent domains (grids of different sizes) solved concurrently: one context per member (own
 * stream, device buffers and solve graph), at most `concurrency` members in flight, each member's
 * persistent coarse-CG kernel sized to 1/concurrency of the device's resident CTAs so that the
 * concurrent cooperative launches always fit together.  The reference has no ensemble call; this is
 * update_velocities! (update_velocities.jl:11-29) for each member, the role SharedMemorySpec's per-
 * subdomain solves on threads play there (src/SharedMemorySpec.jl:101-125).
 * options->use_graphs must be 1.  grids and solver_params are arrays of n. */
typedef struct wavi_ensemble wavi_ensemble;
int wavi_ensemble_create(int n, const wavi_grid_desc* grids, const wavi_solver_params* solver_params,
                         const wavi_options* options, int concurrency, wavi_ensemble** out);
/* update_velocities! for every member: params, fields (device pointers) and stats are arrays of n.
 * Returns when every member's results are in its arrays; per-member convergence is in stats[k].status.
 * A hard error returns the first failing member's status (message in wavi_ensemble_last_error). */
int wavi_ensemble_solve_device(wavi_ensemble* ens, const wavi_params* params, wavi_fields* fields, wavi_stats* stats);
int wavi_ensemble_destroy(wavi_ensemble* ens);
const char* wavi_ensemble_last_error(const wavi_ensemble* ens);

/* ---- Self-test of the bounded waits -------------------------------------------------------------
 * Every wait of the persistent kernels (grid barriers, tagged halo words) gives up after a bounded
 * number of polls, records WAVI_ERR_WATCHDOG and returns, so that the context stays usable.  This call
 * exercises that path without a fault: one thread waits, with the kernels' own bounded wait, for a
 * tagged word that nothing writes (about two seconds), then the error flag is cleared.  *fired = 1 if
 * the wait gave up as designed.  Not part of the reference interface (a test hook). */
int wavi_selftest_watchdog(wavi_ctx* ctx, int* fired);

/* ---- Self-test of the integer conversions -------------------------------------------------------
 * The float relinearisation of a mixed context converts between the caller's FP64 fields and float with
 * integer operations (round to nearest even; exact widening), because GB300 runs the hardware conversions
 * on its FP64 pipe.  This call compares them with the hardware conversions on the context's device over
 * n hashed bit patterns of each width (every exponent, rounding ties, subnormal and overflowing results;
 * 0 <= n <= 2^32): *mismatches = the results that differ (two NaNs agree).  Not part of the reference
 * interface (a test hook). */
int wavi_selftest_conversions(wavi_ctx* ctx, long long n, long long* mismatches);

#ifdef __cplusplus
}
#endif
#endif /* WAVI_GPU_H */
