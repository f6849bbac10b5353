// wavi_gpu.cu — libwavi_gpu.so: context, buffers, the solve graph and the C ABI of include/wavi_gpu.h.
//
// The solve is update_velocities! (src/Models/update_velocities.jl:11-29): per Picard iteration one
// relinearisation (inner_update!, :32-45), the float64 right-hand side and residual with the
// convergence test (:50-65, :106-182), and one wavelet-multigrid V-cycle (Wavelets/
// update_preconditioners.jl:54-83) with its coarse conjugate-gradient solve.  The whole control flow is
// one CUDA graph per context:
//
//   [state init] -> WHILE(picard_continue) {
//       relinearise h, relinearise u/v, rhs, (Dirichlet lift), residual + Picard decision
//       IF(vcycle_needed) {
//           V-cycle init + diagonal, 2*nsmooth*... smoother sweeps, restriction, coarse-CG start
//           WHILE(cg_continue) { direction + prolongation, coarse operator + restriction, update }
//           prolongation of the coarse correction, post-smoother, correction / write-back
//       }
//   }
//
// so a solve is one graph launch and one host synchronisation.  With use_graphs = 0 the same kernels
// run from a host loop that reads the decisions back (a debugging path).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wavi_gpu.h"
#include "kernels.cuh"
#include "fused.cuh"
#include "persistent.cuh"
#include "adjoint.cuh"
#include "timestep.cuh"
#include "anderson.cuh"

using namespace wavi;

namespace {

constexpr int EW_THREADS = 256;
constexpr int CG_BATCH = 8;
// grids with at least this many (nx+1) x (ny+1) points use the row-streaming operator by default
constexpr long kStreamMinPoints = 1L << 19;
// Anderson acceleration: default columns, and the relative residual below which it starts
constexpr int kAADefaultDepth = 3;
constexpr double kAAStartRel = 0.3;

}  // namespace

struct wavi_ctx {
  int dev = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t evc0 = nullptr, evc1 = nullptr;  // around a persistent coarse-CG launch (host-driven mode)
  double coarse_ms = 0.0;
  int coarse_launches = 0;
  bool coarse_pending = false;
  bool skipped = false;  // the last enqueued solve had maxiter_picard <= 0
  int pers_share = 1;    // persistent coarse kernels of this many contexts may run at once (ensembles)
  bool solved = false;   // a solve has left its converged state in the buffers (the adjoint linearises it)
  bool fields_loaded = false;  // a solve, relinearisation or time-stepping run has uploaded model fields
  struct Adj {           // adjoint / tangent-linear buffers, allocated on first use
    bool ready = false;
    AdjCell cell{};
    double *ebar = nullptr, *sbar = nullptr, *dheta_h = nullptr, *dhn = nullptr, *dbeff = nullptr, *dheta_c = nullptr,
           *dbeta_m = nullptr, *zero_h = nullptr, *xstate = nullptr, *ta = nullptr, *tb = nullptr, *b = nullptr,
           *x = nullptr, *uv_keep = nullptr, *xc_keep = nullptr, *dotv = nullptr;
    unsigned* counter = nullptr;
    std::vector<double*> V, Z;
    double** Vdev = nullptr;  // the Krylov basis pointers, for the batched Gram-Schmidt kernels
    double* hdev = nullptr;   // [first pass | second pass | ||w||^2] of one Arnoldi step
    double* gs_partials = nullptr;
  } adj;
  struct Step {          // device time stepping buffers, allocated on first use
    bool ready = false;
    double *b = nullptr, *c_param = nullptr, *acc_param = nullptr, *haf = nullptr, *afq = nullptr, *dhdt = nullptr;
    double *uh = nullptr, *vh = nullptr, *ub = nullptr, *vb = nullptr, *us = nullptr, *vs = nullptr, *wav = nullptr;
    uint8_t* h_isfixed = nullptr;
  } step;
  Dims d{};
  wavi_solver_params sp{};
  wavi_options opt{};
  bool acc64 = false;  // mixed coarse CG with FP64 dot products and scalars (WAVI_SUMS_FP64)
  bool visc32 = false;  // mixed: the σ-level viscosity sweeps in FP32 (the default; FP64 with WAVI_VISCOSITY_FP64)
  bool has_fixed = false;
  int tile = 16;  // Haar / coarse-operator tile: 16 (levels <= 3) or 32 (levels = 4)
  std::string err;
  std::vector<void*> allocs;
  // static masks (device)
  uint8_t *h_mask = nullptr, *c_mask = nullptr, *mask_uv = nullptr, *inner_uv = nullptr, *fixed_uv = nullptr;
  uint8_t* wmask_uv = nullptr;
  std::vector<uint8_t> h_inner_host;
  // inputs
  double *h = nullptr, *s = nullptr, *dsdh = nullptr, *gf = nullptr, *wc = nullptr, *acc = nullptr, *melt = nullptr;
  double *h_uv = nullptr, *s_uv = nullptr, *gf_uv = nullptr, *glen_b = nullptr;
  double *zeta = nullptr, *qw = nullptr;
  float *zeta_f = nullptr, *qw_f = nullptr;  // the same rounded to float
  // state
  double *uv = nullptr, *eta = nullptr, *beta = nullptr, *quad_f2 = nullptr;
  double* xc_full64 = nullptr;  // coarse correction cache (full layout, float64)
  // outputs
  double *shelf = nullptr, *av_speed = nullptr, *bed_speed = nullptr, *tau = nullptr, *eta_av = nullptr, *quad_f1 = nullptr,
         *beta_eff = nullptr, *beta_eff_uv = nullptr, *resid_uv = nullptr, *hn = nullptr;
  // coefficients
  double *heta_h64 = nullptr, *heta_c64 = nullptr, *dimp64 = nullptr, *beta_m64 = nullptr, *h_m64 = nullptr;
  float *heta_h32 = nullptr, *heta_c32 = nullptr, *dimp32 = nullptr, *beta_m32 = nullptr, *h_m32 = nullptr;
  // Picard vectors (float64)
  double *x64 = nullptr, *b64 = nullptr, *r64 = nullptr, *xfix64 = nullptr;
  // V-cycle vectors (float or double; sized for double)
  void *rs = nullptr, *corr[2] = {nullptr, nullptr}, *rsm[2] = {nullptr, nullptr}, *diag = nullptr, *xc = nullptr,
       *rc = nullptr, *uc = nullptr, *cc = nullptr, *w = nullptr, *bc = nullptr;
  // reductions and device state
  double* partials = nullptr;
  int max_partials = 0;
  DevParams* P = nullptr;     // device
  DevParams* P_adj = nullptr; // device: the adjoint's preconditioner V-cycle (capped coarse iterations)
  DevParams* hP = nullptr;    // pinned host staging
  DevState* S = nullptr;      // device
  DevState* hS = nullptr;     // pinned host copy
  // launch shapes
  dim3 op_grid, op_block, pt_grid, pt_block, haar_grid, haar_block, tile_grid, tile_block;
  bool stream_op = false;  // operator and smoother sweeps by the row-streaming kernel (large grids)
  dim3 st_grid;
  int st_rows = 0;
  int ew_blocks = 0;
  // persistent coarse CG: grid barrier, launch shape, tiles per CTA (0 = per-iteration kernels)
  GridBar* bar = nullptr;
  // halo boxes of the FP32 register-resident coarse CG: 8 x tile tagged words per tile
  unsigned long long* halo_box = nullptr;
  // the FP32 persistent smoother (one launch per pass): usable here, and its halo boxes (2 parities)
  bool fused_smooth = false;
  unsigned long long* smooth_box = nullptr;
  unsigned long long* selftest = nullptr;  // [0]: a tagged word nothing writes, [1]: the self-test's result
  int pers_maxt = 0, pers_grid = 0, ntx = 0, nty = 0;  // pers_maxt -1: CG vectors in global memory
  void *gz = nullptr, *gw = nullptr;                    // extra vectors of the global-memory variant
  void *w2 = nullptr, *gcd = nullptr;                   // its Chebyshev solve: second prolongation buffer, direction
  bool coarse64 = false;                                // mixed: the coarse CG in FP64 (WAVI_SUMS_FP64_SOLVE)
  double *bc64 = nullptr, *xc64 = nullptr;              // its right-hand side and iterate
  int coarse_solver = WAVI_COARSE_CG;  // resolved coarse solver (never WAVI_COARSE_AUTO)
  void* dcoarse = nullptr;             // diag(R A P) for the Jacobi-preconditioned single-reduction CG
  void* cheb_eig = nullptr;            // the Chebyshev coarse solve's power vector (kept across V-cycles)
  int aa_depth = 0;                    // Anderson acceleration of the Picard loop: columns (0: off)
  bool forcing = false;                // the coarse CG's tolerance follows the Picard residual
  bool adj_fp32 = false;               // the adjoint's preconditioner V-cycle runs in FP32
  AAWork aa{};                         // its columns, previous f and g, and reduction partials
  // coarse-correction cache mapping: block offsets of the mask scan (u part, then v part from
  // mask_offsets_v), staging for host callers, and the host masks' counts
  int* mask_offsets = nullptr;
  int mask_offsets_v = 0;
  uint8_t* wmask_in = nullptr;
  double* comp_stage = nullptr;
  long nwu = 0, nwv = 0;
  // solve graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // statistics of the current solve (host-side bookkeeping of what one launch sequence issues)
  long launches = 0;
  int host_syncs = 0;
  double picard_head_bytes = 0, vcycle_fixed_bytes = 0, cg_iter_bytes = 0;
  int picard_head_launches = 0, vcycle_fixed_launches = 0, cg_iter_launches = 0;
  int picard_head_ops = 0, vcycle_fixed_ops = 0, cg_iter_ops = 0;
};

namespace {

thread_local std::string g_create_error;

int fail(wavi_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c)
    c->err = buf;
  else
    g_create_error = buf;
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(c, WAVI_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

#define CKL()                                                                                        \
  do {                                                                                               \
    c->launches++;                                                                                   \
    cudaError_t e_ = cudaGetLastError();                                                             \
    if (e_ != cudaSuccess) return fail(c, WAVI_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
  } while (0)

#define TRY(expr)            \
  do {                       \
    int r_ = (expr);         \
    if (r_) return r_;       \
  } while (0)

template <typename T>
int dalloc(wavi_ctx* c, T** p, size_t n) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return fail(c, WAVI_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  c->allocs.push_back(q);
  e = cudaMemset(q, 0, bytes);
  if (e != cudaSuccess) return fail(c, WAVI_ERR_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
  *p = static_cast<T*>(q);
  return 0;
}

bool mixed(const wavi_ctx* c) { return c->opt.precision == WAVI_PRECISION_MIXED; }
// the relinearisation's viscosity sweeps in FP32 (mixed contexts unless WAVI_VISCOSITY_FP64), else FP64
bool visc32(const wavi_ctx* c) { return mixed(c) && c->visc32; }

template <typename T>
OpCoef<T> coef(const wavi_ctx* c);
template <>
OpCoef<double> coef<double>(const wavi_ctx* c) {
  return {c->heta_h64, c->heta_c64, c->dimp64, c->beta_m64, c->h_m64, c->inner_uv};
}

template <>
OpCoef<float> coef<float>(const wavi_ctx* c) {
  return {c->heta_h32, c->heta_c32, c->dimp32, c->beta_m32, c->h_m32, c->inner_uv};
}

// Algorithmic bytes of one operator application: read x, write y,
// coefficients heta_h, dimp (Nh), heta_c (Nc), beta_m, h_m (N), the interior mask (N bytes), plus the
// right-hand side for the residual form.
double op_bytes(const Dims& d, int w, bool resid) {
  return (double)w * (2.0 * d.N + 2.0 * d.Nh + d.Nc + 2.0 * d.N + (resid ? d.N : 0)) + d.N;
}

// ---------------------------------------------------------------------------------------------
// Launch sequences (shared by the graph capture and the host-driven path)
// ---------------------------------------------------------------------------------------------
struct Tally {
  double bytes = 0;
  int launches = 0, ops = 0;
};

int enqueue_picard_head(wavi_ctx* c, const CondHandles& h, Tally& t) {
  const Dims& d = c->d;
  RelinIn in{c->uv, c->mask_uv, c->h_mask, c->c_mask, c->h, c->wc, c->glen_b, c->dsdh, c->zeta, c->qw, c->P, c->zeta_f, c->qw_f};
  RelinOut out{c->shelf, c->av_speed, c->bed_speed, c->beta, c->tau, c->eta, c->eta_av, c->quad_f1, c->quad_f2,
               c->beta_eff, c->heta_h64, c->dimp64, mixed(c) ? c->heta_h32 : nullptr, mixed(c) ? c->dimp32 : nullptr,
               c->hn};
  const int nb = (d.Nh + 127) / 128;
  if (visc32(c))
    k_relin_h<float><<<nb, 128, 0, c->st>>>(d, in, out);
  else
    k_relin_h<double><<<nb, 128, 0, c->st>>>(d, in, out);
  CKL();
  RelinUVIn uin{c->mask_uv, c->h_mask, c->c_mask, c->beta_eff, c->gf, c->gf_uv, c->h_uv, c->hn};
  RelinUVOut uout{c->beta_eff_uv, c->beta_m64, c->h_m64, c->heta_c64, mixed(c) ? c->beta_m32 : nullptr,
                  mixed(c) ? c->h_m32 : nullptr, mixed(c) ? c->heta_c32 : nullptr};
  k_relin_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, uin, uout);
  CKL();
  RhsIn rin{c->h_mask, c->inner_uv, c->fixed_uv, c->s, c->dsdh, c->acc, c->melt, c->h_uv, c->s_uv, c->uv, 0, 0, 0, 0, 0};
  k_rhs_fused<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, rin, c->P, c->b64, c->x64, c->xfix64, c->partials, c->S);
  CKL();
  int nlaunch = 3;
  if (c->has_fixed) {
    k_lift<OP_TX, OP_TY><<<c->op_grid, c->op_block, 0, c->st>>>(d, coef<double>(c), c->xfix64, c->b64, c->partials, c->S);
    CKL();
    nlaunch++;
    t.ops++;
    t.bytes += op_bytes(d, 8, true);
  }
  k_picard_residual<OP_TX, OP_TY><<<c->op_grid, c->op_block, 0, c->st>>>(d, coef<double>(c), c->x64, c->b64, c->r64,
                                                                         c->resid_uv, c->partials, c->S, c->P, h);
  CKL();
  nlaunch++;
  t.ops++;
  t.launches += nlaunch;
  t.bytes += op_bytes(d, 8, true) + 8.0 * (2.0 * d.Nh * d.ns + 22.0 * d.Nh + 8.0 * d.N) + 4.0 * d.N;
  return 0;
}

// One smoother sweep: update = true: the colour update of x_in, then r_out = b - A x_out; update =
// false: r_out = b - A x_in.  Tiled (k_smooth) or row-streaming (k_op_stream) by grid size.
template <typename T>
int launch_smooth(wavi_ctx* c, bool update, int colour, const T* b, const T* diag, const T* x_in, const T* r_in,
                  T* x_out, T* r_out) {
  const Dims& d = c->d;
  if (c->stream_op) {
    if (update)
      k_op_stream<T, 2><<<c->st_grid, 32 * ST_WARPS, 0, c->st>>>(d, coef<T>(c), c->st_rows, x_in, b, r_out, colour, c->P,
                                                                 diag, r_in, x_out);
    else
      k_op_stream<T, 1><<<c->st_grid, 32 * ST_WARPS, 0, c->st>>>(d, coef<T>(c), c->st_rows, x_in, b, r_out, 0, c->P,
                                                                 nullptr, nullptr, nullptr);
  } else {
    if (update)
      k_smooth<T, OP_TX, OP_TY, true><<<c->op_grid, c->op_block, 0, c->st>>>(d, coef<T>(c), colour, c->P, b, diag, x_in,
                                                                            r_in, x_out, r_out);
    else
      k_smooth<T, OP_TX, OP_TY, false><<<c->op_grid, c->op_block, 0, c->st>>>(d, coef<T>(c), 0, c->P, b, diag, x_in,
                                                                             nullptr, nullptr, r_out);
  }
  CKL();
  return 0;
}

template <typename T>
int launch_op(wavi_ctx* c, const T* x, T* y) {
  if (c->stream_op)
    k_op_stream<T, 0><<<c->st_grid, 32 * ST_WARPS, 0, c->st>>>(c->d, coef<T>(c), c->st_rows, x, nullptr, y, 0, c->P,
                                                               nullptr, nullptr, nullptr);
  else
    k_op<T, T, 0><<<c->op_grid, c->op_block, 0, c->st>>>(c->d, coef<T>(c), x, nullptr, y, c->partials, nullptr);
  CKL();
  return 0;
}

// The persistent smoother runs on the coarse CG's cooperative grid (pers_grid CTAs of pers_maxt tiles):
// it is used where that grid is resident for it too.
bool smoother_fits(wavi_ctx* c) {
  if (c->pers_maxt <= 0) return false;
  int nsm = 0, per_sm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev);
  cudaError_t e = c->pers_maxt == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_smooth_persistent<1>, 256, 0)
                  : c->pers_maxt == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_smooth_persistent<2>, 256, 0)
                                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_smooth_persistent<4>, 256, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (long)per_sm * nsm / std::max(1, c->pers_share) >= c->pers_grid;
}

// One smoother pass as one cooperative launch (k_smooth_persistent): a fresh tag generation, the pass,
// and the watchdog check.  x and r in place; residual_first: r = b - A x before the sweeps.
int launch_smooth_fused(wavi_ctx* c, const CondHandles& h, bool residual_first, int order, const float* b,
                        const float* diag, float* x, float* r) {
  k_reset_barrier<<<1, 32, 0, c->st>>>(c->bar, (const DevParams*)c->P);
  CKL();
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c->pers_grid);
  cfg.blockDim = dim3(16, 16);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int rf = residual_first ? 1 : 0, ns = c->sp.nsmooth;
  const DevParams* P = (const DevParams*)c->P;
  if (c->pers_maxt == 1)
    CK(cudaLaunchKernelEx(&cfg, k_smooth_persistent<1>, c->d, coef<float>(c), P, b, diag, x, r, rf, ns, order, c->bar,
                          c->smooth_box, c->ntx, c->nty));
  else if (c->pers_maxt == 2)
    CK(cudaLaunchKernelEx(&cfg, k_smooth_persistent<2>, c->d, coef<float>(c), P, b, diag, x, r, rf, ns, order, c->bar,
                          c->smooth_box, c->ntx, c->nty));
  else
    CK(cudaLaunchKernelEx(&cfg, k_smooth_persistent<4>, c->d, coef<float>(c), P, b, diag, x, r, rf, ns, order, c->bar,
                          c->smooth_box, c->ntx, c->nty));
  c->launches++;
  k_check_barrier<<<1, 32, 0, c->st>>>(c->bar, c->S, h);
  CKL();
  return 0;
}

template <typename T, int TILE>
int enqueue_vcycle_pre(wavi_ctx* c, const CondHandles& h, Tally& t, bool cg_start = true) {
  const Dims& d = c->d;
  const int L = c->sp.levels;
  T* rs = (T*)c->rs;
  T* corr[2] = {(T*)c->corr[0], (T*)c->corr[1]};
  T* rsm[2] = {(T*)c->rsm[0], (T*)c->rsm[1]};
  T* diag = (T*)c->diag;
  k_vcycle_init<T><<<c->pt_grid, c->pt_block, 0, c->st>>>(d, coef<T>(c), c->r64, c->xc_full64, rs, rsm[0], corr[0],
                                                          (T*)c->xc, diag);
  CKL();
  t.launches++;
  static const int fwd[4] = {1, 3, 2, 4};
  int cur = 0;
  if constexpr (std::is_same<T, float>::value && TILE == 16) {
    if (c->fused_smooth) {  // the whole pass in one cooperative launch, in place in corr[0], rsm[0]
      TRY(launch_smooth_fused(c, h, false, fwd[0] | fwd[1] << 3 | fwd[2] << 6 | fwd[3] << 9, rs, diag, corr[0], rsm[0]));
      t.launches += 3;
      t.ops += 4 * c->sp.nsmooth;
      t.bytes += 4.0 * c->sp.nsmooth * (op_bytes(d, sizeof(T), true) + 4.0 * sizeof(T) * d.N);
    }
  }
  if (!(std::is_same<T, float>::value && TILE == 16 && c->fused_smooth))
    for (int it = 0; it < c->sp.nsmooth; ++it)
      for (int oc = 0; oc < 4; ++oc) {
        TRY(launch_smooth<T>(c, true, fwd[oc], rs, diag, corr[cur], rsm[cur], corr[1 - cur], rsm[1 - cur]));
        cur = 1 - cur;
        t.launches++;
        t.ops++;
        t.bytes += op_bytes(d, sizeof(T), true) + 4.0 * sizeof(T) * d.N;
      }
  // b_c = R r  and |b_c|
  k_restrict_norm<T, TILE><<<c->tile_grid, c->tile_block, 0, c->st>>>(d, L, rsm[cur], c->wmask_uv, (T*)c->bc,
                                                                      c->partials, c->S);
  CKL();
  if (cur != 0) return fail(c, WAVI_ERR_ARGUMENT, "internal: smoother parity");
  if (!cg_start) {  // the persistent coarse CG computes its own start
    t.launches++;
    t.bytes += 2.0 * sizeof(T) * d.N + d.N;
    return 0;
  }
  // r_c = b_c - R A P xc, u_c = 0, CG scalars
  k_prolong<T, TILE, 0><<<c->tile_grid, c->tile_block, 0, c->st>>>(d, L, c->inner_uv, (const T*)c->xc, (T*)c->w,
                                                                   nullptr, nullptr, c->S, nullptr);
  CKL();
  k_coarse_op<T, TILE, true><<<c->tile_grid, c->tile_block, 0, c->st>>>(d, L, coef<T>(c), c->wmask_uv, (const T*)c->w,
                                                                        nullptr, (T*)c->uc, (T*)c->rc, (const T*)c->bc,
                                                                        c->partials, c->S, c->P, h, nullptr);
  CKL();
  t.launches += 3;
  t.ops++;
  t.bytes += op_bytes(d, sizeof(T), false) + 8.0 * sizeof(T) * d.N + 3.0 * d.N;
  return 0;
}

template <typename T, int TILE>
int enqueue_cg_iteration(wavi_ctx* c, const CondHandles& h, int* live, Tally& t) {
  const Dims& d = c->d;
  const int L = c->sp.levels;
  k_prolong<T, TILE, 2><<<c->tile_grid, c->tile_block, 0, c->st>>>(d, L, c->inner_uv, nullptr, (T*)c->w, (const T*)c->rc,
                                                                   (T*)c->uc, c->S, live);
  CKL();
  k_coarse_op<T, TILE, false><<<c->tile_grid, c->tile_block, 0, c->st>>>(d, L, coef<T>(c), c->wmask_uv, (const T*)c->w,
                                                                         (T*)c->cc, (T*)c->uc, nullptr, nullptr,
                                                                         c->partials, c->S, c->P, h, live);
  CKL();
  k_cg_update<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, (const T*)c->uc, (const T*)c->cc, (T*)c->xc, (T*)c->rc,
                                                         c->partials, c->S, c->P, h, live);
  CKL();
  t.launches += 3;
  t.ops++;
  t.bytes += op_bytes(d, sizeof(T), false) + sizeof(T) * (4.0 * d.N + 6.0 * d.N) + 2.0 * d.N;
  return 0;
}

// The whole coarse CG as one cooperative persistent kernel (persistent.cuh), then the watchdog check.
// The Chebyshev coarse solve: steps of the Chebyshev-accelerated Jacobi iteration per preconditioner
// application (odd: the preconditioner stays positive definite if λmax is underestimated) and the ratio
// of the interval's ends.  Default steps: 5 in the register-resident single-reduction kernel, whose grid
// reduction (~3.2 µs on GB300) outweighs an operator application with its neighbour exchange (~2.5 µs), so
// that more steps per reduction pay (640 x 80: 2 611 iterations of 15.5 µs against 4 000 of 10.8 µs with
// 3 steps, 47.0 against 49.5 ms per solve; 7 steps 47.9 ms); 3 in the global-memory kernel, where every
// step is a pass over all tiles behind a grid barrier (2560 x 320: 1.96 s per solve with 5 steps against
// 1.79 s with 3), and in the pipelined kernel.  The interval's ratio moves the iteration count by a few
// per cent between 60 and 1000 (the oracle on 640 x 80).
constexpr int kChebStepsResident = 5, kChebStepsOther = 3;
int cheb_steps(const wavi_ctx* c) {
  if (c->opt.cheb_steps > 0) return c->opt.cheb_steps;
  return c->pers_maxt > 0 && c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV ? kChebStepsResident : kChebStepsOther;
}
constexpr float kChebRatio = 120.0f;

template <typename T, int TILE, int MAXT>
int launch_cg_persistent(wavi_ctx* c, const void* bcv, void* xcv) {
  const T* bc = (const T*)bcv;
  T* xc = (T*)xcv;
  const Dims& d = c->d;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c->pers_grid);
  cfg.blockDim = dim3(TILE, TILE);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (c->coarse_solver == WAVI_COARSE_CG) {
    CK(cudaLaunchKernelEx(&cfg, k_cg_persistent<T, TILE, MAXT>, d, c->sp.levels, coef<T>(c), (const uint8_t*)c->wmask_uv,
                          (T*)c->w, bc, xc, c->partials, c->S, (const DevParams*)c->P, c->bar,
                          c->halo_box, c->ntx, c->nty));
  } else if (c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV) {
    if constexpr (std::is_same<T, float>::value && TILE == 16 && MAXT <= 2) {
      CK(cudaLaunchKernelEx(&cfg, k_pcg_persistent<T, TILE, MAXT>, d, c->sp.levels, coef<T>(c),
                            (const uint8_t*)c->wmask_uv, (const T*)c->dcoarse, bc, xc, c->partials,
                            c->S, (const DevParams*)c->P, c->bar, c->halo_box, cheb_steps(c), kChebRatio,
                            (T*)c->cheb_eig, c->ntx, c->nty));
    } else {
      return fail(c, WAVI_ERR_ARGUMENT, "the pipelined coarse CG has no kernel for this precision and tiling");
    }
  } else {
    const bool cheb = c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV;
    const T* dc = (c->coarse_solver == WAVI_COARSE_SRCG_JACOBI || cheb) ? (const T*)c->dcoarse : nullptr;
    if (c->acc64) {
      if constexpr (std::is_same<T, float>::value && TILE == 16 && MAXT <= 2) {
        CK(cudaLaunchKernelEx(&cfg, k_srcg_persistent<T, TILE, MAXT, true>, d, c->sp.levels, coef<T>(c),
                              (const uint8_t*)c->wmask_uv, dc, (T*)c->w, bc, xc, c->partials, c->S,
                              (const DevParams*)c->P, c->bar, c->halo_box, cheb ? cheb_steps(c) : 1, kChebRatio,
                              (T*)c->cheb_eig, c->ntx, c->nty));
      } else {
        return fail(c, WAVI_ERR_ARGUMENT, "FP64 coarse sums have no kernel for this precision and tiling");
      }
    } else {
      CK(cudaLaunchKernelEx(&cfg, k_srcg_persistent<T, TILE, MAXT>, d, c->sp.levels, coef<T>(c), (const uint8_t*)c->wmask_uv,
                            dc, (T*)c->w, bc, xc, c->partials, c->S, (const DevParams*)c->P, c->bar,
                            c->halo_box, cheb ? cheb_steps(c) : 1, kChebRatio, (T*)c->cheb_eig, c->ntx, c->nty));
    }
  }
  c->launches++;
  return 0;
}

// The same with the CG vectors in global memory (grids with more tiles than resident CTAs).
template <typename T, int TILE>
int launch_cg_global(wavi_ctx* c, const void* bcv, void* xcv) {
  const T* bc = (const T*)bcv;
  T* xc = (T*)xcv;
  const Dims& d = c->d;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c->pers_grid);
  cfg.blockDim = dim3(TILE, TILE);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const GlobalCG<T> g{(T*)c->rc, (T*)c->gz, (T*)c->uc, (T*)c->cc, (T*)c->gw};
  if (c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV) {
    CK(cudaLaunchKernelEx(&cfg, k_srcg_cheb_global<T, TILE>, d, c->sp.levels, coef<T>(c), (const uint8_t*)c->wmask_uv,
                          (const T*)c->dcoarse, (T*)c->w, (T*)c->w2, bc, xc, g, (T*)c->gcd,
                          (T*)c->cheb_eig, cheb_steps(c), kChebRatio, c->partials, c->S, (const DevParams*)c->P, c->bar,
                          c->ntx, c->nty));
  } else if (c->coarse_solver == WAVI_COARSE_CG) {
    CK(cudaLaunchKernelEx(&cfg, k_cg_global<T, TILE>, d, c->sp.levels, coef<T>(c), (const uint8_t*)c->wmask_uv, (T*)c->w,
                          bc, xc, g, c->partials, c->S, (const DevParams*)c->P, c->bar, c->ntx,
                          c->nty));
  } else {
    const T* dc = c->coarse_solver == WAVI_COARSE_SRCG_JACOBI ? (const T*)c->dcoarse : nullptr;
    CK(cudaLaunchKernelEx(&cfg, k_srcg_global<T, TILE>, d, c->sp.levels, coef<T>(c), (const uint8_t*)c->wmask_uv, dc,
                          (T*)c->w, bc, xc, g, c->partials, c->S, (const DevParams*)c->P, c->bar,
                          c->ntx, c->nty));
  }
  c->launches++;
  return 0;
}

// diag(R A P) into dst: the separated kernel for 16 x 16 tiles, the general one otherwise.
template <typename T, int TILE>
void launch_coarse_diag(wavi_ctx* c, T* dst) {
  if constexpr (TILE == 16)
    k_coarse_diag_sep<T, TILE><<<c->tile_grid, c->tile_block, 0, c->st>>>(c->d, c->sp.levels, coef<T>(c), c->wmask_uv, dst);
  else
    k_coarse_diag<T, TILE><<<c->tile_grid, c->tile_block, 0, c->st>>>(c->d, c->sp.levels, coef<T>(c), c->wmask_uv, dst);
}

template <typename T, int TILE>
int enqueue_cg_persistent(wavi_ctx* c, const CondHandles& h, Tally& tv, Tally& tc) {
  const Dims& d = c->d;
  if (c->coarse_solver == WAVI_COARSE_SRCG_JACOBI || c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV ||
      c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV) {
    launch_coarse_diag<T, TILE>(c, (T*)c->dcoarse);
    CKL();
    tv.launches++;
  }
  k_reset_barrier<<<1, 32, 0, c->st>>>(c->bar, (const DevParams*)c->P);
  CKL();
  if (c->pers_maxt < 0)
    TRY((launch_cg_global<T, TILE>(c, c->bc, c->xc)));
  else if (c->pers_maxt == 1)
    TRY((launch_cg_persistent<T, TILE, 1>(c, c->bc, c->xc)));
  else if (c->pers_maxt == 2)
    TRY((launch_cg_persistent<T, TILE, 2>(c, c->bc, c->xc)));
  else
    TRY((launch_cg_persistent<T, TILE, 4>(c, c->bc, c->xc)));
  k_check_barrier<<<1, 32, 0, c->st>>>(c->bar, c->S, h);
  CKL();
  tv.launches += 3;
  tv.ops++;  // the start's R A P xc
  tc.ops++;
  tc.bytes += op_bytes(d, sizeof(T), false) + sizeof(T) * 2.0 * d.N + d.N;
  return 0;
}

// The mixed V-cycle's coarse solve in FP64 (WAVI_SUMS_FP64_SOLVE): the FP32 restricted residual and warm
// start widened to FP64, the FP64 persistent kernels on the FP64 coefficients (the same kernels as an FP64
// context's), the solution narrowed back for the FP32 prolongation.
template <int TILE>
int enqueue_cg_persistent64(wavi_ctx* c, const CondHandles& h, Tally& tv, Tally& tc) {
  const Dims& d = c->d;
  k_convert<float, double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, (const float*)c->bc, c->bc64);
  CKL();
  k_convert<float, double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, (const float*)c->xc, c->xc64);
  CKL();
  if (c->coarse_solver == WAVI_COARSE_SRCG_JACOBI || c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV) {
    launch_coarse_diag<double, TILE>(c, (double*)c->dcoarse);
    CKL();
    tv.launches++;
  }
  k_reset_barrier<<<1, 32, 0, c->st>>>(c->bar, (const DevParams*)c->P);
  CKL();
  if (c->pers_maxt < 0)
    TRY((launch_cg_global<double, TILE>(c, c->bc64, c->xc64)));
  else if (c->pers_maxt == 1)
    TRY((launch_cg_persistent<double, TILE, 1>(c, c->bc64, c->xc64)));
  else if (c->pers_maxt == 2)
    TRY((launch_cg_persistent<double, TILE, 2>(c, c->bc64, c->xc64)));
  else
    TRY((launch_cg_persistent<double, TILE, 4>(c, c->bc64, c->xc64)));
  k_check_barrier<<<1, 32, 0, c->st>>>(c->bar, c->S, h);
  CKL();
  k_convert<double, float><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->xc64, (float*)c->xc);
  CKL();
  tv.launches += 6;
  tv.bytes += 4.0 * (4 + 8) * d.N;
  tv.ops++;
  tc.ops++;
  tc.bytes += op_bytes(d, 8, false) + 8.0 * 2.0 * d.N + d.N;
  return 0;
}

// The coarse solve of a V-cycle: the persistent kernel in the context's precision, or FP64 in a mixed
// context with WAVI_SUMS_FP64_SOLVE.
template <typename T, int TILE>
int enqueue_coarse(wavi_ctx* c, const CondHandles& h, Tally& tv, Tally& tc) {
  if constexpr (std::is_same<T, float>::value) {
    if (c->coarse64) return enqueue_cg_persistent64<TILE>(c, h, tv, tc);
  }
  return enqueue_cg_persistent<T, TILE>(c, h, tv, tc);
}

// picard: the V-cycle of a Picard iteration (then followed by the Anderson step where enabled); false for
// the adjoint's preconditioner applications.
template <typename T, int TILE>
int enqueue_vcycle_post(wavi_ctx* c, const CondHandles& h, Tally& t, bool picard = true) {
  (void)h;
  const Dims& d = c->d;
  const int L = c->sp.levels;
  T* rs = (T*)c->rs;
  T* corr[2] = {(T*)c->corr[0], (T*)c->corr[1]};
  T* rsm[2] = {(T*)c->rsm[0], (T*)c->rsm[1]};
  T* diag = (T*)c->diag;
  // corr += P xc
  k_prolong<T, TILE, 1><<<c->tile_grid, c->tile_block, 0, c->st>>>(d, L, c->inner_uv, (const T*)c->xc, corr[0], nullptr,
                                                                   nullptr, c->S, nullptr);
  CKL();
  // r = b - A corr, then the sweeps in reversed colour order
  static const int bwd[4] = {4, 2, 3, 1};
  int cur = 0;
  bool fused = false;
  if constexpr (std::is_same<T, float>::value && TILE == 16) {
    if (c->fused_smooth) {  // the residual and the whole pass in one cooperative launch, in place
      TRY(launch_smooth_fused(c, h, true, bwd[0] | bwd[1] << 3 | bwd[2] << 6 | bwd[3] << 9, rs, diag, corr[0], rsm[0]));
      t.launches += 4;
      t.ops += 1 + 4 * c->sp.nsmooth;
      t.bytes += op_bytes(d, sizeof(T), true) + 3.0 * sizeof(T) * d.N +
                 4.0 * c->sp.nsmooth * (op_bytes(d, sizeof(T), true) + 4.0 * sizeof(T) * d.N);
      fused = true;
    }
  }
  if (!fused) {
    TRY(launch_smooth<T>(c, false, 0, rs, diag, corr[0], nullptr, nullptr, rsm[0]));
    t.launches += 2;
    t.ops++;
    t.bytes += op_bytes(d, sizeof(T), true) + 3.0 * sizeof(T) * d.N;
    for (int it = 0; it < c->sp.nsmooth; ++it)
      for (int oc = 0; oc < 4; ++oc) {
        TRY(launch_smooth<T>(c, true, bwd[oc], rs, diag, corr[cur], rsm[cur], corr[1 - cur], rsm[1 - cur]));
        cur = 1 - cur;
        t.launches++;
        t.ops++;
        t.bytes += op_bytes(d, sizeof(T), true) + 4.0 * sizeof(T) * d.N;
      }
  }
  k_vcycle_finish<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, corr[cur], (const T*)c->xc, c->x64, c->uv,
                                                             c->xc_full64, c->partials, c->S);
  CKL();
  t.launches++;
  t.bytes += (double)(2 * sizeof(T) + 8 * 3) * d.N + d.N;
  if (picard && c->aa_depth > 0) {  // Anderson acceleration: both launches return at once until it has started
    k_aa_stage<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, c->x64, corr[cur], c->aa, c->S,
                                                          (const DevParams*)c->P);
    CKL();
    k_aa_apply<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, c->x64, corr[cur], c->aa, c->uv, c->S,
                                                          (const DevParams*)c->P);
    CKL();
    t.launches += 2;
    t.bytes += (double)(2 * sizeof(T) + 2 + 8 * (8 + 2 * c->aa_depth)) * d.N;
  }
  return 0;
}

// Host-driven mode: add the duration of the last timed persistent coarse-CG launch (its stream has
// been synchronised since).
int collect_coarse_time(wavi_ctx* c) {
  if (!c->coarse_pending) return 0;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->evc0, c->evc1));
  c->coarse_ms += ms;
  c->coarse_launches++;
  c->coarse_pending = false;
  return 0;
}

template <typename T, int TILE>
int enqueue_all_host_driven(wavi_ctx* c) {
  // The same launch sequence as the graph, with the decisions read back on the host.
  CondHandles h{};
  h.active = 0;
  Tally tp, tv, tc;
  k_state_init<<<1, 32, 0, c->st>>>(c->S);
  CKL();
  if (c->cheb_eig) CK(cudaMemsetAsync(c->cheb_eig, 0, c->d.N * sizeof(double), c->st));  // every solve starts cold (N doubles in every context)
  for (;;) {
    TRY(enqueue_picard_head(c, h, tp));
    CK(cudaMemcpyAsync(c->hS, c->S, sizeof(DevState), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->host_syncs++;
    TRY(collect_coarse_time(c));
    if (c->hS->vcycle_needed && c->pers_maxt != 0) {
      TRY((enqueue_vcycle_pre<T, TILE>(c, h, tv, false)));
      CK(cudaEventRecord(c->evc0, c->st));
      TRY((enqueue_coarse<T, TILE>(c, h, tv, tc)));
      CK(cudaEventRecord(c->evc1, c->st));
      c->coarse_pending = true;
      TRY((enqueue_vcycle_post<T, TILE>(c, h, tv)));
    } else if (c->hS->vcycle_needed) {
      TRY((enqueue_vcycle_pre<T, TILE>(c, h, tv)));
      CK(cudaMemcpyAsync(c->hS, c->S, sizeof(DevState), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      c->host_syncs++;
      int* live = &c->S->cg_continue;
      while (c->hS->cg_continue) {
        for (int k = 0; k < CG_BATCH; ++k) TRY((enqueue_cg_iteration<T, TILE>(c, h, live, tc)));
        CK(cudaMemcpyAsync(c->hS, c->S, sizeof(DevState), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        c->host_syncs++;
      }
      TRY((enqueue_vcycle_post<T, TILE>(c, h, tv)));
    }
    if (!c->hS->picard_continue) break;
  }
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Graph construction: capture segments into the top graph and the conditional bodies.
// ---------------------------------------------------------------------------------------------
struct Segment {
  std::vector<cudaGraphNode_t> sinks;
};

int begin_capture(wavi_ctx* c, cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps) {
  CK(cudaStreamBeginCaptureToGraph(c->st, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                   cudaStreamCaptureModeThreadLocal));
  return 0;
}
int end_capture(wavi_ctx* c, cudaGraph_t g, std::vector<cudaGraphNode_t>& sinks) {
  cudaStreamCaptureStatus status;
  const cudaGraphNode_t* deps = nullptr;
  size_t n = 0;
  CK(cudaStreamGetCaptureInfo(c->st, &status, nullptr, nullptr, &deps, nullptr, &n));
  sinks.assign(deps, deps + n);
  cudaGraph_t out = nullptr;
  CK(cudaStreamEndCapture(c->st, &out));
  if (out != g) return fail(c, WAVI_ERR_CUDA, "capture returned a different graph");
  return 0;
}
int add_conditional(wavi_ctx* c, cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps,
                    cudaGraphConditionalHandle handle, cudaGraphConditionalNodeType type, cudaGraph_t* body,
                    cudaGraphNode_t* node) {
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = handle;
  p.conditional.type = type;
  p.conditional.size = 1;
  CK(cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p));
  *body = p.conditional.phGraph_out[0];
  return 0;
}

template <typename T, int TILE>
int build_graph(wavi_ctx* c) {
  cudaGraph_t top = nullptr;
  CK(cudaGraphCreate(&top, 0));
  c->graph = top;
  CondHandles h{};
  h.active = 1;
  CK(cudaGraphConditionalHandleCreate(&h.picard, top, 1, cudaGraphCondAssignDefault));
  std::vector<cudaGraphNode_t> sinks;
  Tally tp, tv, tc;
  const long saved = c->launches;
  // top: state init -> WHILE(picard)
  TRY(begin_capture(c, top, {}));
  k_state_init<<<1, 32, 0, c->st>>>(c->S);
  CKL();
  if (c->cheb_eig) CK(cudaMemsetAsync(c->cheb_eig, 0, c->d.N * sizeof(double), c->st));  // every solve starts cold (N doubles in every context)
  TRY(end_capture(c, top, sinks));
  cudaGraph_t pbody = nullptr, vbody = nullptr, cbody = nullptr;
  cudaGraphNode_t pnode, vnode, cnode;
  TRY(add_conditional(c, top, sinks, h.picard, cudaGraphCondTypeWhile, &pbody, &pnode));
  CK(cudaGraphConditionalHandleCreate(&h.vcycle, pbody, 0, cudaGraphCondAssignDefault));
  // Picard body: head, then IF(vcycle)
  TRY(begin_capture(c, pbody, {}));
  TRY(enqueue_picard_head(c, h, tp));
  TRY(end_capture(c, pbody, sinks));
  TRY(add_conditional(c, pbody, sinks, h.vcycle, cudaGraphCondTypeIf, &vbody, &vnode));
  if (c->pers_maxt != 0) {
    // V-cycle body: pre part, one persistent coarse-CG kernel, post part
    TRY(begin_capture(c, vbody, {}));
    TRY((enqueue_vcycle_pre<T, TILE>(c, h, tv, false)));
    TRY((enqueue_coarse<T, TILE>(c, h, tv, tc)));
    TRY((enqueue_vcycle_post<T, TILE>(c, h, tv)));
    TRY(end_capture(c, vbody, sinks));
  } else {
    CK(cudaGraphConditionalHandleCreate(&h.cg, vbody, 0, cudaGraphCondAssignDefault));
    // V-cycle body: pre part, WHILE(cg), post part
    TRY(begin_capture(c, vbody, {}));
    TRY((enqueue_vcycle_pre<T, TILE>(c, h, tv)));
    TRY(end_capture(c, vbody, sinks));
    TRY(add_conditional(c, vbody, sinks, h.cg, cudaGraphCondTypeWhile, &cbody, &cnode));
    TRY(begin_capture(c, cbody, {}));
    TRY((enqueue_cg_iteration<T, TILE>(c, h, nullptr, tc)));
    TRY(end_capture(c, cbody, sinks));
    TRY(begin_capture(c, vbody, {cnode}));
    TRY((enqueue_vcycle_post<T, TILE>(c, h, tv)));
    TRY(end_capture(c, vbody, sinks));
  }
  CK(cudaGraphInstantiate(&c->exec, top, 0));
  c->launches = saved;
  c->picard_head_bytes = tp.bytes;
  c->picard_head_launches = tp.launches;
  c->picard_head_ops = tp.ops;
  c->vcycle_fixed_bytes = tv.bytes;
  c->vcycle_fixed_launches = tv.launches;
  c->vcycle_fixed_ops = tv.ops;
  c->cg_iter_bytes = tc.bytes;
  c->cg_iter_launches = tc.launches;
  c->cg_iter_ops = tc.ops;
  return 0;
}

// Persistent coarse CG: the smallest tiles-per-CTA (1, 2, 4) for which every CTA of the launch is
// resident at once (the cooperative launch needs that); 0 if none fits.
template <int MAXT, typename T, int TILE>
int resident_ctas(int nsm, int solver, bool acc64) {
  int per_sm = 0;
  if (acc64 && solver != WAVI_COARSE_CG && solver != WAVI_COARSE_PIPELINED_CHEBYSHEV) {
    if constexpr (std::is_same<T, float>::value && TILE == 16 && MAXT <= 2) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_srcg_persistent<T, TILE, MAXT, true>, TILE * TILE, 0) !=
          cudaSuccess)
        return 0;
      return per_sm * nsm;
    }
    return 0;
  }
  if (solver == WAVI_COARSE_PIPELINED_CHEBYSHEV) {
    if constexpr (std::is_same<T, float>::value && TILE == 16 && MAXT <= 2) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_persistent<T, TILE, MAXT>, TILE * TILE, 0) !=
          cudaSuccess)
        return 0;
      return per_sm * nsm;
    }
    return 0;
  }
  cudaError_t e = solver == WAVI_COARSE_CG
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_persistent<T, TILE, MAXT>, TILE * TILE, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_srcg_persistent<T, TILE, MAXT>, TILE * TILE, 0);
  if (e != cudaSuccess) return 0;
  return per_sm * nsm;
}
template <typename T, int TILE>
void choose_persistent(wavi_ctx* c) {
  c->pers_maxt = 0;
  int nsm = 0, coop = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->dev);
  if (!coop || nsm <= 0) return;
  const long ntiles = (long)c->ntx * c->nty;
  const int s = c->coarse_solver;
  const int share = std::max(1, c->pers_share);
  const int caps[3] = {resident_ctas<1, T, TILE>(nsm, s, c->acc64) / share,
                       resident_ctas<2, T, TILE>(nsm, s, c->acc64) / share,
                       resident_ctas<4, T, TILE>(nsm, s, c->acc64) / share};
  const int maxts[3] = {1, 2, 4};
  for (int k = 0; k < 3 && c->opt.coarse_kernel != 3; ++k) {
    const long g = (ntiles + maxts[k] - 1) / maxts[k];
    if (caps[k] > 0 && g <= caps[k]) {
      c->pers_maxt = maxts[k];
      c->pers_grid = (int)g;
      return;
    }
  }
  // global-memory vectors: one CTA per resident slot, looping over the tiles
  int per_sm = 0;
  cudaError_t e =
      s == WAVI_COARSE_CG ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_global<T, TILE>, TILE * TILE, 0)
      : s == WAVI_COARSE_SRCG_CHEBYSHEV
          ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_srcg_cheb_global<T, TILE>, TILE * TILE, 0)
          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_srcg_global<T, TILE>, TILE * TILE, 0);
  if (e != cudaSuccess || per_sm <= 0) return;
  c->pers_maxt = -1;
  c->pers_grid = (int)std::max<long>(1, std::min<long>(ntiles, (long)per_sm * nsm / share));
}

int ensure_graph(wavi_ctx* c) {
  if (c->exec) return 0;
  if (mixed(c)) return c->tile == 16 ? build_graph<float, 16>(c) : build_graph<float, 32>(c);
  return c->tile == 16 ? build_graph<double, 16>(c) : build_graph<double, 32>(c);
}

int set_params(wavi_ctx* c, const wavi_params* p) {
  DevParams& P = *c->hP;
  P.weertman_m = p->weertman_m;
  P.weertman_reg_speed = p->weertman_reg_speed;
  P.glen_n = p->glen_n;
  P.glen_reg_strain_rate = p->glen_reg_strain_rate;
  P.c0 = -p->density_ice * p->g * c->sp.super_implicitness * p->dt;
  P.rho_i = p->density_ice;
  P.rho_w = p->density_ocean;
  P.g = p->g;
  P.sea_level = p->sea_level_wrt_geoid;
  P.theta_dt = c->sp.super_implicitness * p->dt;
  P.tol_picard = c->sp.tol_picard;
  P.tol_coarse = c->sp.tol_coarse;
  P.omega = c->sp.smoother_omega;
  P.maxiter_picard = c->sp.maxiter_picard;
  P.maxiter_coarse = c->sp.maxiter_coarse;
  P.nsmooth = c->sp.nsmooth;
  P.n_iter_viscosity = c->sp.n_iter_viscosity;
  P.picard_test = c->opt.picard_test;
  P.aa_depth = c->aa_depth;
  P.coarse_forcing = c->forcing ? 1 : 0;
  P.aa_start_rel = kAAStartRel;
  P.weertman_ex_f = (float)(1.0 / p->weertman_m - 1.0);
  P.glen_ex_f = (float)(1.0 / p->glen_n - 1.0);
  P.glen_er2_f = (float)(p->glen_reg_strain_rate * p->glen_reg_strain_rate);
  P.weertman_reg_speed_f = (float)p->weertman_reg_speed;
  CK(cudaMemcpyAsync(c->P, c->hP, sizeof(DevParams), cudaMemcpyHostToDevice, c->st));
  return 0;
}

// A solve in two halves: solve_enqueue issues the whole solve on the context's stream (and, in graph
// mode, returns at once); solve_finish waits for it and fills the statistics.
int solve_enqueue(wavi_ctx* c, const wavi_params* p) {
  c->launches = 0;
  c->host_syncs = 0;
  c->coarse_ms = 0.0;
  c->coarse_launches = 0;
  c->coarse_pending = false;
  TRY(set_params(c, p));
  c->skipped = c->sp.maxiter_picard <= 0;
  if (c->skipped) return 0;
  CK(cudaEventRecord(c->ev0, c->st));
  if (c->opt.use_graphs) {
    TRY(ensure_graph(c));
    CK(cudaGraphLaunch(c->exec, c->st));
  } else if (mixed(c)) {
    TRY((c->tile == 16 ? enqueue_all_host_driven<float, 16>(c) : enqueue_all_host_driven<float, 32>(c)));
  } else {
    TRY((c->tile == 16 ? enqueue_all_host_driven<double, 16>(c) : enqueue_all_host_driven<double, 32>(c)));
  }
  CK(cudaEventRecord(c->ev1, c->st));
  CK(cudaMemcpyAsync(c->hS, c->S, sizeof(DevState), cudaMemcpyDeviceToHost, c->st));
  return 0;
}

// The coarse-CG kernel the context runs (the wavi_options.coarse_kernel codes 1-3) and the Chebyshev steps
// of its preconditioner (0 if the coarse solver has none).
void fill_coarse_kind(const wavi_ctx* c, wavi_stats* st) {
  st->coarse_kernel = c->pers_maxt > 0 ? 1 : c->pers_maxt < 0 ? 3 : 2;
  st->picard_accel = c->aa_depth > 0 ? WAVI_PICARD_ANDERSON : WAVI_PICARD_PLAIN;
  st->coarse_forcing = c->forcing ? WAVI_FORCING_ADAPTIVE : WAVI_FORCING_FIXED;
  const bool cheb = c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV || c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV;
  st->cheb_steps = cheb ? cheb_steps(c) : 0;
}

int solve_finish(wavi_ctx* c, wavi_stats* st) {
  if (c->skipped) {
    if (st) {
      *st = wavi_stats{};
      st->coarse_solver = c->coarse_solver;
      fill_coarse_kind(c, st);
    }
    return 0;
  }
  CK(cudaStreamSynchronize(c->st));
  c->host_syncs++;
  c->solved = true;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  TRY(collect_coarse_time(c));
  const DevState& S = *c->hS;
  const int picard = S.picard_it, vcycles = S.converged ? picard - 1 : picard;
  if (c->opt.use_graphs) {  // launches the graph issued, from the per-segment tallies
    c->launches = 1 + (long)picard * c->picard_head_launches + (long)vcycles * c->vcycle_fixed_launches +
                  (long)S.cg_total * c->cg_iter_launches;
  }
  if (S.status == WAVI_ERR_NONFINITE) return fail(c, WAVI_ERR_NONFINITE, "non-finite Picard residual at iteration %d", picard);
  if (st) {
    st->status = S.converged ? WAVI_OK : WAVI_ERR_NOT_CONVERGED;
    st->picard_iterations = picard;
    st->coarse_cg_iterations = S.cg_total;
    st->op_applications = picard * c->picard_head_ops + vcycles * c->vcycle_fixed_ops + S.cg_total * c->cg_iter_ops;
    st->rel_residual = S.rel;
    st->rel_update = S.rel_update;
    st->algorithmic_bytes = picard * c->picard_head_bytes + vcycles * c->vcycle_fixed_bytes + S.cg_total * c->cg_iter_bytes;
    st->elapsed_ms = ms;
    st->kernel_launches = (int32_t)std::min<long>(c->launches, 2147483647L);
    st->host_syncs = c->host_syncs;
    st->coarse_ms = c->opt.use_graphs ? -1.0 : c->coarse_ms;
    st->coarse_solver = c->coarse_solver;
    st->coarse_launches = c->opt.use_graphs ? 0 : c->coarse_launches;
    fill_coarse_kind(c, st);
    st->anderson_steps = S.aa.steps;
  }
  return 0;  // not converging is reported through stats.status only, like the reference's silent stop
}

int solve_resident(wavi_ctx* c, const wavi_params* p, wavi_stats* st) {
  TRY(solve_enqueue(c, p));
  return solve_finish(c, st);
}

// ---------------------------------------------------------------------------------------------
// Upload / download between wavi_fields and the context
// ---------------------------------------------------------------------------------------------
int copy_in(wavi_ctx* c, double* dst, const double* src, size_t n, cudaMemcpyKind kind, const char* name) {
  if (!src) return fail(c, WAVI_ERR_ARGUMENT, "field %s is null", name);
  CK(cudaMemcpyAsync(dst, src, n * sizeof(double), kind, c->st));
  return 0;
}
int copy_out(wavi_ctx* c, double* dst, const double* src, size_t n, cudaMemcpyKind kind, const char* name) {
  if (!dst) return fail(c, WAVI_ERR_ARGUMENT, "field %s is null", name);
  CK(cudaMemcpyAsync(dst, src, n * sizeof(double), kind, c->st));
  return 0;
}

// Full <-> compact coarse-correction cache for one part (u: base 0, n = Nu; v: base Nu, n = Nv).
// EXPAND also writes the normalised wavelet mask and the part's block offsets, which the compaction
// after the solve reuses (the solve does not change the mask).
template <bool EXPAND>
int map_coarse_cache(wavi_ctx* c, const uint8_t* mask, int n, int base, double* compact) {
  const int nb = (n + MS_BLOCK - 1) / MS_BLOCK;
  int* off = c->mask_offsets + (base == 0 ? 0 : c->mask_offsets_v);
  if (EXPAND) {
    k_mask_count<<<nb, MS_BLOCK, 0, c->st>>>(mask, n, off);
    CKL();
    k_scan_counts<<<1, MS_BLOCK, 0, c->st>>>(off, nb);
    CKL();
  }
  k_mask_map<EXPAND><<<nb, MS_BLOCK, 0, c->st>>>(mask, n, off, c->xc_full64 + base, compact, c->wmask_uv + base);
  CKL();
  return 0;
}

int upload(wavi_ctx* c, const wavi_fields* f, bool host) {
  c->fields_loaded = true;
  const Dims& d = c->d;
  const cudaMemcpyKind k = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
#define IN(dst, src, n) TRY(copy_in(c, dst, src, n, k, #src));
  IN(c->h, f->h, d.Nh) IN(c->s, f->s, d.Nh) IN(c->dsdh, f->dsdh, d.Nh) IN(c->gf, f->grounded_fraction, d.Nh)
  IN(c->wc, f->weertman_c, d.Nh) IN(c->acc, f->accumulation, d.Nh) IN(c->melt, f->basal_melt, d.Nh)
  IN(c->h_uv, f->gu_h, d.Nu) IN(c->h_uv + d.Nu, f->gv_h, d.Nv)
  IN(c->s_uv, f->gu_s, d.Nu) IN(c->s_uv + d.Nu, f->gv_s, d.Nv)
  IN(c->gf_uv, f->gu_grounded_fraction, d.Nu) IN(c->gf_uv + d.Nu, f->gv_grounded_fraction, d.Nv)
  IN(c->glen_b, f->glen_b, (size_t)d.Nh * d.ns)
  IN(c->uv, f->u, d.Nu) IN(c->uv + d.Nu, f->v, d.Nv)
  IN(c->eta, f->eta, (size_t)d.Nh * d.ns) IN(c->beta, f->beta, d.Nh) IN(c->quad_f2, f->quad_f2, d.Nh)
  // outputs that the reference only partially overwrites start from the caller's values
  IN(c->beta_eff_uv, f->gu_beta_eff, d.Nu) IN(c->beta_eff_uv + d.Nu, f->gv_beta_eff, d.Nv)
  IN(c->resid_uv, f->gu_residual, d.Nu) IN(c->resid_uv + d.Nu, f->gv_residual, d.Nv)
#undef IN
  // adaptive coarse space and its compact correction cache -> full layout, on the device
  if (!f->wu_mask || !f->wv_mask || !f->wu_correction_coarse || !f->wv_correction_coarse)
    return fail(c, WAVI_ERR_ARGUMENT, "wavelet masks / coarse corrections are null");
  const uint8_t* mu = f->wu_mask;
  const uint8_t* mv = f->wv_mask;
  const double* cu = f->wu_correction_coarse;
  const double* cv = f->wv_correction_coarse;
  if (host) {  // stage the host arrays (the compact lengths are the host masks' counts)
    c->nwu = c->nwv = 0;
    for (int i = 0; i < d.Nu; ++i) c->nwu += f->wu_mask[i] != 0;
    for (int i = 0; i < d.Nv; ++i) c->nwv += f->wv_mask[i] != 0;
    CK(cudaMemcpyAsync(c->wmask_in, f->wu_mask, d.Nu, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->wmask_in + d.Nu, f->wv_mask, d.Nv, cudaMemcpyHostToDevice, c->st));
    if (c->nwu) CK(cudaMemcpyAsync(c->comp_stage, f->wu_correction_coarse, sizeof(double) * c->nwu, cudaMemcpyHostToDevice, c->st));
    if (c->nwv) CK(cudaMemcpyAsync(c->comp_stage + d.Nu, f->wv_correction_coarse, sizeof(double) * c->nwv, cudaMemcpyHostToDevice, c->st));
    mu = c->wmask_in;
    mv = c->wmask_in + d.Nu;
    cu = c->comp_stage;
    cv = c->comp_stage + d.Nu;
  }
  TRY(map_coarse_cache<true>(c, mu, d.Nu, 0, const_cast<double*>(cu)));
  TRY(map_coarse_cache<true>(c, mv, d.Nv, d.Nu, const_cast<double*>(cv)));
  return 0;
}

int download(wavi_ctx* c, wavi_fields* f, bool host) {
  const Dims& d = c->d;
  const cudaMemcpyKind k = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
#define OUT(dst, src, n) TRY(copy_out(c, dst, src, n, k, #dst));
  OUT(f->u, c->uv, d.Nu) OUT(f->v, c->uv + d.Nu, d.Nv) OUT(f->eta, c->eta, (size_t)d.Nh * d.ns)
  OUT(f->beta, c->beta, d.Nh) OUT(f->quad_f2, c->quad_f2, d.Nh)
  OUT(f->shelf_strain_rate, c->shelf, d.Nh) OUT(f->av_speed, c->av_speed, d.Nh) OUT(f->bed_speed, c->bed_speed, d.Nh)
  OUT(f->tau_bed, c->tau, d.Nh) OUT(f->eta_av, c->eta_av, d.Nh) OUT(f->quad_f1, c->quad_f1, d.Nh)
  OUT(f->beta_eff, c->beta_eff, d.Nh)
  OUT(f->gu_beta_eff, c->beta_eff_uv, d.Nu) OUT(f->gv_beta_eff, c->beta_eff_uv + d.Nu, d.Nv)
  OUT(f->gu_residual, c->resid_uv, d.Nu) OUT(f->gv_residual, c->resid_uv + d.Nu, d.Nv)
#undef OUT
  // coarse correction cache: full -> compact in mask order, on the device
  if (host) {
    TRY(map_coarse_cache<false>(c, c->wmask_uv, d.Nu, 0, c->comp_stage));
    TRY(map_coarse_cache<false>(c, c->wmask_uv + d.Nu, d.Nv, d.Nu, c->comp_stage + d.Nu));
    if (c->nwu) CK(cudaMemcpyAsync(f->wu_correction_coarse, c->comp_stage, sizeof(double) * c->nwu, cudaMemcpyDeviceToHost, c->st));
    if (c->nwv) CK(cudaMemcpyAsync(f->wv_correction_coarse, c->comp_stage + d.Nu, sizeof(double) * c->nwv, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  } else {
    TRY(map_coarse_cache<false>(c, c->wmask_uv, d.Nu, 0, f->wu_correction_coarse));
    TRY(map_coarse_cache<false>(c, c->wmask_uv + d.Nu, d.Nv, d.Nu, f->wv_correction_coarse));
  }
  return 0;
}

int check_ctx(wavi_ctx* c) {
  if (!c) return WAVI_ERR_ARGUMENT;
  cudaError_t e = cudaSetDevice(c->dev);
  if (e != cudaSuccess) return fail(c, WAVI_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  return 0;
}

int check_params(wavi_ctx* c, const wavi_params* p) {
  if (!p) return fail(c, WAVI_ERR_ARGUMENT, "params is null");
  if (!(p->glen_n > 0) || !(p->weertman_m > 0)) return fail(c, WAVI_ERR_ARGUMENT, "glen_n and weertman_m must be positive");
  return 0;
}


// ---------------------------------------------------------------------------------------------
// Adjoint and tangent linear of the converged solve (adjoint.cuh): J_F v, J_Fᵀ w, one V-cycle as the
// preconditioner, restarted right-preconditioned FGMRES (Saad 1993) for both linear systems.
// ---------------------------------------------------------------------------------------------
constexpr int ADJ_RESTART = 40;
constexpr int kAdjCoarseIters = 100;  // coarse-CG iterations of the adjoint's preconditioner V-cycle
constexpr int kGsBlocks = 152;        // blocks per basis vector of the batched Gram-Schmidt dot products

int adj_alloc(wavi_ctx* c) {
  auto& a = c->adj;
  if (a.ready) return 0;
  const Dims& d = c->d;
  const size_t Nh = d.Nh, N = d.N;
  int r = 0;
#define AA(p, n) \
  if ((r = dalloc(c, &p, n))) return r;
  AA(a.cell.ux, Nh) AA(a.cell.vy, Nh) AA(a.cell.sh, Nh) AA(a.cell.uc, Nh) AA(a.cell.vc, Nh) AA(a.cell.S, Nh)
  AA(a.cell.L, 8 * Nh) AA(a.ebar, Nh) AA(a.sbar, Nh) AA(a.dheta_h, Nh) AA(a.dhn, Nh) AA(a.dbeff, Nh)
  AA(a.dheta_c, std::max<size_t>(d.Nc, 1)) AA(a.dbeta_m, N) AA(a.zero_h, Nh) AA(a.xstate, N) AA(a.ta, N) AA(a.tb, N)
  AA(a.b, N) AA(a.x, N) AA(a.uv_keep, N) AA(a.xc_keep, N) AA(a.dotv, 1) AA(a.counter, 1)
  AA(c->P_adj, 1)
#undef AA
  a.V.assign(ADJ_RESTART + 1, nullptr);
  a.Z.assign(ADJ_RESTART, nullptr);
  for (auto& v : a.V)
    if ((r = dalloc(c, &v, N))) return r;
  for (auto& v : a.Z)
    if ((r = dalloc(c, &v, N))) return r;
  if ((r = dalloc(c, &a.Vdev, (size_t)ADJ_RESTART + 1))) return r;
  if ((r = dalloc(c, &a.hdev, (size_t)2 * (ADJ_RESTART + 1) + 1))) return r;
  if ((r = dalloc(c, &a.gs_partials, (size_t)(ADJ_RESTART + 1) * kGsBlocks))) return r;
  if (cudaMemcpy(a.Vdev, a.V.data(), sizeof(double*) * a.V.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(c, WAVI_ERR_CUDA, "adjoint basis pointers upload failed");
  a.ready = true;
  return 0;
}

AdjUV adj_uv(wavi_ctx* c) { return {c->mask_uv, c->h_mask, c->c_mask, c->gf, c->gf_uv, c->h}; }

double adj_dot(wavi_ctx* c, const double* x, const double* y, int* err) {
  k_dot<<<c->ew_blocks, EW_THREADS, 0, c->st>>>(c->d.N, x, y, c->partials, c->adj.counter, c->adj.dotv);
  double v = 0.0;
  if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&v, c->adj.dotv, sizeof(double), cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    *err = fail(c, WAVI_ERR_CUDA, "adjoint dot product failed");
  return v;
}

// out = J_F v (transpose = false) or J_Fᵀ v (transpose = true), interior vectors.
int adj_apply(wavi_ctx* c, bool transpose, const double* v, double* out) {
  const Dims& d = c->d;
  auto& a = c->adj;
  const OpCoef<double> cf = coef<double>(c);
  if (!transpose) {
    k_tlm_cell<<<(d.Nh + 127) / 128, 128, 0, c->st>>>(d, a.cell, adj_uv(c), v, nullptr, nullptr, a.dheta_h, a.dhn, a.dbeff);
    CKL();
    k_tlm_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, adj_uv(c), a.dhn, a.dbeff, a.dbeta_m, a.dheta_c);
    CKL();
    TRY(launch_op<double>(c, v, a.ta));
    const OpCoef<double> dcf{a.dheta_h, a.dheta_c, a.zero_h, a.dbeta_m, c->h_m64, c->inner_uv};
    k_op<double, double, 0><<<c->op_grid, c->op_block, 0, c->st>>>(d, dcf, a.xstate, nullptr, a.tb, c->partials, nullptr);
    CKL();
    k_add_inner<<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, a.ta, a.tb, out);
    CKL();
  } else {
    TRY(launch_op<double>(c, v, a.ta));  // the operator is symmetric
    k_adj_cell<<<(d.Nh + 127) / 128, 128, 0, c->st>>>(d, a.cell, adj_uv(c), c->inner_uv, a.xstate, v, a.ebar, a.sbar,
                                                     nullptr, nullptr);
    CKL();
    k_adj_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, a.cell, adj_uv(c), c->inner_uv, a.ebar, a.sbar, a.ta, out);
    CKL();
  }
  (void)cf;
  return 0;
}

template <typename T, int TILE>
int adj_vcycle_body(wavi_ctx* c, const double* v, double* out);

// out = one V-cycle of the solve's preconditioner applied to v (zero start, zero coarse warm start), its
// coarse CG capped at kAdjCoarseIters iterations (P_adj): FGMRES takes any fixed preconditioner, and the
// cold coarse solve would otherwise run towards maxiter_coarse in every application.
template <typename T, int TILE>
int adj_vcycle(wavi_ctx* c, const double* v, double* out) {
  DevParams* const P_solve = c->P;
  c->P = c->P_adj;
  const int r = adj_vcycle_body<T, TILE>(c, v, out);
  c->P = P_solve;
  return r;
}
template <typename T, int TILE>
int adj_vcycle_body(wavi_ctx* c, const double* v, double* out) {
  const size_t bytes = sizeof(double) * c->d.N;
  CK(cudaMemcpyAsync(c->r64, v, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemsetAsync(c->x64, 0, bytes, c->st));
  CK(cudaMemsetAsync(c->xc_full64, 0, bytes, c->st));
  CondHandles h{};
  h.active = 0;
  Tally tv, tc;
  if (c->pers_maxt != 0) {
    TRY((enqueue_vcycle_pre<T, TILE>(c, h, tv, false)));
    TRY((enqueue_coarse<T, TILE>(c, h, tv, tc)));
    TRY((enqueue_vcycle_post<T, TILE>(c, h, tv, false)));
  } else {
    TRY((enqueue_vcycle_pre<T, TILE>(c, h, tv)));
    CK(cudaMemcpyAsync(c->hS, c->S, sizeof(DevState), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    int* live = &c->S->cg_continue;
    while (c->hS->cg_continue) {
      for (int k = 0; k < CG_BATCH; ++k) TRY((enqueue_cg_iteration<T, TILE>(c, h, live, tc)));
      CK(cudaMemcpyAsync(c->hS, c->S, sizeof(DevState), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
    }
    TRY((enqueue_vcycle_post<T, TILE>(c, h, tv, false)));
  }
  CK(cudaMemcpyAsync(out, c->x64, bytes, cudaMemcpyDeviceToDevice, c->st));
  return 0;
}

int adj_precond(wavi_ctx* c, const double* v, double* out) {
  if (c->adj_fp32) return adj_vcycle<float, 16>(c, v, out);
  return c->tile == 16 ? adj_vcycle<double, 16>(c, v, out) : adj_vcycle<double, 32>(c, v, out);
}

// Whether the FP32 V-cycle's coarse kernel can run on this FP64 context's cooperative grid (pers_grid
// CTAs of pers_maxt tiles, sized for the FP64 kernel): the FP32 kernel must keep as many CTAs resident.
bool adj_float_fits(wavi_ctx* c) {
  if (c->tile != 16) return false;
  if (c->pers_maxt == 0) return true;  // per-iteration kernels: no cooperative launch
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev);
  const int share = std::max(1, c->pers_share);
  if (c->pers_maxt < 0) {
    int per_sm = 0;
    cudaError_t e = c->coarse_solver == WAVI_COARSE_CG
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_global<float, 16>, 256, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_srcg_global<float, 16>, 256, 0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return (long)per_sm * nsm / share >= c->pers_grid;
  }
  const int cap = c->pers_maxt == 1   ? resident_ctas<1, float, 16>(nsm, c->coarse_solver, false)
                  : c->pers_maxt == 2 ? resident_ctas<2, float, 16>(nsm, c->coarse_solver, false)
                                      : resident_ctas<4, float, 16>(nsm, c->coarse_solver, false);
  return cap / share >= c->pers_grid;
}

// Solve K x = b (K = J_F or J_Fᵀ) by FGMRES(ADJ_RESTART) to ||b - K x|| <= tol ||b||.
int adj_fgmres(wavi_ctx* c, bool transpose, const double* b, double* x, double tol, int maxit, int* iters, double* relres) {
  auto& a = c->adj;
  const int n = c->d.N, m = ADJ_RESTART;
  const int nb = c->ew_blocks;
  int err = 0;
  CK(cudaMemsetAsync(x, 0, sizeof(double) * n, c->st));
  const double bnorm = std::sqrt(adj_dot(c, b, b, &err));
  if (err) return err;
  *iters = 0;
  *relres = 0.0;
  if (bnorm == 0.0) return 0;
  double* r = a.V[0];
  CK(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->st));
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
  auto Hij = [&](int i, int j) -> double& { return H[(size_t)i * m + j]; };
  for (;;) {
    double beta = std::sqrt(adj_dot(c, r, r, &err));
    if (err) return err;
    *relres = beta / bnorm;
    if (*relres <= tol || *iters >= maxit) break;
    k_scale<<<nb, EW_THREADS, 0, c->st>>>(n, 1.0 / beta, r, a.V[0]);
    CKL();
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < m && *iters < maxit; ++k) {
      TRY(adj_precond(c, a.V[k], a.Z[k]));
      TRY(adj_apply(c, transpose, a.Z[k], a.V[k + 1]));
      // w = V[k+1] against V[0..k]: classical Gram-Schmidt twice, then |w|², one host round trip
      double* w = a.V[k + 1];
      const int m1 = k + 1;
      for (int pass = 0; pass < 2; ++pass) {
        k_multi_dot<<<dim3(kGsBlocks, m1), 256, 0, c->st>>>(n, a.Vdev, w, a.gs_partials);
        CKL();
        k_sum_rows<<<1, 256, 0, c->st>>>(a.gs_partials, kGsBlocks, m1, a.hdev + pass * (ADJ_RESTART + 1), 0);
        CKL();
        k_multi_axpy<<<nb, EW_THREADS, 0, c->st>>>(n, a.Vdev, m1, a.hdev + pass * (ADJ_RESTART + 1), w);
        CKL();
      }
      k_multi_dot<<<dim3(kGsBlocks, 1), 256, 0, c->st>>>(n, a.Vdev + k + 1, w, a.gs_partials);
      CKL();
      k_sum_rows<<<1, 256, 0, c->st>>>(a.gs_partials, kGsBlocks, 1, a.hdev + 2 * (ADJ_RESTART + 1), 0);
      CKL();
      double hh[2 * (ADJ_RESTART + 1) + 1];
      CK(cudaMemcpyAsync(hh, a.hdev, sizeof(hh), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      for (int i = 0; i <= k; ++i) Hij(i, k) = hh[i] + hh[ADJ_RESTART + 1 + i];
      const double hn = std::sqrt(std::max(0.0, hh[2 * (ADJ_RESTART + 1)]));
      Hij(k + 1, k) = hn;
      if (hn > 0.0) {
        k_scale<<<nb, EW_THREADS, 0, c->st>>>(n, 1.0 / hn, a.V[k + 1], a.V[k + 1]);
        CKL();
      }
      for (int i = 0; i < k; ++i) {  // previous Givens rotations
        const double t = cs[i] * Hij(i, k) + sn[i] * Hij(i + 1, k);
        Hij(i + 1, k) = -sn[i] * Hij(i, k) + cs[i] * Hij(i + 1, k);
        Hij(i, k) = t;
      }
      const double den = std::hypot(Hij(k, k), Hij(k + 1, k));
      cs[k] = den > 0.0 ? Hij(k, k) / den : 1.0;
      sn[k] = den > 0.0 ? Hij(k + 1, k) / den : 0.0;
      Hij(k, k) = den;
      Hij(k + 1, k) = 0.0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      ++*iters;
      if (std::fabs(g[k + 1]) <= tol * bnorm || hn == 0.0) {
        ++k;
        break;
      }
    }
    for (int i = k - 1; i >= 0; --i) {  // H y = g
      double v = g[i];
      for (int j = i + 1; j < k; ++j) v -= Hij(i, j) * y[j];
      y[i] = Hij(i, i) != 0.0 ? v / Hij(i, i) : 0.0;
    }
    for (int i = 0; i < k; ++i) {
      k_axpy<<<nb, EW_THREADS, 0, c->st>>>(n, y[i], a.Z[i], x);
      CKL();
    }
    // true residual r = b - K x
    TRY(adj_apply(c, transpose, x, a.tb));
    k_scale<<<nb, EW_THREADS, 0, c->st>>>(n, 1.0, b, r);
    CKL();
    k_axpy<<<nb, EW_THREADS, 0, c->st>>>(n, -1.0, a.tb, r);
    CKL();
  }
  return 0;
}

// Linearisation point: the per-cell sensitivities of the converged state, its interior vector, and
// copies of the state the V-cycle preconditioner overwrites.
int adj_prepare(wavi_ctx* c, const wavi_params* p) {
  if (mixed(c)) return fail(c, WAVI_ERR_ARGUMENT, "the adjoint needs a float64 context");
  if (c->has_fixed) return fail(c, WAVI_ERR_ARGUMENT, "the adjoint does not support Dirichlet (isfixed) points");
  if (!c->solved) return fail(c, WAVI_ERR_ARGUMENT, "no converged solve to linearise: call a solve first");
  TRY(adj_alloc(c));
  TRY(set_params(c, p));
  {
    DevParams pa = *c->hP;
    pa.maxiter_coarse = std::min(pa.maxiter_coarse, kAdjCoarseIters);
    pa.aa_depth = 0;  // a fixed preconditioner: no Picard acceleration and the fixed coarse tolerance
    pa.coarse_forcing = 0;
    CK(cudaMemcpyAsync(c->P_adj, &pa, sizeof(DevParams), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));  // (pa lives on this stack frame)
  }
  // the preconditioner's precision: an FP32 V-cycle on the FP32-rounded coefficients of the linearisation
  // (FGMRES is flexible and keeps its own FP64 residual), where the FP32 coarse kernel fits this context
  const bool fits = adj_float_fits(c);
  if (c->opt.adjoint_precond == WAVI_ADJ_PRECOND_FP32 && !fits)
    return fail(c, WAVI_ERR_ARGUMENT, "the FP32 adjoint preconditioner needs 16 x 16 coarse tiles and a resident FP32 coarse kernel");
  c->adj_fp32 = c->opt.adjoint_precond != WAVI_ADJ_PRECOND_FP64 && fits;
  if (c->adj_fp32) {
    const Dims& dd = c->d;
    const double* src[5] = {c->heta_h64, c->dimp64, c->heta_c64, c->beta_m64, c->h_m64};
    float* dst[5] = {c->heta_h32, c->dimp32, c->heta_c32, c->beta_m32, c->h_m32};
    const int n[5] = {dd.Nh, dd.Nh, dd.Nc, dd.N, dd.N};
    for (int k = 0; k < 5; ++k) {
      if (n[k] <= 0) continue;
      k_convert<double, float><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(n[k], src[k], dst[k]);
      CKL();
    }
    // a Chebyshev coarse solve's power vector holds the FP64 solve's doubles: start the FP32 one from zero
    if (c->cheb_eig) CK(cudaMemsetAsync(c->cheb_eig, 0, c->d.N * sizeof(double), c->st));
  }
  auto& a = c->adj;
  const Dims& d = c->d;
  const size_t bytes = sizeof(double) * d.N;
  AdjIn in{c->uv, c->mask_uv, c->h_mask, c->c_mask, c->eta, c->beta, c->quad_f2, c->wc, c->glen_b, c->h, c->zeta, c->qw, c->P};
  k_adj_local<<<(d.Nh + 127) / 128, 128, 0, c->st>>>(d, in, a.cell);
  CKL();
  CK(cudaMemcpyAsync(a.xstate, c->x64, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(a.uv_keep, c->uv, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(a.xc_keep, c->xc_full64, bytes, cudaMemcpyDeviceToDevice, c->st));
  return 0;
}

int adj_restore(wavi_ctx* c) {
  const size_t bytes = sizeof(double) * c->d.N;
  CK(cudaMemcpyAsync(c->uv, c->adj.uv_keep, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(c->xc_full64, c->adj.xc_keep, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(c->x64, c->adj.xstate, bytes, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}


// ---------------------------------------------------------------------------------------------
// Device time stepping (timestep.cuh): update_state! around the solve and update_thickness!
// ---------------------------------------------------------------------------------------------
int step_alloc(wavi_ctx* c) {
  auto& t = c->step;
  if (t.ready) return 0;
  const size_t Nh = c->d.Nh, N = c->d.N;
  int r = 0;
#define SA(p, n) \
  if ((r = dalloc(c, &p, n))) return r;
  SA(t.b, Nh) SA(t.c_param, Nh) SA(t.acc_param, Nh) SA(t.haf, Nh) SA(t.afq, 4 * Nh) SA(t.dhdt, Nh) SA(t.uh, Nh)
  SA(t.vh, Nh) SA(t.ub, Nh) SA(t.vb, Nh) SA(t.us, Nh) SA(t.vs, Nh) SA(t.wav, N) SA(t.h_isfixed, Nh)
#undef SA
  t.ready = true;
  return 0;
}

StepState step_state(wavi_ctx* c) {
  return {c->h_mask, c->mask_uv, c->h, c->s, c->dsdh, c->gf, c->wc, c->acc, c->melt, c->h_uv, c->s_uv, c->gf_uv, c->P};
}
StepBuf step_buf(wavi_ctx* c, double melt) {
  auto& t = c->step;
  return {t.b, t.c_param, t.acc_param, t.h_isfixed, melt, t.haf, t.afq, t.dhdt, t.uh, t.vh, t.ub, t.vb, t.us, t.vs};
}

// The update_state! steps before the solve (update_state.jl:51-147), into the solve's own buffers.
int step_pre(wavi_ctx* c, double melt) {
  const Dims& d = c->d;
  const int hb = (d.Nh + 127) / 128;
  k_step_pre_h<<<hb, 128, 0, c->st>>>(d, step_state(c), step_buf(c, melt));
  CKL();
  k_step_geom_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, step_state(c));
  CKL();
  k_step_pos_quarters<<<hb, 128, 0, c->st>>>(d, c->h_mask, c->step.haf, c->step.afq);
  CKL();
  k_step_pos_gather<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, step_state(c), c->step.afq, c->step.c_param);
  CKL();
  return 0;
}

// update_wavelets! (update_wavelets.jl:6-32) on the context's velocities: forward Haar transform of
// mask ⊙ (u, v), the threshold |w| >= wavelet_threshold into the wavelet mask, the coarse cache cleared.
int step_wavelets(wavi_ctx* c) {
  const Dims& d = c->d;
  k_haar<double, double, 2, false, false><<<c->haar_grid, c->haar_block, 0, c->st>>>(
      d, c->sp.levels, c->uv, c->step.wav, nullptr, c->mask_uv, nullptr, c->partials, nullptr);
  CKL();
  k_step_wavelet_mask<<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->step.wav, c->sp.wavelet_threshold, c->wmask_uv,
                                                               c->xc_full64);
  CKL();
  return 0;
}

// After the solve: velocities on the h grid, dh/dt, the wavelet coarse space (update_state.jl:17-19),
// then update_thickness!.
int step_post(wavi_ctx* c, double melt, double dt, double h_min) {
  const Dims& d = c->d;
  const int hb = (d.Nh + 127) / 128;
  k_step_post_h<<<hb, 128, 0, c->st>>>(d, step_state(c), step_buf(c, melt), c->uv, c->beta, c->quad_f1, c->quad_f2);
  CKL();
  TRY(step_wavelets(c));
  k_step_thickness<<<hb, 128, 0, c->st>>>(d, step_state(c), step_buf(c, melt), dt, h_min);
  CKL();
  return 0;
}

}  // namespace

namespace wavi {
// Errors of entry points that have no context (wavi_ctx_create, wavi_residual_noalloc).
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace wavi

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

int wavi_abi_version(void) { return WAVI_ABI_VERSION; }

int wavi_abi_struct_sizes(int32_t* out, int n) {
  const int32_t s[6] = {(int32_t)sizeof(wavi_grid_desc), (int32_t)sizeof(wavi_params),
                        (int32_t)sizeof(wavi_solver_params), (int32_t)sizeof(wavi_options),
                        (int32_t)sizeof(wavi_fields), (int32_t)sizeof(wavi_stats)};
  for (int i = 0; out && i < n && i < 6; ++i) out[i] = s[i];
  return 6;
}

int wavi_device_count(void) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return WAVI_ERR_NO_DEVICE;
  return n;
}

const char* wavi_last_error(const wavi_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

void* wavi_ctx_stream(const wavi_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }

static int create_ctx(const wavi_grid_desc* g, const wavi_solver_params* sp, const wavi_options* opt, int share,
                      wavi_ctx** out) {
  wavi_ctx* c = nullptr;
  if (!out) return fail(nullptr, WAVI_ERR_ARGUMENT, "out is null");
  *out = nullptr;
  if (!g || !sp || !opt) return fail(nullptr, WAVI_ERR_ARGUMENT, "null argument");
  if (g->nx < 2 || g->ny < 2 || g->nsigma < 2) return fail(nullptr, WAVI_ERR_ARGUMENT, "nx, ny, nsigma must be > 1");
  if (!g->sigma || !g->quadrature_weights || !g->h_mask || !g->u_iszero || !g->v_iszero || !g->u_isfixed || !g->v_isfixed)
    return fail(nullptr, WAVI_ERR_ARGUMENT, "grid arrays must not be null");
  if (sp->levels < 0 || sp->levels > 4) return fail(nullptr, WAVI_ERR_ARGUMENT, "levels must be in 0..4 (got %d)", sp->levels);
  if (sp->n_iter_viscosity < 1) return fail(nullptr, WAVI_ERR_ARGUMENT, "n_iter_viscosity must be >= 1");
  if (sp->nsmooth < 0) return fail(nullptr, WAVI_ERR_ARGUMENT, "nsmooth must be >= 0");
  if (opt->precision != WAVI_PRECISION_FP64 && opt->precision != WAVI_PRECISION_MIXED)
    return fail(nullptr, WAVI_ERR_ARGUMENT, "unknown precision %d", opt->precision);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(nullptr, WAVI_ERR_NO_DEVICE, "no CUDA device");
  if (opt->device < 0 || opt->device >= ndev) return fail(nullptr, WAVI_ERR_ARGUMENT, "device %d out of range", opt->device);
  if ((long)(g->nx + 1) * (g->ny + 1) > (1L << 30)) return fail(nullptr, WAVI_ERR_ARGUMENT, "grid too large");
  c = new wavi_ctx();
  c->pers_share = std::max(1, share);
  c->dev = opt->device;
  c->sp = *sp;
  c->opt = *opt;
  c->tile = sp->levels <= 3 ? 16 : 32;
  auto bail = [&](int code) {
    g_create_error = c->err;
    wavi_ctx_destroy(c);
    return code;
  };
  if (cudaSetDevice(c->dev) != cudaSuccess) return bail(fail(c, WAVI_ERR_CUDA, "cudaSetDevice failed"));
  Dims& d = c->d;
  d.nx = g->nx;
  d.ny = g->ny;
  d.ns = g->nsigma;
  d.Nh = d.nx * d.ny;
  d.Nu = (d.nx + 1) * d.ny;
  d.Nv = d.nx * (d.ny + 1);
  d.Nc = (d.nx - 1) * (d.ny - 1);
  d.N = d.Nu + d.Nv;
  d.dx = g->dx;
  d.dy = g->dy;
  d.rdx = 1.0 / g->dx;
  d.rdy = 1.0 / g->dy;
  d.rdx_f = (float)d.rdx;
  d.rdy_f = (float)d.rdy;
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(c, WAVI_ERR_CUDA, "stream creation failed"));
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  cudaEventCreate(&c->evc0);
  cudaEventCreate(&c->evc1);
  // masks (src/Fields/Fields.jl:28-35; utilities.jl:475-507; UGrid.jl:76)
  std::vector<uint8_t> hm((size_t)d.Nh), cm((size_t)d.Nc, 0), mk((size_t)d.N, 0), in((size_t)d.N, 0), fx((size_t)d.N, 0);
  for (int i = 0; i < d.Nh; ++i) hm[i] = g->h_mask[i] ? 1 : 0;
  for (int j = 0; j < d.ny; ++j)
    for (int i = 0; i < d.nx; ++i)
      if (hm[i + d.nx * j]) {
        mk[i + (d.nx + 1) * j] = mk[i + 1 + (d.nx + 1) * j] = 1;
        mk[d.Nu + i + d.nx * j] = mk[d.Nu + i + d.nx * (j + 1)] = 1;
      }
  for (int j = 0; j < d.ny - 1; ++j)
    for (int i = 0; i < d.nx - 1; ++i)
      cm[i + (d.nx - 1) * j] = hm[i + d.nx * j] && hm[i + d.nx * (j + 1)] && hm[i + 1 + d.nx * j] && hm[i + 1 + d.nx * (j + 1)];
  for (int i = 0; i < d.Nu; ++i) {
    if (g->u_iszero[i]) mk[i] = 0;
    fx[i] = g->u_isfixed[i] ? 1 : 0;
  }
  for (int i = 0; i < d.Nv; ++i) {
    if (g->v_iszero[i]) mk[d.Nu + i] = 0;
    fx[d.Nu + i] = g->v_isfixed[i] ? 1 : 0;
  }
  int ninner = 0;
  for (int i = 0; i < d.N; ++i) {
    in[i] = mk[i] && !fx[i];
    ninner += in[i];
    if (fx[i]) c->has_fixed = true;
  }
  if (ninner == 0) return bail(fail(c, WAVI_ERR_ARGUMENT, "the interior mask is empty"));
  c->h_inner_host = in;
  int r = 0;
  const size_t Nh = d.Nh, Nc = d.Nc, N = d.N, N3 = (size_t)d.Nh * d.ns;
#define A(p, n) \
  if ((r = dalloc(c, &c->p, n))) return bail(r);
  A(h_mask, Nh) A(c_mask, Nc) A(mask_uv, N) A(inner_uv, N) A(fixed_uv, N) A(wmask_uv, N)
  A(h, Nh) A(s, Nh) A(dsdh, Nh) A(gf, Nh) A(wc, Nh) A(acc, Nh) A(melt, Nh)
  A(h_uv, N) A(s_uv, N) A(gf_uv, N) A(glen_b, N3) A(zeta, (size_t)d.ns) A(qw, (size_t)d.ns)
  A(zeta_f, (size_t)d.ns) A(qw_f, (size_t)d.ns)
  A(uv, N) A(eta, N3) A(beta, Nh) A(quad_f2, Nh) A(xc_full64, N)
  A(shelf, Nh) A(av_speed, Nh) A(bed_speed, Nh) A(tau, Nh) A(eta_av, Nh) A(quad_f1, Nh) A(beta_eff, Nh)
  A(beta_eff_uv, N) A(resid_uv, N) A(hn, Nh)
  A(heta_h64, Nh) A(heta_c64, Nc) A(dimp64, Nh) A(beta_m64, N) A(h_m64, N)
  A(heta_h32, Nh) A(heta_c32, Nc) A(dimp32, Nh) A(beta_m32, N) A(h_m32, N)
  A(x64, N) A(b64, N) A(r64, N) A(xfix64, N) A(wmask_in, N) A(comp_stage, N)
#undef A
  c->mask_offsets_v = (d.Nu + MS_BLOCK - 1) / MS_BLOCK;
  if ((r = dalloc(c, &c->mask_offsets, (size_t)c->mask_offsets_v + (d.Nv + MS_BLOCK - 1) / MS_BLOCK))) return bail(r);
  for (void** p : {&c->rs, &c->corr[0], &c->corr[1], &c->rsm[0], &c->rsm[1], &c->diag, &c->xc, &c->rc, &c->uc, &c->cc,
                   &c->w, &c->bc}) {
    double* q = nullptr;
    if ((r = dalloc(c, &q, N))) return bail(r);
    *p = q;
  }
  // launch shapes
  c->op_block = dim3(OP_TX, OP_TY);
  c->op_grid = dim3((d.nx + 1 + OP_TX - 1) / OP_TX, (d.ny + 1 + OP_TY - 1) / OP_TY);
  c->pt_block = dim3(32, 8);
  c->pt_grid = dim3((d.nx + 1 + 31) / 32, (d.ny + 1 + 7) / 8);
  const int B = 1 << (sp->levels + 1);
  c->haar_block = dim3(B, B);
  c->haar_grid = dim3((d.nx + 1 + B - 1) / B, (d.ny + 1 + B - 1) / B, 2);
  c->tile_block = dim3(c->tile, c->tile);
  c->tile_grid = dim3((d.nx + 1 + c->tile - 1) / c->tile, (d.ny + 1 + c->tile - 1) / c->tile);
  c->ew_blocks = (int)std::min<size_t>((N + EW_THREADS - 1) / EW_THREADS, 152 * 4);
  {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev);
    stream_shape(d, std::max(nsm, 1), c->st_grid, c->st_rows);
    const long points = (long)(d.nx + 1) * (d.ny + 1);
    if (opt->stencil_kernel < 0 || opt->stencil_kernel > 2)
      return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown stencil_kernel %d", opt->stencil_kernel));
    c->stream_op = opt->stencil_kernel == 2 || (opt->stencil_kernel == 0 && points >= kStreamMinPoints);
  }
  const int pt_blocks = (int)(c->pt_grid.x * c->pt_grid.y);
  const int op_blocks = (int)(c->op_grid.x * c->op_grid.y);
  const int tile_blocks = (int)(c->tile_grid.x * c->tile_grid.y);
  const int haar_blocks = (int)(c->haar_grid.x * c->haar_grid.y * c->haar_grid.z);
  c->ntx = (int)c->tile_grid.x;
  c->nty = (int)c->tile_grid.y;
  // coarse solver: the reference's cg! recurrence, or (persistent kernel only) single-reduction CG
  const int want = opt->coarse_solver;
  if (want < WAVI_COARSE_AUTO || want > WAVI_COARSE_PIPELINED_CHEBYSHEV)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown coarse_solver %d", want));
  if (opt->coarse_kernel < 0 || opt->coarse_kernel > 3)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown coarse_kernel %d", opt->coarse_kernel));
  if (opt->cheb_steps != 0 && (opt->cheb_steps < 1 || opt->cheb_steps > 15 || opt->cheb_steps % 2 == 0))
    return bail(fail(c, WAVI_ERR_ARGUMENT, "cheb_steps must be 0 (default) or odd in 1..15 (got %d)", opt->cheb_steps));
  if (opt->coarse_sums < WAVI_SUMS_DEFAULT || opt->coarse_sums > WAVI_SUMS_FP64_SOLVE)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown coarse_sums %d", opt->coarse_sums));
  if (opt->viscosity < WAVI_VISCOSITY_DEFAULT || opt->viscosity > WAVI_VISCOSITY_FP64)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown viscosity precision %d", opt->viscosity));
  if (opt->picard_accel < WAVI_PICARD_AUTO || opt->picard_accel > WAVI_PICARD_ANDERSON)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown picard_accel %d", opt->picard_accel));
  if (opt->anderson_depth < 0 || opt->anderson_depth > kAAMax)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "anderson_depth must be 0 (default) or 1..%d (got %d)", kAAMax,
                     opt->anderson_depth));
  const bool anderson = opt->picard_accel == WAVI_PICARD_ANDERSON || (opt->picard_accel == WAVI_PICARD_AUTO && mixed(c));
  c->aa_depth = anderson ? (opt->anderson_depth > 0 ? opt->anderson_depth : kAADefaultDepth) : 0;
  if (opt->coarse_forcing < WAVI_FORCING_AUTO || opt->coarse_forcing > WAVI_FORCING_ADAPTIVE)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown coarse_forcing %d", opt->coarse_forcing));
  c->forcing = opt->coarse_forcing == WAVI_FORCING_ADAPTIVE || (opt->coarse_forcing == WAVI_FORCING_AUTO && mixed(c));
  if (opt->adjoint_precond < WAVI_ADJ_PRECOND_AUTO || opt->adjoint_precond > WAVI_ADJ_PRECOND_FP32)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "unknown adjoint_precond %d", opt->adjoint_precond));
  c->visc32 = mixed(c) && opt->viscosity != WAVI_VISCOSITY_FP64;
  if (want != WAVI_COARSE_AUTO && want != WAVI_COARSE_CG && opt->coarse_kernel == 2)
    return bail(fail(c, WAVI_ERR_ARGUMENT, "the single-reduction coarse solvers run only in the persistent coarse kernel"));
  // auto: FP64 runs the reference's cg!; mixed runs the Chebyshev-Jacobi single-reduction CG (register-
  // resident or, on grids too large for that, global-memory), also where the ice mask cuts the domain: there
  // masked Haar functions can coincide on the interior and R A P turns singular, which the FP32 solve
  // survives because a coarse solve that misses its tolerance does not become the next warm start
  c->coarse_solver = want == WAVI_COARSE_AUTO ? (mixed(c) ? WAVI_COARSE_SRCG_CHEBYSHEV : WAVI_COARSE_CG) : want;
  c->acc64 = mixed(c) && opt->coarse_sums == WAVI_SUMS_FP64;
  c->coarse64 = mixed(c) && opt->coarse_sums == WAVI_SUMS_FP64_SOLVE;
  if (c->coarse64 && (opt->coarse_kernel == 2 || c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV))
    return bail(fail(c, WAVI_ERR_ARGUMENT,
                     "the FP64 coarse solve runs in the persistent coarse kernels, with a solver other than the "
                     "pipelined one"));
  if (c->acc64 && (c->tile != 16 || opt->coarse_kernel == 2 || opt->coarse_kernel == 3 || c->coarse_solver == WAVI_COARSE_CG ||
                   c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV))
    return bail(fail(c, WAVI_ERR_ARGUMENT,
                     "FP64 coarse sums need a single-reduction coarse solver on the register-resident kernel with "
                     "16 x 16 tiles"));
  if (opt->coarse_kernel != 2) {
    if (mixed(c) && !c->coarse64)
      c->tile == 16 ? choose_persistent<float, 16>(c) : choose_persistent<float, 32>(c);
    else
      c->tile == 16 ? choose_persistent<double, 16>(c) : choose_persistent<double, 32>(c);
    if (c->pers_maxt == 0 && c->coarse_solver != WAVI_COARSE_CG) {
      if (want != WAVI_COARSE_AUTO)
        return bail(fail(c, WAVI_ERR_ARGUMENT, "the single-reduction coarse CG does not fit this grid on this device"));
      c->coarse_solver = WAVI_COARSE_CG;
      c->tile == 16 ? (mixed(c) && !c->coarse64 ? choose_persistent<float, 16>(c) : choose_persistent<double, 16>(c))
                    : (mixed(c) && !c->coarse64 ? choose_persistent<float, 32>(c) : choose_persistent<double, 32>(c));
    }
    if ((opt->coarse_kernel == 1 || opt->coarse_kernel == 3) && c->pers_maxt == 0)
      return bail(fail(c, WAVI_ERR_ARGUMENT, "the persistent coarse CG does not fit this grid on this device"));
    if (c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV && (!mixed(c) || c->tile != 16 || c->pers_maxt <= 0))
      return bail(fail(c, WAVI_ERR_ARGUMENT,
                       "the pipelined coarse CG needs mixed precision, 16 x 16 tiles and the register-resident kernel"));
    if (c->acc64 && (c->pers_maxt <= 0 || c->pers_maxt > 2))
      return bail(fail(c, WAVI_ERR_ARGUMENT, "FP64 coarse sums: the register-resident kernel does not fit this grid"));
  } else {
    c->coarse_solver = WAVI_COARSE_CG;
  }
  // reduction partials: per-block slots of the one-pass kernels, and 2 parities x 4 sums per CTA of the
  // persistent kernel
  c->max_partials = 4 * std::max({pt_blocks, op_blocks, tile_blocks, haar_blocks, c->ew_blocks, 1});
  c->max_partials = std::max(c->max_partials, 8 * std::max(c->pers_grid, 1));
  if ((r = dalloc(c, &c->partials, (size_t)c->max_partials))) return bail(r);
  if ((r = dalloc(c, &c->bar, 1))) return bail(r);
  if ((r = dalloc(c, &c->selftest, 2))) return bail(r);
  if (c->pers_maxt > 0) {
    if ((r = dalloc(c, &c->halo_box, (size_t)2 * c->ntx * c->nty * 8 * c->tile))) return bail(r);
    if (mixed(c) && c->tile == 16 && !c->stream_op && smoother_fits(c)) {
      if ((r = dalloc(c, &c->smooth_box, (size_t)2 * c->ntx * c->nty * 8 * 16))) return bail(r);
      c->fused_smooth = true;
    }
  }
  {
    double* q = nullptr;
    if ((r = dalloc(c, &q, N))) return bail(r);
    c->dcoarse = q;
    if (c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV || c->coarse_solver == WAVI_COARSE_PIPELINED_CHEBYSHEV) {
      if ((r = dalloc(c, &q, N))) return bail(r);
      c->cheb_eig = q;
    }
    if (c->coarse64) {
      if ((r = dalloc(c, &c->bc64, N))) return bail(r);
      if ((r = dalloc(c, &c->xc64, N))) return bail(r);
    }
    if (c->pers_maxt < 0) {
      if ((r = dalloc(c, &q, N))) return bail(r);
      c->gz = q;
      if ((r = dalloc(c, &q, N))) return bail(r);
      c->gw = q;
      if (c->coarse_solver == WAVI_COARSE_SRCG_CHEBYSHEV) {
        if ((r = dalloc(c, &q, N))) return bail(r);
        c->w2 = q;
        if ((r = dalloc(c, &q, N))) return bail(r);
        c->gcd = q;
      }
    }
  }
  if (c->aa_depth > 0) {
    if ((r = dalloc(c, &c->aa.dF, (size_t)c->aa_depth * N))) return bail(r);
    if ((r = dalloc(c, &c->aa.dG, (size_t)c->aa_depth * N))) return bail(r);
    if ((r = dalloc(c, &c->aa.fprev, N))) return bail(r);
    if ((r = dalloc(c, &c->aa.gprev, N))) return bail(r);
    if ((r = dalloc(c, &c->aa.partials, (size_t)2 * kAAMax * c->ew_blocks))) return bail(r);
  }
  if ((r = dalloc(c, &c->P, 1))) return bail(r);
  if ((r = dalloc(c, &c->S, 1))) return bail(r);
  if (cudaMallocHost(&c->hP, sizeof(DevParams)) != cudaSuccess || cudaMallocHost(&c->hS, sizeof(DevState)) != cudaSuccess)
    return bail(fail(c, WAVI_ERR_ALLOC, "pinned allocation failed"));
  std::vector<double> zeta((size_t)d.ns);
  for (int k = 0; k < d.ns; ++k) zeta[k] = 1.0 - g->sigma[k];  // Grid.jl:170
  cudaError_t e = cudaSuccess;
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->h_mask, hm.data(), Nh, cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->c_mask, cm.data(), std::max<size_t>(Nc, 1), cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->mask_uv, mk.data(), N, cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->inner_uv, in.data(), N, cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->fixed_uv, fx.data(), N, cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->zeta, zeta.data(), sizeof(double) * d.ns, cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->qw, g->quadrature_weights, sizeof(double) * d.ns, cudaMemcpyHostToDevice);
  std::vector<float> zeta_f((size_t)d.ns), qw_f((size_t)d.ns);
  for (int k = 0; k < d.ns; ++k) {
    zeta_f[k] = (float)zeta[k];
    qw_f[k] = (float)g->quadrature_weights[k];
  }
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->zeta_f, zeta_f.data(), sizeof(float) * d.ns, cudaMemcpyHostToDevice);
  e = (e != cudaSuccess) ? e : cudaMemcpy(c->qw_f, qw_f.data(), sizeof(float) * d.ns, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bail(fail(c, WAVI_ERR_CUDA, "mask upload: %s", cudaGetErrorString(e)));
  *out = c;
  return WAVI_OK;
}

int wavi_ctx_create(const wavi_grid_desc* g, const wavi_solver_params* sp, const wavi_options* opt, wavi_ctx** out) {
  return create_ctx(g, sp, opt, 1, out);
}

int wavi_ctx_destroy(wavi_ctx* c) {
  if (!c) return WAVI_OK;
  cudaSetDevice(c->dev);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  for (void* p : c->allocs) cudaFree(p);
  if (c->hP) cudaFreeHost(c->hP);
  if (c->hS) cudaFreeHost(c->hS);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->evc0) cudaEventDestroy(c->evc0);
  if (c->evc1) cudaEventDestroy(c->evc1);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return WAVI_OK;
}

int wavi_solve_velocities(wavi_ctx* c, const wavi_params* p, wavi_fields* f, wavi_stats* st) {
  TRY(check_ctx(c));
  TRY(check_params(c, p));
  if (!f) return fail(c, WAVI_ERR_ARGUMENT, "fields is null");
  TRY(upload(c, f, true));
  TRY(solve_resident(c, p, st));
  return download(c, f, true);
}

int wavi_solve_velocities_device(wavi_ctx* c, const wavi_params* p, wavi_fields* f, wavi_stats* st) {
  TRY(check_ctx(c));
  TRY(check_params(c, p));
  if (!f) return fail(c, WAVI_ERR_ARGUMENT, "fields is null");
  TRY(upload(c, f, false));
  TRY(solve_resident(c, p, st));
  TRY(download(c, f, false));
  CK(cudaStreamSynchronize(c->st));  // results are in the caller's arrays on return
  return 0;
}

int wavi_relinearise_device(wavi_ctx* c, const wavi_params* p, wavi_fields* f) {
  TRY(check_ctx(c));
  TRY(check_params(c, p));
  if (!f) return fail(c, WAVI_ERR_ARGUMENT, "fields is null");
  TRY(upload(c, f, false));
  TRY(set_params(c, p));
  const Dims& d = c->d;
  RelinIn in{c->uv, c->mask_uv, c->h_mask, c->c_mask, c->h, c->wc, c->glen_b, c->dsdh, c->zeta, c->qw, c->P, c->zeta_f, c->qw_f};
  RelinOut out{c->shelf, c->av_speed, c->bed_speed, c->beta, c->tau, c->eta, c->eta_av, c->quad_f1, c->quad_f2,
               c->beta_eff, c->heta_h64, c->dimp64, mixed(c) ? c->heta_h32 : nullptr, mixed(c) ? c->dimp32 : nullptr,
               c->hn};
  const int nb = (d.Nh + 127) / 128;
  if (visc32(c))
    k_relin_h<float><<<nb, 128, 0, c->st>>>(d, in, out);
  else
    k_relin_h<double><<<nb, 128, 0, c->st>>>(d, in, out);
  CKL();
  RelinUVIn uin{c->mask_uv, c->h_mask, c->c_mask, c->beta_eff, c->gf, c->gf_uv, c->h_uv, c->hn};
  RelinUVOut uout{c->beta_eff_uv, c->beta_m64, c->h_m64, c->heta_c64, mixed(c) ? c->beta_m32 : nullptr,
                  mixed(c) ? c->h_m32 : nullptr, mixed(c) ? c->heta_c32 : nullptr};
  k_relin_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, uin, uout);
  CKL();
  TRY(download(c, f, false));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int wavi_apply_operator_device(wavi_ctx* c, int precision, const void* in_uv, void* out_uv) {
  TRY(check_ctx(c));
  if (!in_uv || !out_uv) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  if (precision == WAVI_PRECISION_FP64) {
    TRY(launch_op<double>(c, (const double*)in_uv, (double*)out_uv));
  } else if (precision == WAVI_PRECISION_MIXED && mixed(c)) {
    TRY(launch_op<float>(c, (const float*)in_uv, (float*)out_uv));
  } else {
    return fail(c, WAVI_ERR_ARGUMENT, "float32 operator needs a mixed-precision context");
  }
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int wavi_time_operator_device(wavi_ctx* c, int precision, const void* in_uv, void* out_uv, int repeats, double* avg_ms) {
  TRY(check_ctx(c));
  if (!in_uv || !out_uv || !avg_ms || repeats < 1) return fail(c, WAVI_ERR_ARGUMENT, "bad arguments");
  if (precision != WAVI_PRECISION_FP64 && !(precision == WAVI_PRECISION_MIXED && mixed(c)))
    return fail(c, WAVI_ERR_ARGUMENT, "float32 operator needs a mixed-precision context");
  CK(cudaEventRecord(c->ev0, c->st));
  for (int k = 0; k < repeats; ++k) {
    if (precision == WAVI_PRECISION_FP64)
      TRY(launch_op<double>(c, (const double*)in_uv, (double*)out_uv));
    else
      TRY(launch_op<float>(c, (const float*)in_uv, (float*)out_uv));
  }
  CK(cudaEventRecord(c->ev1, c->st));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  *avg_ms = (double)ms / repeats;
  return 0;
}

int wavi_time_relinearise_device(wavi_ctx* c, int repeats, double* avg_ms_h, double* avg_ms_uv) {
  TRY(check_ctx(c));
  if (!avg_ms_h || !avg_ms_uv || repeats < 1) return fail(c, WAVI_ERR_ARGUMENT, "bad arguments");
  if (!c->fields_loaded) return fail(c, WAVI_ERR_ARGUMENT, "no fields on the context yet (relinearise or solve first)");
  const Dims& d = c->d;
  RelinIn in{c->uv, c->mask_uv, c->h_mask, c->c_mask, c->h, c->wc, c->glen_b, c->dsdh, c->zeta, c->qw, c->P, c->zeta_f, c->qw_f};
  RelinOut out{c->shelf, c->av_speed, c->bed_speed, c->beta, c->tau, c->eta, c->eta_av, c->quad_f1, c->quad_f2,
               c->beta_eff, c->heta_h64, c->dimp64, mixed(c) ? c->heta_h32 : nullptr, mixed(c) ? c->dimp32 : nullptr,
               c->hn};
  RelinUVIn uin{c->mask_uv, c->h_mask, c->c_mask, c->beta_eff, c->gf, c->gf_uv, c->h_uv, c->hn};
  RelinUVOut uout{c->beta_eff_uv, c->beta_m64, c->h_m64, c->heta_c64, mixed(c) ? c->beta_m32 : nullptr,
                  mixed(c) ? c->h_m32 : nullptr, mixed(c) ? c->heta_c32 : nullptr};
  const int nb = (d.Nh + 127) / 128;
  float ms = 0.f;
  CK(cudaEventRecord(c->ev0, c->st));
  for (int k = 0; k < repeats; ++k) {
    if (visc32(c))
      k_relin_h<float><<<nb, 128, 0, c->st>>>(d, in, out);
    else
      k_relin_h<double><<<nb, 128, 0, c->st>>>(d, in, out);
    CKL();
  }
  CK(cudaEventRecord(c->ev1, c->st));
  CK(cudaEventSynchronize(c->ev1));
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  *avg_ms_h = (double)ms / repeats;
  CK(cudaEventRecord(c->ev0, c->st));
  for (int k = 0; k < repeats; ++k) {
    k_relin_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, uin, uout);
    CKL();
  }
  CK(cudaEventRecord(c->ev1, c->st));
  CK(cudaEventSynchronize(c->ev1));
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  *avg_ms_uv = (double)ms / repeats;
  return 0;
}

int wavi_op_diagonal_device(wavi_ctx* c, int precision, void* diag_uv) {
  TRY(check_ctx(c));
  if (!diag_uv) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  if (precision == WAVI_PRECISION_FP64)
    k_op_diag<double><<<c->pt_grid, c->pt_block, 0, c->st>>>(c->d, coef<double>(c), (double*)diag_uv);
  else if (mixed(c))
    k_op_diag<float><<<c->pt_grid, c->pt_block, 0, c->st>>>(c->d, coef<float>(c), (float*)diag_uv);
  else
    return fail(c, WAVI_ERR_ARGUMENT, "float32 diagonal needs a mixed-precision context");
  CKL();
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int wavi_selftest_conversions(wavi_ctx* c, long long n, long long* mismatches) {
  TRY(check_ctx(c));
  if (!mismatches) return fail(c, WAVI_ERR_ARGUMENT, "null pointer");
  if (n < 0 || n > (1LL << 32)) return fail(c, WAVI_ERR_ARGUMENT, "n must be in 0..2^32 (got %lld)", n);
  CK(cudaMemsetAsync(c->selftest, 0, 2 * sizeof(unsigned long long), c->st));
  int nsm = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev));
  k_selftest_conversions<<<std::max(1, nsm) * 8, 256, 0, c->st>>>(n, c->selftest);
  CKL();
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(&out, c->selftest, sizeof(out), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *mismatches = (long long)out;
  return 0;
}

int wavi_selftest_watchdog(wavi_ctx* c, int* fired) {
  TRY(check_ctx(c));
  if (!fired) return fail(c, WAVI_ERR_ARGUMENT, "null pointer");
  CK(cudaMemsetAsync(c->selftest, 0, 2 * sizeof(unsigned long long), c->st));
  k_reset_barrier<<<1, 32, 0, c->st>>>(c->bar, (const DevParams*)c->P);
  CKL();
  k_selftest_wait<<<1, 32, 0, c->st>>>(c->bar, c->selftest, (int*)(c->selftest + 1));
  CKL();
  int out = 0;
  CK(cudaMemcpyAsync(&out, c->selftest + 1, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  k_reset_barrier<<<1, 32, 0, c->st>>>(c->bar, (const DevParams*)c->P);  // the barrier idle again (no error)
  CKL();
  CK(cudaStreamSynchronize(c->st));
  *fired = out;
  return 0;
}

int wavi_coarse_diagonal_device(wavi_ctx* c, int precision, void* diag_uv) {
  TRY(check_ctx(c));
  if (!diag_uv) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  if (precision == WAVI_PRECISION_FP64) {
    if (c->tile == 16)
      launch_coarse_diag<double, 16>(c, (double*)diag_uv);
    else
      launch_coarse_diag<double, 32>(c, (double*)diag_uv);
  } else if (precision == WAVI_PRECISION_MIXED && mixed(c)) {
    if (c->tile == 16)
      launch_coarse_diag<float, 16>(c, (float*)diag_uv);
    else
      launch_coarse_diag<float, 32>(c, (float*)diag_uv);
  } else {
    return fail(c, WAVI_ERR_ARGUMENT, "float32 diagonal needs a mixed-precision context");
  }
  CKL();
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int wavi_adjoint_device(wavi_ctx* c, const wavi_params* p, const double* dJ_du, const double* dJ_dv, double* dJ_dlogC,
                        double* dJ_dlogA, double tol, int maxiter, wavi_adjoint_stats* stats) {
  TRY(check_ctx(c));
  TRY(check_params(c, p));
  if (!dJ_du || !dJ_dv || !dJ_dlogC || !dJ_dlogA) return fail(c, WAVI_ERR_ARGUMENT, "null adjoint argument");
  if (!(tol > 0.0) || maxiter < 1) return fail(c, WAVI_ERR_ARGUMENT, "tol must be > 0 and maxiter >= 1");
  const auto t0 = std::chrono::steady_clock::now();
  TRY(adj_prepare(c, p));
  auto& a = c->adj;
  const Dims& d = c->d;
  CK(cudaMemcpyAsync(a.b, dJ_du, sizeof(double) * d.Nu, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(a.b + d.Nu, dJ_dv, sizeof(double) * d.Nv, cudaMemcpyDeviceToDevice, c->st));
  k_mask_inner<<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, a.b);
  CKL();
  int iters = 0;
  double rr = 0.0;
  int r = adj_fgmres(c, true, a.b, a.x, tol, maxiter, &iters, &rr);
  if (!r) {
    k_adj_cell<<<(d.Nh + 127) / 128, 128, 0, c->st>>>(d, a.cell, adj_uv(c), c->inner_uv, a.xstate, a.x, nullptr, nullptr,
                                                     dJ_dlogC, dJ_dlogA);
    if (cudaGetLastError() != cudaSuccess) r = fail(c, WAVI_ERR_CUDA, "adjoint gradient kernel");
  }
  const int rr2 = adj_restore(c);
  if (r) return r;
  if (rr2) return rr2;
  if (stats) {
    stats->status = rr <= tol ? WAVI_OK : WAVI_ERR_NOT_CONVERGED;
    stats->iterations = iters;
    stats->rel_residual = rr;
    stats->elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return 0;
}

int wavi_tangent_device(wavi_ctx* c, const wavi_params* p, const double* dlogC, const double* dlogA, double* du,
                        double* dv, double tol, int maxiter, wavi_adjoint_stats* stats) {
  TRY(check_ctx(c));
  TRY(check_params(c, p));
  if (!du || !dv) return fail(c, WAVI_ERR_ARGUMENT, "null tangent output");
  if (!(tol > 0.0) || maxiter < 1) return fail(c, WAVI_ERR_ARGUMENT, "tol must be > 0 and maxiter >= 1");
  const auto t0 = std::chrono::steady_clock::now();
  TRY(adj_prepare(c, p));
  auto& a = c->adj;
  const Dims& d = c->d;
  // b = -A(∂coef/∂θ dθ) x
  k_tlm_cell<<<(d.Nh + 127) / 128, 128, 0, c->st>>>(d, a.cell, adj_uv(c), nullptr, dlogC, dlogA, a.dheta_h, a.dhn, a.dbeff);
  CKL();
  k_tlm_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, adj_uv(c), a.dhn, a.dbeff, a.dbeta_m, a.dheta_c);
  CKL();
  const OpCoef<double> dcf{a.dheta_h, a.dheta_c, a.zero_h, a.dbeta_m, c->h_m64, c->inner_uv};
  k_op<double, double, 0><<<c->op_grid, c->op_block, 0, c->st>>>(d, dcf, a.xstate, nullptr, a.tb, c->partials, nullptr);
  CKL();
  k_scale<<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, -1.0, a.tb, a.b);
  CKL();
  int iters = 0;
  double rr = 0.0;
  int r = adj_fgmres(c, false, a.b, a.x, tol, maxiter, &iters, &rr);
  if (!r && (cudaMemcpyAsync(du, a.x, sizeof(double) * d.Nu, cudaMemcpyDeviceToDevice, c->st) != cudaSuccess ||
             cudaMemcpyAsync(dv, a.x + d.Nu, sizeof(double) * d.Nv, cudaMemcpyDeviceToDevice, c->st) != cudaSuccess))
    r = fail(c, WAVI_ERR_CUDA, "tangent output copy");
  const int rr2 = adj_restore(c);
  if (r) return r;
  if (rr2) return rr2;
  if (stats) {
    stats->status = rr <= tol ? WAVI_OK : WAVI_ERR_NOT_CONVERGED;
    stats->iterations = iters;
    stats->rel_residual = rr;
    stats->elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return 0;
}

int wavi_run_device(wavi_ctx* c, const wavi_params* p, double dt, int nsteps, const wavi_step_inputs* in, wavi_fields* f,
                    wavi_step_outputs* out, wavi_stats* st) {
  TRY(check_ctx(c));
  TRY(check_params(c, p));
  if (!in || !f || !in->bed || !in->weertman_c || !in->accumulation || !in->h_isfixed)
    return fail(c, WAVI_ERR_ARGUMENT, "null time-stepping argument");
  if (nsteps < 0 || !(dt >= 0.0)) return fail(c, WAVI_ERR_ARGUMENT, "nsteps must be >= 0 and dt >= 0");
  TRY(step_alloc(c));
  const Dims& d = c->d;
  auto& t = c->step;
  wavi_params pp = *p;
  pp.dt = dt;  // set_dt_in_model! (Simulation.jl:56-59)
  TRY(upload(c, f, false));
  CK(cudaMemcpyAsync(t.b, in->bed, sizeof(double) * d.Nh, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(t.c_param, in->weertman_c, sizeof(double) * d.Nh, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(t.acc_param, in->accumulation, sizeof(double) * d.Nh, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(t.h_isfixed, in->h_isfixed, d.Nh, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemsetAsync(t.dhdt, 0, sizeof(double) * d.Nh, c->st));
  wavi_stats acc{}, one{};
  for (int k = 0; k < nsteps; ++k) {
    TRY(set_params(c, &pp));
    TRY(step_pre(c, in->basal_melt_rate));
    TRY(solve_enqueue(c, &pp));
    TRY(solve_finish(c, &one));
    acc.picard_iterations += one.picard_iterations;
    acc.coarse_cg_iterations += one.coarse_cg_iterations;
    acc.op_applications += one.op_applications;
    acc.algorithmic_bytes += one.algorithmic_bytes;
    acc.elapsed_ms += one.elapsed_ms;
    acc.kernel_launches += one.kernel_launches;
    acc.host_syncs += one.host_syncs;
    acc.status = one.status;
    acc.rel_residual = one.rel_residual;
    acc.rel_update = one.rel_update;
    acc.coarse_solver = one.coarse_solver;
    TRY(step_post(c, in->basal_melt_rate, dt, p->minimum_thickness));
  }
  // the model state after the last step (update_state! overwrites these fields in the reference too)
  const cudaMemcpyKind dd = cudaMemcpyDeviceToDevice;
#define OUTD(dst, src, n) CK(cudaMemcpyAsync(const_cast<double*>(dst), src, sizeof(double) * (n), dd, c->st));
  OUTD(f->h, c->h, d.Nh) OUTD(f->s, c->s, d.Nh) OUTD(f->dsdh, c->dsdh, d.Nh) OUTD(f->grounded_fraction, c->gf, d.Nh)
  OUTD(f->weertman_c, c->wc, d.Nh) OUTD(f->accumulation, c->acc, d.Nh) OUTD(f->basal_melt, c->melt, d.Nh)
  OUTD(f->gu_h, c->h_uv, d.Nu) OUTD(f->gv_h, c->h_uv + d.Nu, d.Nv) OUTD(f->gu_s, c->s_uv, d.Nu) OUTD(f->gv_s, c->s_uv + d.Nu, d.Nv)
  OUTD(f->gu_grounded_fraction, c->gf_uv, d.Nu) OUTD(f->gv_grounded_fraction, c->gf_uv + d.Nu, d.Nv)
  OUTD(f->u, c->uv, d.Nu) OUTD(f->v, c->uv + d.Nu, d.Nv) OUTD(f->eta, c->eta, (size_t)d.Nh * d.ns)
  OUTD(f->beta, c->beta, d.Nh) OUTD(f->quad_f2, c->quad_f2, d.Nh) OUTD(f->shelf_strain_rate, c->shelf, d.Nh)
  OUTD(f->av_speed, c->av_speed, d.Nh) OUTD(f->bed_speed, c->bed_speed, d.Nh) OUTD(f->tau_bed, c->tau, d.Nh)
  OUTD(f->eta_av, c->eta_av, d.Nh) OUTD(f->quad_f1, c->quad_f1, d.Nh) OUTD(f->beta_eff, c->beta_eff, d.Nh)
  OUTD(f->gu_beta_eff, c->beta_eff_uv, d.Nu) OUTD(f->gv_beta_eff, c->beta_eff_uv + d.Nu, d.Nv)
  OUTD(f->gu_residual, c->resid_uv, d.Nu) OUTD(f->gv_residual, c->resid_uv + d.Nu, d.Nv)
  if (out) {
    if (out->dhdt) OUTD(out->dhdt, t.dhdt, d.Nh)
    if (out->u_h) OUTD(out->u_h, t.uh, d.Nh)
    if (out->v_h) OUTD(out->v_h, t.vh, d.Nh)
    if (out->u_bed) OUTD(out->u_bed, t.ub, d.Nh)
    if (out->v_bed) OUTD(out->v_bed, t.vb, d.Nh)
    if (out->u_surf) OUTD(out->u_surf, t.us, d.Nh)
    if (out->v_surf) OUTD(out->v_surf, t.vs, d.Nh)
  }
#undef OUTD
  CK(cudaMemcpyAsync(const_cast<uint8_t*>(f->wu_mask), c->wmask_uv, d.Nu, dd, c->st));
  CK(cudaMemcpyAsync(const_cast<uint8_t*>(f->wv_mask), c->wmask_uv + d.Nu, d.Nv, dd, c->st));
  std::vector<uint8_t> wm((size_t)d.N);
  CK(cudaMemcpyAsync(wm.data(), c->wmask_uv, d.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (out) {
    out->n_wu = out->n_wv = 0;
    for (int i = 0; i < d.Nu; ++i) out->n_wu += wm[i] != 0;
    for (int i = d.Nu; i < d.N; ++i) out->n_wv += wm[i] != 0;
    out->steps = nsteps;
  }
  c->solved = false;  // the state moved on after the last solve; the adjoint needs a fresh solve
  if (st) *st = acc;
  return 0;
}

int wavi_haar_device(wavi_ctx* c, int kind, const double* in_uv, double* out_uv, const uint8_t* mask_uv) {
  TRY(check_ctx(c));
  if (!in_uv || !out_uv) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  const Dims& d = c->d;
  const int L = c->sp.levels;
  if (kind == 0)
    k_haar<double, double, 0, false, false><<<c->haar_grid, c->haar_block, 0, c->st>>>(
        d, L, in_uv, out_uv, mask_uv ? mask_uv : c->inner_uv, nullptr, nullptr, c->partials, nullptr);
  else if (kind == 1)
    k_haar<double, double, 1, false, false><<<c->haar_grid, c->haar_block, 0, c->st>>>(
        d, L, in_uv, out_uv, mask_uv ? mask_uv : c->wmask_uv, nullptr, nullptr, c->partials, nullptr);
  else if (kind == 2)
    k_haar<double, double, 2, false, false><<<c->haar_grid, c->haar_block, 0, c->st>>>(
        d, L, in_uv, out_uv, nullptr, mask_uv ? mask_uv : c->mask_uv, nullptr, c->partials, nullptr);
  else
    return fail(c, WAVI_ERR_ARGUMENT, "unknown transform %d", kind);
  CKL();
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

// update_wavelets! (Wavelets/update_wavelets.jl:6-32) with the device time stepping's own kernels: the
// forward Haar transform of the u/v model masks times the given velocities, the threshold, and the
// cleared coarse-correction cache, on this context; the new wavelet mask is copied to wmask_out.
int wavi_update_wavelets_device(wavi_ctx* c, const double* uv_in, uint8_t* wmask_out) {
  TRY(check_ctx(c));
  if (!uv_in || !wmask_out) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  TRY(step_alloc(c));
  const Dims& d = c->d;
  CK(cudaMemcpyAsync(c->uv, uv_in, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, c->st));
  TRY(step_wavelets(c));
  CK(cudaMemcpyAsync(wmask_out, c->wmask_uv, d.N, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}


// ---------------------------------------------------------------------------------------------
// Ensembles: independent domains solved concurrently, one context (stream, graph) per member
// ---------------------------------------------------------------------------------------------
}  // extern "C"

struct wavi_ensemble {
  std::vector<wavi_ctx*> m;
  std::vector<cudaEvent_t> done;
  int concurrency = 1;
  std::string err;
};

namespace {
int ens_fail(wavi_ensemble* e, int code, const std::string& msg) {
  e->err = msg;
  return code;
}
}  // namespace

extern "C" {

int wavi_ensemble_create(int n, const wavi_grid_desc* grids, const wavi_solver_params* sps, const wavi_options* opt,
                         int concurrency, wavi_ensemble** out) {
  if (!out) return fail(nullptr, WAVI_ERR_ARGUMENT, "out is null");
  *out = nullptr;
  if (n < 1 || !grids || !sps || !opt) return fail(nullptr, WAVI_ERR_ARGUMENT, "bad ensemble arguments");
  if (!opt->use_graphs) return fail(nullptr, WAVI_ERR_ARGUMENT, "ensemble members run as CUDA graphs (use_graphs = 1)");
  auto* e = new wavi_ensemble();
  e->concurrency = std::max(1, std::min(concurrency, n));
  for (int k = 0; k < n; ++k) {
    wavi_ctx* c = nullptr;
    const int r = create_ctx(&grids[k], &sps[k], opt, e->concurrency, &c);
    cudaEvent_t ev = nullptr;
    if (r == 0 && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      wavi_ctx_destroy(c);
      c = nullptr;
    }
    if (!c) {
      const std::string msg = "member " + std::to_string(k) + ": " + (r ? g_create_error : std::string("event creation failed"));
      wavi_ensemble_destroy(e);
      return fail(nullptr, r ? r : WAVI_ERR_CUDA, "%s", msg.c_str());
    }
    e->m.push_back(c);
    e->done.push_back(ev);
  }
  *out = e;
  return WAVI_OK;
}

int wavi_ensemble_destroy(wavi_ensemble* e) {
  if (!e) return WAVI_OK;
  for (wavi_ctx* c : e->m) wavi_ctx_destroy(c);
  for (cudaEvent_t ev : e->done)
    if (ev) cudaEventDestroy(ev);
  delete e;
  return WAVI_OK;
}

const char* wavi_ensemble_last_error(const wavi_ensemble* e) { return e ? e->err.c_str() : g_create_error.c_str(); }

int wavi_ensemble_solve_device(wavi_ensemble* e, const wavi_params* params, wavi_fields* fields, wavi_stats* stats) {
  if (!e || !params || !fields) return WAVI_ERR_ARGUMENT;
  const int n = (int)e->m.size(), S = e->concurrency;
  int err = 0, err_k = -1;
  int issued = 0;
  // largest members first (longest-processing-time order), so that big domains do not form the tail
  std::vector<int> order(n);
  for (int k = 0; k < n; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return e->m[a]->d.N > e->m[b]->d.N; });
  for (int o = 0; o < n && !err; ++o) {
    const int k = order[o];
    wavi_ctx* c = e->m[k];
    int r = check_ctx(c);
    if (!r) r = check_params(c, &params[k]);
    // at most S members in flight: the o-th member starts after the (o - S)-th has finished
    if (!r && o >= S && cudaStreamWaitEvent(c->st, e->done[order[o - S]], 0) != cudaSuccess)
      r = fail(c, WAVI_ERR_CUDA, "stream wait");
    if (!r) r = upload(c, &fields[k], false);
    if (!r) r = solve_enqueue(c, &params[k]);
    if (!r) r = download(c, &fields[k], false);
    if (!r && cudaEventRecord(e->done[k], c->st) != cudaSuccess) r = fail(c, WAVI_ERR_CUDA, "event record");
    if (r) {
      err = r;
      err_k = k;
    } else {
      issued = o + 1;
    }
  }
  for (int o = 0; o < issued; ++o) {
    const int k = order[o];
    const int r = solve_finish(e->m[k], stats ? &stats[k] : nullptr);
    if (r && !err) {
      err = r;
      err_k = k;
    }
  }
  if (err) return ens_fail(e, err, "member " + std::to_string(err_k) + ": " + e->m[err_k]->err);
  return WAVI_OK;
}

}  // extern "C"
