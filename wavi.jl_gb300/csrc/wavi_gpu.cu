// wavi_gpu.cu — libwavi_gpu.so: context, buffers, the Picard loop and the C ABI of include/wavi_gpu.h.
//
// The solve is update_velocities! (src/Models/update_velocities.jl:11-29): per Picard iteration one
// relinearisation (inner_update!, :32-45), the float64 residual and convergence test (:50-65), and one
// wavelet-multigrid V-cycle (Wavelets/update_preconditioners.jl:54-83) whose coarse CG runs with its
// scalars on the device.  Everything stays on the context's stream; the host only reads the Picard
// convergence scalars and, every CG_BATCH coarse iterations, the CG termination flag.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wavi_gpu.h"
#include "kernels.cuh"

using namespace wavi;

namespace {

constexpr int EW_THREADS = 256;
constexpr int CG_BATCH = 8;

}  // namespace

struct wavi_ctx {
  int dev = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Dims d{};
  wavi_solver_params sp{};
  wavi_options opt{};
  bool has_fixed = false;
  std::string err;
  std::vector<void*> allocs;
  // static masks (device)
  uint8_t *h_mask = nullptr, *c_mask = nullptr, *mask_uv = nullptr, *inner_uv = nullptr, *fixed_uv = nullptr;
  uint8_t* wmask_uv = nullptr;
  std::vector<uint8_t> h_inner_host, h_mask_uv_host;  // host copies for masked downloads
  // inputs
  double *h = nullptr, *s = nullptr, *dsdh = nullptr, *gf = nullptr, *wc = nullptr, *acc = nullptr, *melt = nullptr;
  double *h_uv = nullptr, *s_uv = nullptr, *gf_uv = nullptr, *glen_b = nullptr;
  double *zeta = nullptr, *qw = nullptr;
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
  double *x64 = nullptr, *b64 = nullptr, *r64 = nullptr, *t64 = nullptr, *xfix64 = nullptr;
  // V-cycle vectors (float or double; sized for double)
  void *rs = nullptr, *rsm = nullptr, *corr = nullptr, *diag = nullptr, *xc = nullptr, *rc = nullptr, *uc = nullptr,
       *cc = nullptr, *w = nullptr, *y = nullptr, *bc = nullptr;
  // reductions
  double* partials = nullptr;
  int max_partials = 0;
  double* S = nullptr;
  int* I = nullptr;
  double* h_S = nullptr;  // pinned
  int* h_I = nullptr;     // pinned
  // launch shapes
  dim3 op_grid, op_block, pt_grid, pt_block, haar_grid, haar_block;
  int ew_blocks = 0;
  // statistics of the current solve
  int op_apps = 0;
  double alg_bytes = 0.0;
  long launches = 0;
  int host_syncs = 0;
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

// Algorithmic bytes of one operator application: read x, write y, coefficients heta_h, dimp (Nh),
// heta_c (Nc), beta_m, h_m (N), interior mask (N bytes), b for the residual form.
double op_bytes(const Dims& d, int w, bool resid) {
  return (double)w * (2.0 * d.N + 2.0 * d.Nh + d.Nc + 2.0 * d.N + (resid ? d.N : 0)) + d.N;
}

template <typename T>
int launch_op(wavi_ctx* c, const T* x, const T* b, T* y, bool resid, const int* skip = nullptr) {
  if (resid)
    k_op<T, T, 1><<<c->op_grid, c->op_block, 0, c->st>>>(c->d, coef<T>(c), x, b, y, c->partials, skip);
  else
    k_op<T, T, 0><<<c->op_grid, c->op_block, 0, c->st>>>(c->d, coef<T>(c), x, b, y, c->partials, skip);
  CKL();
  c->op_apps++;
  c->alg_bytes += op_bytes(c->d, (int)sizeof(T), resid);
  return 0;
}
int op_partials(const wavi_ctx* c) { return (int)(c->op_grid.x * c->op_grid.y); }
int haar_partials(const wavi_ctx* c) { return (int)(c->haar_grid.x * c->haar_grid.y * c->haar_grid.z); }

template <typename TI, typename TO, int KIND, bool ACC, bool DOT>
int launch_haar(wavi_ctx* c, const TI* in, TO* out, const uint8_t* outmask, const uint8_t* inmask, const TO* dotv,
                const int* skip) {
  k_haar<TI, TO, KIND, ACC, DOT><<<c->haar_grid, c->haar_block, 0, c->st>>>(c->d, c->sp.levels, in, out, outmask, inmask,
                                                                             dotv, c->partials, skip);
  CKL();
  c->alg_bytes += (double)(sizeof(TI) + sizeof(TO) * (ACC ? 2 : 1) + (DOT ? sizeof(TO) : 0)) * c->d.N + c->d.N;
  return 0;
}

int reduce_to(wavi_ctx* c, int np, double* out) {
  k_reduce<<<1, 1024, 0, c->st>>>(c->partials, np, out);
  CKL();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// One V-cycle (precondition!(x, p, b), update_preconditioners.jl:54-83) on the T vectors:
// corr = V(rs), with the coarse iterate xc warm-started from its current contents.
// ---------------------------------------------------------------------------------------------
template <typename T>
int vcycle(wavi_ctx* c, int* cg_iters) {
  const Dims& d = c->d;
  const int N = d.N;
  T* rs = (T*)c->rs;
  T* rsm = (T*)c->rsm;
  T* corr = (T*)c->corr;
  T* diag = (T*)c->diag;
  T* xc = (T*)c->xc;
  T* rc = (T*)c->rc;
  T* uc = (T*)c->uc;
  T* cvec = (T*)c->cc;
  T* w = (T*)c->w;
  T* y = (T*)c->y;
  T* bc = (T*)c->bc;
  const T omega = (T)c->sp.smoother_omega;
  int rc_;
  k_op_diag<T><<<c->pt_grid, c->pt_block, 0, c->st>>>(d, coef<T>(c), diag);
  CKL();
  k_fill<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(N, corr, (T)0);
  CKL();
  // smoother residual starts as rs - A*0 = rs
  CK(cudaMemcpyAsync(rsm, rs, sizeof(T) * N, cudaMemcpyDeviceToDevice, c->st));
  static const int fwd[4] = {1, 3, 2, 4}, bwd[4] = {4, 2, 3, 1};
  auto smooth = [&](const int* order) -> int {
    for (int it = 0; it < c->sp.nsmooth; ++it)
      for (int oc = 0; oc < 4; ++oc) {
        k_colour_update<T><<<c->pt_grid, c->pt_block, 0, c->st>>>(d, order[oc], omega, c->inner_uv, rsm, diag, corr);
        CKL();
        int r = launch_op<T>(c, corr, rs, rsm, true);
        if (r) return r;
      }
    return 0;
  };
  if ((rc_ = smooth(fwd))) return rc_;
  // b_coarse = R r;  abstol = tol_coarse |b_coarse|
  if ((rc_ = launch_haar<T, T, 1, false, true>(c, rsm, bc, c->wmask_uv, nullptr, bc, nullptr))) return rc_;
  if ((rc_ = reduce_to(c, haar_partials(c), c->S + CG_SUM))) return rc_;
  // r_c = b_c - R A P xc
  if ((rc_ = launch_haar<T, T, 0, false, false>(c, xc, w, c->inner_uv, nullptr, nullptr, nullptr))) return rc_;
  if ((rc_ = launch_op<T>(c, w, nullptr, y, false))) return rc_;
  if ((rc_ = launch_haar<T, T, 1, false, false>(c, y, cvec, c->wmask_uv, nullptr, nullptr, nullptr))) return rc_;
  k_cg_start_sub<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(N, bc, cvec, rc, uc, c->partials);
  CKL();
  // |b_c| from the reduced sum, then the CG scalars
  k_sqrt_slot<<<1, 1, 0, c->st>>>(c->S + CG_SUM, c->S + CG_BNORM);
  CKL();
  k_cg_start_scalars<<<1, 1024, 0, c->st>>>(c->partials, c->ew_blocks, c->sp.tol_coarse, c->sp.maxiter_coarse, c->S, c->I);
  CKL();
  const int* done = c->I + CG_DONE;
  for (;;) {
    for (int k = 0; k < CG_BATCH; ++k) {
      k_cg_dir<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(N, c->S, c->I, rc, uc);
      CKL();
      if ((rc_ = launch_haar<T, T, 0, false, false>(c, uc, w, c->inner_uv, nullptr, nullptr, done))) return rc_;
      if ((rc_ = launch_op<T>(c, w, nullptr, y, false, done))) return rc_;
      if ((rc_ = launch_haar<T, T, 1, false, true>(c, y, cvec, c->wmask_uv, nullptr, uc, done))) return rc_;
      k_cg_alpha<<<1, 1024, 0, c->st>>>(c->partials, haar_partials(c), c->S, c->I);
      CKL();
      k_cg_axpy<T><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(N, c->S, c->I, uc, cvec, xc, rc, c->partials);
      CKL();
      k_cg_res<<<1, 1024, 0, c->st>>>(c->partials, c->ew_blocks, c->S, c->I);
      CKL();
    }
    CK(cudaMemcpyAsync(c->h_I, c->I, sizeof(int) * I_COUNT, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->host_syncs++;
    if (c->h_I[CG_DONE]) break;
  }
  *cg_iters = c->h_I[CG_IT];
  // corr += P xc
  if ((rc_ = launch_haar<T, T, 0, true, false>(c, xc, corr, c->inner_uv, nullptr, nullptr, nullptr))) return rc_;
  // post-smoother starts from rs - A corr
  if ((rc_ = launch_op<T>(c, corr, rs, rsm, true))) return rc_;
  if ((rc_ = smooth(bwd))) return rc_;
  return 0;
}

int relinearise(wavi_ctx* c, const wavi_params* P) {
  const Dims& d = c->d;
  RelinIn in{c->uv, c->mask_uv, c->h_mask, c->c_mask, c->h, c->wc, c->glen_b, c->dsdh, c->zeta, c->qw,
             P->weertman_m, P->weertman_reg_speed, P->glen_n, P->glen_reg_strain_rate,
             -P->density_ice * P->g * c->sp.super_implicitness * P->dt, c->sp.n_iter_viscosity};
  RelinOut out{c->shelf, c->av_speed, c->bed_speed, c->beta, c->tau, c->eta, c->eta_av, c->quad_f1, c->quad_f2,
               c->beta_eff, c->heta_h64, c->dimp64, mixed(c) ? c->heta_h32 : nullptr, mixed(c) ? c->dimp32 : nullptr,
               c->hn};
  const int nb = (d.Nh + 127) / 128;
  if (mixed(c))
    k_relin_h<float><<<nb, 128, 0, c->st>>>(d, in, out);
  else
    k_relin_h<double><<<nb, 128, 0, c->st>>>(d, in, out);
  CKL();
  RelinUVIn uin{c->mask_uv, c->h_mask, c->c_mask, c->beta_eff, c->gf, c->gf_uv, c->h_uv, c->hn};
  RelinUVOut uout{c->beta_eff_uv, c->beta_m64, c->h_m64, c->heta_c64, mixed(c) ? c->beta_m32 : nullptr,
                  mixed(c) ? c->h_m32 : nullptr, mixed(c) ? c->heta_c32 : nullptr};
  k_relin_uv<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, uin, uout);
  CKL();
  c->alg_bytes += 8.0 * (2.0 * d.Nh * d.ns + 22.0 * d.Nh + 8.0 * d.N) + 4.0 * d.N;
  return 0;
}

// Build b (get_rhs incl. the Dirichlet lift), x (start guess), r = b - A x and ||r||^2, ||b||^2.
int picard_residual(wavi_ctx* c, const wavi_params* P) {
  const Dims& d = c->d;
  RhsIn in{c->h_mask, c->inner_uv, c->fixed_uv, c->s, c->dsdh, c->acc, c->melt, c->h_uv, c->s_uv, c->uv,
           P->density_ice, P->density_ocean, P->g, P->sea_level_wrt_geoid, c->sp.super_implicitness * P->dt};
  k_rhs<<<c->pt_grid, c->pt_block, 0, c->st>>>(d, in, c->b64, c->x64, c->xfix64);
  CKL();
  int r;
  if (c->has_fixed) {
    if ((r = launch_op<double>(c, c->xfix64, nullptr, c->t64, false))) return r;
    k_sub<double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->b64, c->t64, c->b64);
    CKL();
  }
  if ((r = launch_op<double>(c, c->x64, c->b64, c->r64, true))) return r;
  if ((r = reduce_to(c, op_partials(c), c->S + S_RR))) return r;
  k_dot<double, double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->b64, c->b64, c->partials);
  CKL();
  if ((r = reduce_to(c, c->ew_blocks, c->S + S_BB))) return r;
  return 0;
}

int solve_resident(wavi_ctx* c, const wavi_params* P, wavi_stats* st) {
  const Dims& d = c->d;
  c->op_apps = 0;
  c->alg_bytes = 0.0;
  c->launches = 0;
  c->host_syncs = 0;
  int total_cg = 0, it = 0, r;
  bool converged = false;
  double rel = INFINITY, relu = INFINITY;
  CK(cudaEventRecord(c->ev0, c->st));
  while (!converged && it < c->sp.maxiter_picard) {
    ++it;
    if ((r = relinearise(c, P))) return r;
    if ((r = picard_residual(c, P))) return r;
    CK(cudaMemcpyAsync(c->h_S, c->S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->host_syncs++;
    rel = std::sqrt(c->h_S[S_RR]) / std::sqrt(c->h_S[S_BB]);
    if (!std::isfinite(rel)) return fail(c, WAVI_ERR_NONFINITE, "non-finite Picard residual at iteration %d", it);
    CK(cudaMemcpyAsync(c->resid_uv, c->r64, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, c->st));
    converged = rel < c->sp.tol_picard;
    if (converged && c->opt.picard_test == 1 && it > 1 && !(relu <= c->sp.tol_picard)) converged = false;
    if (converged) break;
    int cg = 0;
    if (mixed(c)) {
      k_convert<double, float><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->r64, (float*)c->rs);
      CKL();
      k_convert<double, float><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->xc_full64, (float*)c->xc);
      CKL();
      if ((r = vcycle<float>(c, &cg))) return r;
      k_convert<float, double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, (float*)c->xc, c->xc_full64);
      CKL();
      k_update_norms<float><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, (float*)c->corr, c->x64, c->partials);
      CKL();
      k_apply_correction<float><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, (float*)c->corr, c->x64, c->uv);
      CKL();
    } else {
      CK(cudaMemcpyAsync(c->rs, c->r64, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, c->st));
      CK(cudaMemcpyAsync(c->xc, c->xc_full64, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, c->st));
      if ((r = vcycle<double>(c, &cg))) return r;
      CK(cudaMemcpyAsync(c->xc_full64, c->xc, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, c->st));
      k_update_norms<double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, (double*)c->corr, c->x64, c->partials);
      CKL();
      k_apply_correction<double><<<c->ew_blocks, EW_THREADS, 0, c->st>>>(d.N, c->inner_uv, (double*)c->corr, c->x64, c->uv);
      CKL();
    }
    k_reduce<<<1, 1024, 0, c->st>>>(c->partials, c->ew_blocks, c->S + S_DU);
    CKL();
    k_reduce<<<1, 1024, 0, c->st>>>(c->partials + c->ew_blocks, c->ew_blocks, c->S + S_UU);
    CKL();
    CK(cudaMemcpyAsync(c->h_S, c->S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->host_syncs++;
    relu = std::sqrt(c->h_S[S_DU]) / std::sqrt(c->h_S[S_UU]);
    total_cg += cg;
  }
  CK(cudaEventRecord(c->ev1, c->st));
  CK(cudaStreamSynchronize(c->st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  int status = converged ? WAVI_OK : WAVI_ERR_NOT_CONVERGED;
  if (st) {
    st->status = status;
    st->picard_iterations = it;
    st->coarse_cg_iterations = total_cg;
    st->op_applications = c->op_apps;
    st->rel_residual = rel;
    st->rel_update = relu;
    st->algorithmic_bytes = c->alg_bytes;
    st->elapsed_ms = ms;
    st->kernel_launches = (int32_t)std::min<long>(c->launches, 2147483647L);
    st->host_syncs = c->host_syncs;
  }
  return 0;  // not converging is reported through stats.status only, like the reference's silent stop
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

int upload(wavi_ctx* c, const wavi_fields* f, bool host) {
  const Dims& d = c->d;
  const cudaMemcpyKind k = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  int r;
#define IN(dst, src, n) \
  if ((r = copy_in(c, dst, src, n, k, #src))) return r;
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
#undef IN
  // adaptive coarse space and its compact correction cache -> full layout
  if (!f->wu_mask || !f->wv_mask || !f->wu_correction_coarse || !f->wv_correction_coarse)
    return fail(c, WAVI_ERR_ARGUMENT, "wavelet masks / coarse corrections are null");
  std::vector<uint8_t> wm((size_t)d.N);
  CK(cudaMemcpyAsync(wm.data(), f->wu_mask, d.Nu, host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(wm.data() + d.Nu, f->wv_mask, d.Nv, host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  size_t nwu = 0, nwv = 0;
  for (int i = 0; i < d.Nu; ++i) nwu += (wm[i] = wm[i] ? 1 : 0);
  for (int i = d.Nu; i < d.N; ++i) nwv += (wm[i] = wm[i] ? 1 : 0);
  std::vector<double> cu(nwu), cv(nwv), full((size_t)d.N, 0.0);
  CK(cudaMemcpyAsync(cu.data(), f->wu_correction_coarse, nwu * sizeof(double), host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(cv.data(), f->wv_correction_coarse, nwv * sizeof(double), host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  size_t a = 0, b = 0;
  for (int i = 0; i < d.Nu; ++i)
    if (wm[i]) full[i] = cu[a++];
  for (int i = d.Nu; i < d.N; ++i)
    if (wm[i]) full[i] = cv[b++];
  CK(cudaMemcpyAsync(c->wmask_uv, wm.data(), d.N, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->xc_full64, full.data(), sizeof(double) * d.N, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int download(wavi_ctx* c, wavi_fields* f, bool host) {
  const Dims& d = c->d;
  const cudaMemcpyKind k = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  int r;
#define OUT(dst, src, n) \
  if ((r = copy_out(c, dst, src, n, k, #dst))) return r;
  OUT(f->u, c->uv, d.Nu) OUT(f->v, c->uv + d.Nu, d.Nv) OUT(f->eta, c->eta, (size_t)d.Nh * d.ns)
  OUT(f->beta, c->beta, d.Nh) OUT(f->quad_f2, c->quad_f2, d.Nh)
  OUT(f->shelf_strain_rate, c->shelf, d.Nh) OUT(f->av_speed, c->av_speed, d.Nh) OUT(f->bed_speed, c->bed_speed, d.Nh)
  OUT(f->tau_bed, c->tau, d.Nh) OUT(f->eta_av, c->eta_av, d.Nh) OUT(f->quad_f1, c->quad_f1, d.Nh)
  OUT(f->beta_eff, c->beta_eff, d.Nh)
  OUT(f->gu_beta_eff, c->beta_eff_uv, d.Nu) OUT(f->gv_beta_eff, c->beta_eff_uv + d.Nu, d.Nv)
#undef OUT
  // residual: written at the interior points only (set_residual!, update_velocities.jl:428-433)
  if (!f->gu_residual || !f->gv_residual) return fail(c, WAVI_ERR_ARGUMENT, "residual outputs are null");
  std::vector<double> res((size_t)d.N), gu((size_t)d.Nu), gv((size_t)d.Nv);
  CK(cudaMemcpyAsync(res.data(), c->resid_uv, sizeof(double) * d.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(gu.data(), f->gu_residual, sizeof(double) * d.Nu, host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(gv.data(), f->gv_residual, sizeof(double) * d.Nv, host ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, c->st));
  // coarse correction cache: full -> compact in mask order
  std::vector<double> full((size_t)d.N);
  std::vector<uint8_t> wm((size_t)d.N);
  CK(cudaMemcpyAsync(full.data(), c->xc_full64, sizeof(double) * d.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(wm.data(), c->wmask_uv, d.N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int i = 0; i < d.Nu; ++i)
    if (c->h_inner_host[i]) gu[i] = res[i];
  for (int i = 0; i < d.Nv; ++i)
    if (c->h_inner_host[d.Nu + i]) gv[i] = res[d.Nu + i];
  std::vector<double> cu, cv;
  for (int i = 0; i < d.Nu; ++i)
    if (wm[i]) cu.push_back(full[i]);
  for (int i = d.Nu; i < d.N; ++i)
    if (wm[i]) cv.push_back(full[i]);
  const cudaMemcpyKind hk = host ? cudaMemcpyHostToHost : cudaMemcpyHostToDevice;
  CK(cudaMemcpyAsync(f->gu_residual, gu.data(), sizeof(double) * d.Nu, hk, c->st));
  CK(cudaMemcpyAsync(f->gv_residual, gv.data(), sizeof(double) * d.Nv, hk, c->st));
  if (!cu.empty()) CK(cudaMemcpyAsync(f->wu_correction_coarse, cu.data(), sizeof(double) * cu.size(), hk, c->st));
  if (!cv.empty()) CK(cudaMemcpyAsync(f->wv_correction_coarse, cv.data(), sizeof(double) * cv.size(), hk, c->st));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int check_ctx(wavi_ctx* c) {
  if (!c) return WAVI_ERR_ARGUMENT;
  cudaError_t e = cudaSetDevice(c->dev);
  if (e != cudaSuccess) return fail(c, WAVI_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  return 0;
}

}  // namespace

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

int wavi_ctx_create(const wavi_grid_desc* g, const wavi_solver_params* sp, const wavi_options* opt, wavi_ctx** out) {
  wavi_ctx* c = nullptr;
  if (!out) return fail(nullptr, WAVI_ERR_ARGUMENT, "out is null");
  *out = nullptr;
  if (!g || !sp || !opt) return fail(nullptr, WAVI_ERR_ARGUMENT, "null argument");
  if (g->nx < 2 || g->ny < 2 || g->nsigma < 2) return fail(nullptr, WAVI_ERR_ARGUMENT, "nx, ny, nsigma must be > 1");
  if (!g->sigma || !g->quadrature_weights || !g->h_mask || !g->u_iszero || !g->v_iszero || !g->u_isfixed || !g->v_isfixed)
    return fail(nullptr, WAVI_ERR_ARGUMENT, "grid arrays must not be null");
  if (sp->levels < 0 || sp->levels > 4) return fail(nullptr, WAVI_ERR_ARGUMENT, "levels must be in 0..4 (got %d)", sp->levels);
  if (sp->n_iter_viscosity < 1) return fail(nullptr, WAVI_ERR_ARGUMENT, "n_iter_viscosity must be >= 1");
  if (opt->precision != WAVI_PRECISION_FP64 && opt->precision != WAVI_PRECISION_MIXED)
    return fail(nullptr, WAVI_ERR_ARGUMENT, "unknown precision %d", opt->precision);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(nullptr, WAVI_ERR_NO_DEVICE, "no CUDA device");
  if (opt->device < 0 || opt->device >= ndev) return fail(nullptr, WAVI_ERR_ARGUMENT, "device %d out of range", opt->device);
  if ((long)(g->nx + 1) * (g->ny + 1) > (1L << 30)) return fail(nullptr, WAVI_ERR_ARGUMENT, "grid too large");
  c = new wavi_ctx();
  c->dev = opt->device;
  c->sp = *sp;
  c->opt = *opt;
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
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(c, WAVI_ERR_CUDA, "stream creation failed"));
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
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
  c->h_mask_uv_host = mk;
  int r = 0;
  const size_t Nh = d.Nh, Nc = d.Nc, N = d.N, N3 = (size_t)d.Nh * d.ns;
#define A(p, n) \
  if ((r = dalloc(c, &c->p, n))) return bail(r);
  A(h_mask, Nh) A(c_mask, Nc) A(mask_uv, N) A(inner_uv, N) A(fixed_uv, N) A(wmask_uv, N)
  A(h, Nh) A(s, Nh) A(dsdh, Nh) A(gf, Nh) A(wc, Nh) A(acc, Nh) A(melt, Nh)
  A(h_uv, N) A(s_uv, N) A(gf_uv, N) A(glen_b, N3) A(zeta, (size_t)d.ns) A(qw, (size_t)d.ns)
  A(uv, N) A(eta, N3) A(beta, Nh) A(quad_f2, Nh) A(xc_full64, N)
  A(shelf, Nh) A(av_speed, Nh) A(bed_speed, Nh) A(tau, Nh) A(eta_av, Nh) A(quad_f1, Nh) A(beta_eff, Nh)
  A(beta_eff_uv, N) A(resid_uv, N) A(hn, Nh)
  A(heta_h64, Nh) A(heta_c64, Nc) A(dimp64, Nh) A(beta_m64, N) A(h_m64, N)
  A(heta_h32, Nh) A(heta_c32, Nc) A(dimp32, Nh) A(beta_m32, N) A(h_m32, N)
  A(x64, N) A(b64, N) A(r64, N) A(t64, N) A(xfix64, N)
#undef A
  for (void** p : {&c->rs, &c->rsm, &c->corr, &c->diag, &c->xc, &c->rc, &c->uc, &c->cc, &c->w, &c->y, &c->bc}) {
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
  c->ew_blocks = (int)std::min<size_t>((N + EW_THREADS - 1) / EW_THREADS, 152 * 8);
  c->max_partials = std::max({op_partials(c), haar_partials(c), 2 * c->ew_blocks, 1});
  if ((r = dalloc(c, &c->partials, (size_t)c->max_partials))) return bail(r);
  if ((r = dalloc(c, &c->S, (size_t)S_COUNT))) return bail(r);
  if ((r = dalloc(c, &c->I, (size_t)I_COUNT))) return bail(r);
  if (cudaMallocHost(&c->h_S, sizeof(double) * S_COUNT) != cudaSuccess ||
      cudaMallocHost(&c->h_I, sizeof(int) * I_COUNT) != cudaSuccess)
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
  if (e != cudaSuccess) return bail(fail(c, WAVI_ERR_CUDA, "mask upload: %s", cudaGetErrorString(e)));
  *out = c;
  return WAVI_OK;
}

int wavi_ctx_destroy(wavi_ctx* c) {
  if (!c) return WAVI_OK;
  cudaSetDevice(c->dev);
  if (c->st) cudaStreamSynchronize(c->st);
  for (void* p : c->allocs) cudaFree(p);
  if (c->h_S) cudaFreeHost(c->h_S);
  if (c->h_I) cudaFreeHost(c->h_I);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return WAVI_OK;
}

static int check_params(wavi_ctx* c, const wavi_params* p) {
  if (!p) return fail(c, WAVI_ERR_ARGUMENT, "params is null");
  if (!(p->glen_n > 0) || !(p->weertman_m > 0)) return fail(c, WAVI_ERR_ARGUMENT, "glen_n and weertman_m must be positive");
  return 0;
}

int wavi_solve_velocities(wavi_ctx* c, const wavi_params* p, wavi_fields* f, wavi_stats* st) {
  int r;
  if ((r = check_ctx(c))) return r;
  if ((r = check_params(c, p))) return r;
  if (!f) return fail(c, WAVI_ERR_ARGUMENT, "fields is null");
  if ((r = upload(c, f, true))) return r;
  if ((r = solve_resident(c, p, st))) return r;
  return download(c, f, true);
}

int wavi_solve_velocities_device(wavi_ctx* c, const wavi_params* p, wavi_fields* f, wavi_stats* st) {
  int r;
  if ((r = check_ctx(c))) return r;
  if ((r = check_params(c, p))) return r;
  if (!f) return fail(c, WAVI_ERR_ARGUMENT, "fields is null");
  if ((r = upload(c, f, false))) return r;
  if ((r = solve_resident(c, p, st))) return r;
  return download(c, f, false);
}

int wavi_relinearise_device(wavi_ctx* c, const wavi_params* p, wavi_fields* f) {
  int r;
  if ((r = check_ctx(c))) return r;
  if ((r = check_params(c, p))) return r;
  if (!f) return fail(c, WAVI_ERR_ARGUMENT, "fields is null");
  if ((r = upload(c, f, false))) return r;
  if ((r = relinearise(c, p))) return r;
  CK(cudaStreamSynchronize(c->st));
  return download(c, f, false);
}

int wavi_apply_operator_device(wavi_ctx* c, int precision, const void* in_uv, void* out_uv) {
  int r;
  if ((r = check_ctx(c))) return r;
  if (!in_uv || !out_uv) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  if (precision == WAVI_PRECISION_FP64)
    r = launch_op<double>(c, (const double*)in_uv, nullptr, (double*)out_uv, false);
  else if (precision == WAVI_PRECISION_MIXED && mixed(c))
    r = launch_op<float>(c, (const float*)in_uv, nullptr, (float*)out_uv, false);
  else
    return fail(c, WAVI_ERR_ARGUMENT, "float32 operator needs a mixed-precision context");
  if (r) return r;
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int wavi_op_diagonal_device(wavi_ctx* c, int precision, void* diag_uv) {
  int r;
  if ((r = check_ctx(c))) return r;
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

int wavi_haar_device(wavi_ctx* c, int kind, const double* in_uv, double* out_uv, const uint8_t* mask_uv) {
  int r;
  if ((r = check_ctx(c))) return r;
  if (!in_uv || !out_uv) return fail(c, WAVI_ERR_ARGUMENT, "null vector");
  if (kind == 0)
    r = launch_haar<double, double, 0, false, false>(c, in_uv, out_uv, mask_uv ? mask_uv : c->inner_uv, nullptr, nullptr, nullptr);
  else if (kind == 1)
    r = launch_haar<double, double, 1, false, false>(c, in_uv, out_uv, mask_uv ? mask_uv : c->wmask_uv, nullptr, nullptr, nullptr);
  else if (kind == 2)
    r = launch_haar<double, double, 2, false, false>(c, in_uv, out_uv, nullptr, mask_uv ? mask_uv : c->mask_uv, nullptr, nullptr);
  else
    return fail(c, WAVI_ERR_ARGUMENT, "unknown transform %d", kind);
  if (r) return r;
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

}  // extern "C"
