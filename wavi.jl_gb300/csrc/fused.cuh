// fused.cuh — the fused, graph-resident kernels of the velocity solve.
//
// Every kernel here is launched inside one CUDA graph per solve (Picard WHILE node -> V-cycle IF node ->
// coarse-CG WHILE node).  Kernels that end a reduction use the last-block pattern: each block writes a
// partial, the last block to arrive sums all partials in a fixed order (deterministic) and publishes
// the scalar, and, where the scalar decides control flow, sets the enclosing conditional node.
//
// The operator is evaluated on shared-memory tiles: stage 1 loads the velocity region
// [i0-1, i0+TX] x [j0-1, j0+TY] (optionally transformed, e.g. by a Jacobi colour update), stage 2 the
// h-cell / c-point stresses of [i0-1, i0+TX) x [j0-1, j0+TY), stage 3 the divergences at the tile's
// own points.  A TILE x TILE tile with TILE a multiple of the Haar block 2^(levels+1) also holds whole
// Haar blocks of both velocity components, so the coarse-grid restriction follows in shared memory.
#pragma once
#include <algorithm>

#include "kernels.cuh"

namespace wavi {

// Anderson acceleration of the Picard loop (anderson.cuh): at most kAAMax columns; a pivot below kAAPivot
// of its diagonal entry drops that column and every older one.
constexpr int kAAMax = 5;
constexpr double kAAPivot = 1e-10;
struct AAState {
  int started, have_prev;  // the acceleration acts from this iteration on; f and g of the last are kept
  int cols, head;          // columns held; ring slot of the newest
  int used, steps;         // columns in the last step's gamma; accelerated steps in this solve
  int slot[kAAMax];        // ring slots of gamma[0..used), newest first
  double gamma[kAAMax];
  double gram[kAAMax][kAAMax];  // dF^T dF by ring slot
};

// Device-side solver state: scalars, counters and the flags that steer the conditional nodes.
struct DevState {
  double rr, bb, rel, rel_prev_update;   // Picard residual norms
  double du2, uu2, rel_update;
  double cg_res, cg_prev, cg_tol, cg_alpha, cg_bnorm;
  int picard_it, picard_continue, vcycle_needed, converged;
  int cg_it, cg_continue, cg_total, status;
  unsigned counter[8];                   // last-block counters, one per reduction site
  AAState aa;
};
enum { CNT_A = 0, CNT_B = 1, CNT_C = 2, CNT_D = 3, CNT_AA_STAGE = 4, CNT_AA_APPLY = 5 };

// Relative tolerance of a V-cycle's coarse CG (abstol = tolerance x |b_c|, update_preconditioners.jl:73).
// The reference's is tol_coarse.  With coarse_forcing (wavi_options.coarse_forcing; inexact Newton's forcing
// terms, Eisenstat & Walker 1996) it is max(tol_coarse, min(kForcingMax, kForcingRatio x rel)), rel the
// Picard iteration's relative residual: early, far from the fixed point, where the relinearisation
// rather than the linear solve limits the next iterate, the coarse CG stops sooner; from
// rel <= tol_coarse / kForcingRatio on it is the reference's.  Only in solves of more than one Picard
// iteration: with maxiter_picard = 1 (a time step's single V-cycle) no later iteration follows.
constexpr double kForcingRatio = 0.1, kForcingMax = 0.1;
__device__ __forceinline__ double coarse_tolerance(const DevParams* P, const DevState* st) {
  return P->coarse_forcing && P->maxiter_picard > 1 ? fmax(P->tol_coarse, fmin(kForcingMax, kForcingRatio * st->rel))
                                                    : P->tol_coarse;
}

struct CondHandles {
  cudaGraphConditionalHandle picard, vcycle, cg;
  int active;  // 0: launched outside a graph, do not touch the handles
};

__device__ __forceinline__ int flat_tid() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ __forceinline__ int flat_nthreads() { return blockDim.x * blockDim.y * blockDim.z; }
__device__ __forceinline__ int flat_bid() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ __forceinline__ int flat_nblocks() { return gridDim.x * gridDim.y * gridDim.z; }

__device__ __forceinline__ double block_sum_any(double v, double* sh) {
  const int t = flat_tid(), nt = flat_nthreads();
  const int lane = t & 31, wid = t >> 5, nw = (nt + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < nw ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;  // valid in thread 0
}

// Each block contributes (v0, v1); the last block to finish receives the two totals, summed over all
// blocks' partials in block order, in tot[0..1] (valid for every thread of that block) and returns
// true.  Other blocks return false.  Uses partials[0 .. 2*nblocks).
__device__ __forceinline__ bool last_block_sum2(double v0, double v1, double* __restrict__ partials,
                                                unsigned* counter, double tot[2]) {
  __shared__ double sh[32];
  __shared__ double stot[2];
  __shared__ int slast;
  const int t = flat_tid(), nb = flat_nblocks(), b = flat_bid();
  double s0 = block_sum_any(v0, sh);
  __syncthreads();
  double s1 = block_sum_any(v1, sh);
  if (t == 0) {
    partials[b] = s0;
    partials[nb + b] = s1;
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    slast = (prev == (unsigned)nb - 1u);
  }
  __syncthreads();
  if (!slast) return false;
  __threadfence();
  double a0 = 0.0, a1 = 0.0;
  for (int k = t; k < nb; k += flat_nthreads()) {
    a0 += __ldcg(partials + k);
    a1 += __ldcg(partials + nb + k);
  }
  a0 = block_sum_any(a0, sh);
  __syncthreads();
  a1 = block_sum_any(a1, sh);
  if (t == 0) {
    stot[0] = a0;
    stot[1] = a1;
    *counter = 0u;
  }
  __syncthreads();
  tot[0] = stot[0];
  tot[1] = stot[1];
  return true;
}

// ------------------------------------------------------------------------------------------------
// Staged operator tile
// ------------------------------------------------------------------------------------------------
template <typename T, int TX, int TY>
struct OpTile {
  T xu[TY + 2][TX + 2];
  T xv[TY + 2][TX + 2];
  T rxx[TY + 1][TX + 1];
  T ryy[TY + 1][TX + 1];
  T e[TY + 1][TX + 1];
  T rxy[TY + 1][TX + 1];
};

// Stage 1: x region; f(q) gives the (transformed) value of solver-vector entry q.
template <typename T, int TX, int TY, typename F>
__device__ __forceinline__ void stage_x(const Dims& d, int i0, int j0, OpTile<T, TX, TY>& s, F&& f) {
  for (int p = flat_tid(); p < (TX + 2) * (TY + 2); p += flat_nthreads()) {
    const int li = p % (TX + 2), lj = p / (TX + 2);
    const int i = i0 - 1 + li, j = j0 - 1 + lj;
    s.xu[lj][li] = (i >= 0 && i <= d.nx && j >= 0 && j < d.ny) ? f(uidx(d, i, j)) : (T)0;
    s.xv[lj][li] = (i >= 0 && i < d.nx && j >= 0 && j <= d.ny) ? f(vidx(d, i, j)) : (T)0;
  }
}

// Stage 2: stresses (see k_op for the formulas).
template <typename T, int TX, int TY>
__device__ __forceinline__ void stage_stress(const Dims& d, const OpCoef<T>& cf, int i0, int j0, OpTile<T, TX, TY>& s) {
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  for (int p = flat_tid(); p < (TX + 1) * (TY + 1); p += flat_nthreads()) {
    const int la = p % (TX + 1), lb = p / (TX + 1);
    const int a = i0 - 1 + la, b = j0 - 1 + lb;
    T rxx = 0, ryy = 0, e = 0, rxy = 0;
    if (a >= 0 && a < d.nx && b >= 0 && b < d.ny) {
      const int hc = hidx(d, a, b);
      const T u0 = s.xu[lb][la], u1 = s.xu[lb][la + 1], v0 = s.xv[lb][la], v1 = s.xv[lb + 1][la];
      const T ux = (u1 - u0) * rdx, vy = (v1 - v0) * rdy;
      const T he2 = (T)2 * cf.heta_h[hc];
      rxx = he2 * ((T)2 * ux + vy);
      ryy = he2 * ((T)2 * vy + ux);
      const T dm = cf.dimp[hc];
      if (dm != (T)0) {
        const T divq = (cf.h_m[uidx(d, a + 1, b)] * u1 - cf.h_m[uidx(d, a, b)] * u0) * rdx +
                       (cf.h_m[vidx(d, a, b + 1)] * v1 - cf.h_m[vidx(d, a, b)] * v0) * rdy;
        e = dm * divq;
      }
    }
    if (a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1) {
      const T hc = cf.heta_c[cidx(d, a, b)];
      if (hc != (T)0) {
        const T uy = (s.xu[lb + 1][la + 1] - s.xu[lb][la + 1]) * rdy;
        const T vx = (s.xv[lb + 1][la + 1] - s.xv[lb + 1][la]) * rdx;
        rxy = hc * (uy + vx);
      }
    }
    s.rxx[lb][la] = rxx;
    s.ryy[lb][la] = ryy;
    s.e[lb][la] = e;
    s.rxy[lb][la] = rxy;
  }
}

// Stage 3: operator at the u point of local (li, lj) (1-based in the tile) / at the v point.
template <typename T, int TX, int TY>
__device__ __forceinline__ T stage_out_u(const Dims& d, const OpCoef<T>& cf, const OpTile<T, TX, TY>& s, int li, int lj, int q) {
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  return (s.rxx[lj][li] - s.rxx[lj][li - 1]) * rdx + (s.rxy[lj][li - 1] - s.rxy[lj - 1][li - 1]) * rdy -
         cf.beta_m[q] * s.xu[lj][li] - cf.h_m[q] * ((s.e[lj][li] - s.e[lj][li - 1]) * rdx);
}
template <typename T, int TX, int TY>
__device__ __forceinline__ T stage_out_v(const Dims& d, const OpCoef<T>& cf, const OpTile<T, TX, TY>& s, int li, int lj, int q) {
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  return (s.ryy[lj][li] - s.ryy[lj - 1][li]) * rdy + (s.rxy[lj - 1][li] - s.rxy[lj - 1][li - 1]) * rdx -
         cf.beta_m[q] * s.xv[lj][li] - cf.h_m[q] * ((s.e[lj][li] - s.e[lj - 1][li]) * rdy);
}

// ------------------------------------------------------------------------------------------------
// Haar lifting on a TILE x TILE shared-memory tile (one thread per element), for the grid component
// whose extent is (nxg, nyg) and whose tile origin is (bx0, by0).  KIND 0: idwt (M_B ... M_2 applied
// coarse-first), KIND 1: idwtᵀ (M_2ᵀ first), KIND 2: dwt (F_2 first); along y, then x.
// ------------------------------------------------------------------------------------------------
template <int TILE, int KIND, typename TT>
__device__ __forceinline__ void haar_tile(TT (*tile)[TILE + 1], int levels, int bx0, int by0, int nxg, int nyg) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int B = 1 << (levels + 1);
  const bool inside = (bx0 + tx) < nxg && (by0 + ty) < nyg;
  for (int dir = 0; dir < 2; ++dir) {
    const int n = dir == 0 ? nyg : nxg;
    const int base = dir == 0 ? by0 : bx0;
    const int pos = dir == 0 ? ty : tx;
    for (int lv = 0; lv <= levels; ++lv) {
      const int st = (KIND == 0) ? (B >> lv) : (2 << lv);
      const int half = st >> 1;
      const TT a = tile[ty][tx];
      TT nv = a;
      const int r = pos % st;
      if (inside && (r == 0 || r == half)) {
        const int po = r == 0 ? pos : pos - half;
        const int pe = po + half;
        if (base + pe < n) {
          const TT xo = dir == 0 ? tile[po][tx] : tile[ty][po];
          const TT xe = dir == 0 ? tile[pe][tx] : tile[ty][pe];
          const bool is_o = r == 0;
          if (KIND == 0) nv = is_o ? xo - xe : xe + xo;
          else if (KIND == 1) nv = is_o ? xo + xe : xe - xo;
          else nv = is_o ? (TT)0.5 * (xo + xe) : (TT)0.5 * (xe - xo);
        }
      }
      __syncthreads();
      tile[ty][tx] = nv;
      __syncthreads();
    }
  }
}

// ------------------------------------------------------------------------------------------------
// Picard-level kernels
// ------------------------------------------------------------------------------------------------
// Right-hand side, start guess, Dirichlet values, and |b|^2 (last block -> st->bb).
static __global__ void k_rhs_fused(Dims d, RhsIn in, const DevParams* __restrict__ P, double* __restrict__ b,
                            double* __restrict__ x, double* __restrict__ xfixed, double* __restrict__ partials,
                            DevState* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const double rho_i = P->rho_i, rho_w = P->rho_w, g = P->g, sl = P->sea_level, tdt = P->theta_dt;
  auto sadj = [&](int a, int c) -> double {
    if (a < 0 || a >= d.nx || c < 0 || c >= d.ny) return 0.0;
    const int q = hidx(d, a, c);
    if (!in.h_mask[q]) return 0.0;
    return in.s[q] + tdt * in.dsdh[q] * (in.acc[q] - in.melt[q]);
  };
  auto hmk = [&](int a, int c) -> double {
    return (a >= 0 && a < d.nx && c >= 0 && c < d.ny && in.h_mask[hidx(d, a, c)]) ? 1.0 : 0.0;
  };
  double bb = 0.0;
  auto point = [&](int q, int a0, int b0, int a1, int b1, double rd) {
    double bv = 0.0;
    if (in.inner[q]) {
      const double ds = sadj(a1, b1) * rd - sadj(a0, b0) * rd;
      const double dm = hmk(a1, b1) * rd - hmk(a0, b0) * rd;
      const double hh = in.h_uv[q], ss = in.s_uv[q];
      const double draft = fmax(hh - (ss - sl), 0.0);
      const double f1 = (rho_i * g * hh) * ds;
      const double f2 = dm * g * (0.5 * rho_i * (hh * hh) - 0.5 * rho_w * (draft * draft) - rho_i * hh * ss);
      bv = f1 + f2;
    }
    b[q] = bv;
    bb += bv * bv;
    x[q] = in.inner[q] ? in.uv[q] : 0.0;
    xfixed[q] = in.fixed[q] ? in.uv[q] : 0.0;
  };
  if (i <= d.nx && j < d.ny) point(uidx(d, i, j), i - 1, j, i, j, d.rdx);
  if (i < d.nx && j <= d.ny) point(vidx(d, i, j), i, j - 1, i, j, d.rdy);
  double tot[2];
  if (last_block_sum2(bb, 0.0, partials, &st->counter[CNT_A], tot)) {
    if (flat_tid() == 0) st->bb = tot[0];
  }
}

// b -= A xfixed (the Dirichlet lift, get_rhs_dirichlet!, update_velocities.jl:406-421), recomputing |b|^2.
template <int TX, int TY>
__global__ void __launch_bounds__(TX* TY)
    k_lift(Dims d, OpCoef<double> cf, const double* __restrict__ xfixed, double* __restrict__ b,
           double* __restrict__ partials, DevState* st) {
  __shared__ OpTile<double, TX, TY> s;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  stage_x(d, i0, j0, s, [&](int q) { return xfixed[q]; });
  __syncthreads();
  stage_stress(d, cf, i0, j0, s);
  __syncthreads();
  const int li = threadIdx.x + 1, lj = threadIdx.y + 1, i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  double bb = 0.0;
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    double v = b[q];
    if (cf.inner[q]) v = v - stage_out_u(d, cf, s, li, lj, q);
    b[q] = v;
    bb += v * v;
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    double v = b[q];
    if (cf.inner[q]) v = v - stage_out_v(d, cf, s, li, lj, q);
    b[q] = v;
    bb += v * v;
  }
  double tot[2];
  if (last_block_sum2(bb, 0.0, partials, &st->counter[CNT_B], tot)) {
    if (flat_tid() == 0) st->bb = tot[0];
  }
}

// r = b - A x (float64), |r|^2; the last block takes the Picard decision (update_velocities.jl:20, :59-65)
// and sets the Picard WHILE and V-cycle IF conditions.
template <int TX, int TY>
__global__ void __launch_bounds__(TX* TY)
    k_picard_residual(Dims d, OpCoef<double> cf, const double* __restrict__ x, const double* __restrict__ b,
                      double* __restrict__ r, double* __restrict__ resid_out, double* __restrict__ partials,
                      DevState* st, const DevParams* __restrict__ P, CondHandles h) {
  __shared__ OpTile<double, TX, TY> s;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  stage_x(d, i0, j0, s, [&](int q) { return x[q]; });
  __syncthreads();
  stage_stress(d, cf, i0, j0, s);
  __syncthreads();
  const int li = threadIdx.x + 1, lj = threadIdx.y + 1, i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  double rr = 0.0;
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    double v = 0.0;
    if (cf.inner[q]) {
      v = b[q] - stage_out_u(d, cf, s, li, lj, q);
      resid_out[q] = v;
    }
    r[q] = v;
    rr += v * v;
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    double v = 0.0;
    if (cf.inner[q]) {
      v = b[q] - stage_out_v(d, cf, s, li, lj, q);
      resid_out[q] = v;
    }
    r[q] = v;
    rr += v * v;
  }
  double tot[2];
  if (last_block_sum2(rr, 0.0, partials, &st->counter[CNT_C], tot)) {
    if (flat_tid() == 0) {
      st->rr = tot[0];
      const double rel = sqrt(tot[0]) / sqrt(st->bb);
      st->rel = rel;
      const int it = st->picard_it + 1;
      st->picard_it = it;
      bool conv = rel < P->tol_picard;
      if (conv && P->picard_test == 1 && it > 1 && !(st->rel_update <= P->tol_picard)) conv = false;
      if (!isfinite(rel)) {
        st->status = WAVI_ERR_NONFINITE;
        conv = true;  // stop: nothing sensible can follow a non-finite residual
      }
      st->converged = conv ? 1 : 0;
      st->vcycle_needed = conv ? 0 : 1;
      st->picard_continue = (!conv && it < P->maxiter_picard) ? 1 : 0;
      if (h.active) {
        cudaGraphSetConditional(h.vcycle, st->vcycle_needed);
        cudaGraphSetConditional(h.picard, st->picard_continue);
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------
// V-cycle kernels
// ------------------------------------------------------------------------------------------------
// V-cycle start: rs = (T) r, rsm = rs, corr = 0, xc = (T) xc64, diag = op diagonal (closed form).
template <typename T>
__global__ void k_vcycle_init(Dims d, OpCoef<T> cf, const double* __restrict__ r64, const double* __restrict__ xc64,
                              T* __restrict__ rs, T* __restrict__ rsm, T* __restrict__ corr, T* __restrict__ xc,
                              T* __restrict__ diag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d), rdx2 = rdx * rdx, rdy2 = rdy * rdy;
  auto heh = [&](int a, int b) -> T { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny) ? cf.heta_h[hidx(d, a, b)] : (T)0; };
  auto dim = [&](int a, int b) -> T { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny) ? cf.dimp[hidx(d, a, b)] : (T)0; };
  auto hec = [&](int a, int b) -> T {
    return (a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1) ? cf.heta_c[cidx(d, a, b)] : (T)0;
  };
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    const T rv = (T)r64[q];
    rs[q] = rv;
    rsm[q] = rv;
    corr[q] = (T)0;
    xc[q] = (T)xc64[q];
    T v = 0;
    if (cf.inner[q]) {
      const T hu = cf.h_m[q];
      v = -(T)4 * rdx2 * (heh(i, j) + heh(i - 1, j)) - rdy2 * (hec(i - 1, j) + hec(i - 1, j - 1)) - cf.beta_m[q] +
          hu * hu * rdx2 * (dim(i, j) + dim(i - 1, j));
    }
    diag[q] = v;
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    const T rv = (T)r64[q];
    rs[q] = rv;
    rsm[q] = rv;
    corr[q] = (T)0;
    xc[q] = (T)xc64[q];
    T v = 0;
    if (cf.inner[q]) {
      const T hv = cf.h_m[q];
      v = -(T)4 * rdy2 * (heh(i, j) + heh(i, j - 1)) - rdx2 * (hec(i, j - 1) + hec(i - 1, j - 1)) - cf.beta_m[q] +
          hv * hv * rdy2 * (dim(i, j) + dim(i, j - 1));
    }
    diag[q] = v;
  }
}

// One smoother sweep (gauss_seidel_smoother!, update_preconditioners.jl:133-150), fused: the Jacobi
// update of colour `colour` (x += ω r / diag, recomputed for the tile and its halo from the previous
// x and r) followed by the full residual r = b - A x on the tile.  Ping-pong buffers: reads (x_in,
// r_in), writes (x_out, r_out).  UPDATE = false computes only r_out = b - A x_in.
template <typename T, int TX, int TY, bool UPDATE>
__global__ void __launch_bounds__(TX* TY)
    k_smooth(Dims d, OpCoef<T> cf, int colour, const DevParams* __restrict__ P, const T* __restrict__ b,
             const T* __restrict__ diag, const T* __restrict__ x_in, const T* __restrict__ r_in,
             T* __restrict__ x_out, T* __restrict__ r_out) {
  __shared__ OpTile<T, TX, TY> s;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const T omega = (T)P->omega;
  const int Nu = d.Nu, nxu = d.nx + 1, nxv = d.nx;
  stage_x(d, i0, j0, s, [&](int q) -> T {
    T v = x_in[q];
    if (UPDATE && cf.inner[q]) {
      int i, j, base;
      if (q < Nu) { i = q % nxu; j = q / nxu; base = 1; }
      else { i = (q - Nu) % nxv; j = (q - Nu) / nxv; base = 3; }
      const int par = ((i - j) % 2 + 2) % 2;
      if (base + par == colour) v = v + omega * r_in[q] / diag[q];
    }
    return v;
  });
  __syncthreads();
  stage_stress(d, cf, i0, j0, s);
  __syncthreads();
  const int li = threadIdx.x + 1, lj = threadIdx.y + 1, i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    T f = 0;
    if (cf.inner[q]) f = b[q] - stage_out_u(d, cf, s, li, lj, q);
    r_out[q] = f;
    if (UPDATE) x_out[q] = s.xu[lj][li];
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    T f = 0;
    if (cf.inner[q]) f = b[q] - stage_out_v(d, cf, s, li, lj, q);
    r_out[q] = f;
    if (UPDATE) x_out[q] = s.xv[lj][li];
  }
}

// ------------------------------------------------------------------------------------------------
// Row-streaming operator for large grids (the same arithmetic as k_op / k_smooth, in the same order).
// A warp owns 32 consecutive columns i = ib-1 .. ib+30 of the (nx+1) x (ny+1) index space and walks up
// the rows of its strip; lanes 1..30 write the outputs of columns ib .. ib+29.  The x-neighbours of a
// point come from the adjacent lanes (warp shuffles) and its y-neighbours from the registers of the
// previous row, so every array element is read once per strip, with whole-row coalesced loads, and no
// shared memory or block barrier is involved.  While row j computes, a lane's loads for the next rows
// are in flight: u, v, h_u, h_v of row j+2 and hη_h, dimp, hη_c, β_u, β_v and the interior masks of
// row j+1.  It writes f_u(i,j), f_v(i,j).
//   MODE 0: y = A x      MODE 2: smoother sweep: x_out = x_in + ω r_in / diag on colour `colour`,
//                                r_out = b - A x_out on the interior (the fused k_smooth<UPDATE>)
//   MODE 1: y = b - A x on the interior (k_smooth<!UPDATE>)
// ------------------------------------------------------------------------------------------------
constexpr int ST_WARPS = 4;   // warps per block
constexpr int ST_COLS = 30;   // output columns per warp

template <typename T, int MODE>
__global__ void __launch_bounds__(32 * ST_WARPS)
    k_op_stream(Dims d, OpCoef<T> cf, int rows, const T* __restrict__ x, const T* __restrict__ b, T* __restrict__ y,
                int colour, const DevParams* __restrict__ P, const T* __restrict__ diag, const T* __restrict__ r_in,
                T* __restrict__ x_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ib = (blockIdx.x * ST_WARPS + warp) * ST_COLS;
  const int i = ib - 1 + lane;
  const int j0 = blockIdx.y * rows, j1 = min(j0 + rows, d.ny + 1);
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  const T omega = MODE == 2 ? (T)P->omega : (T)0;
  const bool out_lane = lane >= 1 && lane <= ST_COLS;
  const bool col_u = i >= 0 && i <= d.nx, col_v = i >= 0 && i < d.nx;
  auto xu_at = [&](int jj) -> T {
    if (!col_u || jj < 0 || jj >= d.ny) return (T)0;
    const int q = uidx(d, i, jj);
    T v = x[q];
    if (MODE == 2 && 1 + ((i - jj) & 1) == colour && cf.inner[q]) v = v + omega * r_in[q] / diag[q];
    return v;
  };
  auto xv_at = [&](int jj) -> T {
    if (!col_v || jj < 0 || jj > d.ny) return (T)0;
    const int q = vidx(d, i, jj);
    T v = x[q];
    if (MODE == 2 && 3 + ((i - jj) & 1) == colour && cf.inner[q]) v = v + omega * r_in[q] / diag[q];
    return v;
  };
  auto hu_at = [&](int jj) -> T { return (col_u && jj >= 0 && jj < d.ny) ? cf.h_m[uidx(d, i, jj)] : (T)0; };
  auto hv_at = [&](int jj) -> T { return (col_v && jj >= 0 && jj <= d.ny) ? cf.h_m[vidx(d, i, jj)] : (T)0; };
  // per-row coefficients, loaded one row ahead of their use
  struct RowCoef {
    T heh, dm, hec, bu, bv;
    uint8_t iu, iv;
  };
  auto coef_at = [&](int jj) -> RowCoef {
    RowCoef r{(T)0, (T)0, (T)0, (T)0, (T)0, 0, 0};
    if (col_v && jj >= 0 && jj < d.ny) {
      r.heh = cf.heta_h[hidx(d, i, jj)];
      r.dm = cf.dimp[hidx(d, i, jj)];
    }
    if (i >= 0 && i < d.nx - 1 && jj >= 0 && jj < d.ny - 1) r.hec = cf.heta_c[cidx(d, i, jj)];
    if (jj >= j0 && out_lane) {
      if (col_u && jj < d.ny) {
        const int q = uidx(d, i, jj);
        r.iu = cf.inner[q];
        r.bu = cf.beta_m[q];
      }
      if (col_v && jj <= d.ny) {
        const int q = vidx(d, i, jj);
        r.iv = cf.inner[q];
        r.bv = cf.beta_m[q];
      }
    }
    return r;
  };
  int j = j0 - 1;
  T u_c = xu_at(j), v_c = xv_at(j), hu_c = hu_at(j), hv_c = hv_at(j);
  T u_n = xu_at(j + 1), v_n = xv_at(j + 1), hv_n = hv_at(j + 1), hu_n = hu_at(j + 1);
  RowCoef k_c = coef_at(j);
  T ryy_p = 0, e_p = 0, rxyc_p = 0, rxyc_pl = 0;
  for (; j < j1; ++j) {
    const bool hcell = col_v && j >= 0 && j < d.ny;
    const bool cpt = i >= 0 && i < d.nx - 1 && j >= 0 && j < d.ny - 1;
    // next rows' loads go out before this row's arithmetic
    const RowCoef k_n = coef_at(j + 1);
    const T u_nn = xu_at(j + 2), v_nn = xv_at(j + 2), hv_nn = hv_at(j + 2), hu_nn = hu_at(j + 2);
    const T uR = __shfl_down_sync(0xffffffffu, u_c, 1), huR = __shfl_down_sync(0xffffffffu, hu_c, 1);
    const T u_nR = __shfl_down_sync(0xffffffffu, u_n, 1), v_nR = __shfl_down_sync(0xffffffffu, v_n, 1);
    T rxx = 0, ryy = 0, e = 0, rxyc = 0;
    if (hcell) {
      const T ux = (uR - u_c) * rdx, vy = (v_n - v_c) * rdy;
      const T he2 = (T)2 * k_c.heh;
      rxx = he2 * ((T)2 * ux + vy);
      ryy = he2 * ((T)2 * vy + ux);
      if (k_c.dm != (T)0) e = k_c.dm * ((huR * uR - hu_c * u_c) * rdx + (hv_n * v_n - hv_c * v_c) * rdy);
    }
    if (cpt && k_c.hec != (T)0) rxyc = k_c.hec * ((u_nR - uR) * rdy + (v_nR - v_n) * rdx);
    const T rxx_l = __shfl_up_sync(0xffffffffu, rxx, 1), e_l = __shfl_up_sync(0xffffffffu, e, 1);
    const T rxyc_l = __shfl_up_sync(0xffffffffu, rxyc, 1);
    if (j >= j0 && out_lane) {
      if (col_u && j < d.ny) {
        const int q = uidx(d, i, j);
        T f = 0;
        if (k_c.iu) {
          f = (rxx - rxx_l) * rdx + (rxyc_l - rxyc_pl) * rdy - k_c.bu * u_c - hu_c * ((e - e_l) * rdx);
          if (MODE != 0) f = b[q] - f;
        }
        y[q] = f;
        if (MODE == 2) x_out[q] = u_c;
      }
      if (col_v && j <= d.ny) {
        const int q = vidx(d, i, j);
        T f = 0;
        if (k_c.iv) {
          f = (ryy - ryy_p) * rdy + (rxyc_p - rxyc_pl) * rdx - k_c.bv * v_c - hv_c * ((e - e_p) * rdy);
          if (MODE != 0) f = b[q] - f;
        }
        y[q] = f;
        if (MODE == 2) x_out[q] = v_c;
      }
    }
    ryy_p = ryy;
    e_p = e;
    rxyc_p = rxyc;
    rxyc_pl = rxyc_l;
    u_c = u_n;
    v_c = v_n;
    hu_c = hu_n;
    hv_c = hv_n;
    u_n = u_nn;
    v_n = v_nn;
    hu_n = hu_nn;
    hv_n = hv_nn;
    k_c = k_n;
  }
}

// Launch shape of k_op_stream: column blocks of ST_WARPS * ST_COLS, row strips sized for ~8 blocks per SM.
inline void stream_shape(const Dims& d, int nsm, dim3& grid, int& rows) {
  const int ncb = (d.nx + 1 + ST_WARPS * ST_COLS - 1) / (ST_WARPS * ST_COLS);
  const long target = 8L * nsm;
  rows = (int)std::min<long>(64, std::max<long>(8, ((long)(d.ny + 1) * ncb + target - 1) / target));
  grid = dim3((unsigned)ncb, (unsigned)((d.ny + 1 + rows - 1) / rows));
}

// ------------------------------------------------------------------------------------------------
// Compact <-> full coarse-correction cache on the device.  The reference stores the coarse correction
// compactly, one entry per true wavelet-mask point in column-major order (UWavelets.jl:46,
// get_correction_coarse / set_correction_coarse!, update_preconditioners.jl:195-216); the solver keeps
// it on the full grid.  A point's compact index is the number of mask points before it: per-block
// counts (k_mask_count), an exclusive scan of the counts (k_scan_counts, one block), then each block
// ranks its points with warp ballots (k_mask_map).  One range (the u part or the v part) per launch.
// ------------------------------------------------------------------------------------------------
constexpr int MS_BLOCK = 1024;

static __global__ void __launch_bounds__(MS_BLOCK) k_mask_count(const uint8_t* __restrict__ m, int n, int* __restrict__ counts) {
  const int i = blockIdx.x * MS_BLOCK + threadIdx.x;
  const int c = __syncthreads_count(i < n && m[i] != 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

static __global__ void __launch_bounds__(MS_BLOCK) k_scan_counts(int* __restrict__ counts, int nblocks) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (t == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nblocks; base += MS_BLOCK) {
    const int k = base + t;
    const int v = k < nblocks ? counts[k] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      int w = warp_tot[lane], wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += y;
      }
      warp_tot[lane] = wi - w;  // exclusive warp offsets
    }
    __syncthreads();
    const int excl = carry + warp_tot[wid] + incl - v;
    __syncthreads();
    if (k < nblocks) counts[k] = excl;
    if (t == MS_BLOCK - 1) carry = excl + v;
    __syncthreads();
  }
}

// EXPAND: full[i] = m[i] ? compact[rank(i)] : 0 (and m01[i] = m[i] != 0); else compact[rank(i)] = full[i].
template <bool EXPAND>
__global__ void __launch_bounds__(MS_BLOCK)
    k_mask_map(const uint8_t* __restrict__ m, int n, const int* __restrict__ offsets, double* __restrict__ full,
               double* __restrict__ compact, uint8_t* __restrict__ m01) {
  __shared__ int warp_off[32];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int i = blockIdx.x * MS_BLOCK + t;
  const bool on = i < n && m[i] != 0;
  const unsigned bal = __ballot_sync(0xffffffffu, on);
  if (lane == 0) warp_off[wid] = __popc(bal);
  __syncthreads();
  if (wid == 0) {
    const int w = warp_off[lane];
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    warp_off[lane] = wi - w;
  }
  __syncthreads();
  if (i >= n) return;
  const int pos = offsets[blockIdx.x] + warp_off[wid] + __popc(bal & ((1u << lane) - 1u));
  if (EXPAND) {
    full[i] = on ? compact[pos] : 0.0;
    m01[i] = on ? 1 : 0;
  } else if (on) {
    compact[pos] = full[i];
  }
}

// Haar restriction of a fine vector (KIND 1, masked by the wavelet mask) with |out|^2; the last block
// stores |b_c| = sqrt(total) for the coarse CG's absolute tolerance (update_preconditioners.jl:65-70).
template <typename T, int TILE>
__global__ void __launch_bounds__(TILE* TILE)
    k_restrict_norm(Dims d, int levels, const T* __restrict__ in, const uint8_t* __restrict__ wmask, T* __restrict__ out,
                    double* __restrict__ partials, DevState* st) {
  __shared__ T tile[2][TILE][TILE + 1];
  const int bx0 = blockIdx.x * TILE, by0 = blockIdx.y * TILE, tx = threadIdx.x, ty = threadIdx.y;
  const int i = bx0 + tx, j = by0 + ty;
  const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
  tile[0][ty][tx] = inu ? in[uidx(d, i, j)] : (T)0;
  tile[1][ty][tx] = inv ? in[vidx(d, i, j)] : (T)0;
  __syncthreads();
  haar_tile<TILE, 1>(tile[0], levels, bx0, by0, d.nx + 1, d.ny);
  haar_tile<TILE, 1>(tile[1], levels, bx0, by0, d.nx, d.ny + 1);
  double s2 = 0.0;
  if (inu) {
    const int q = uidx(d, i, j);
    const T o = wmask[q] ? tile[0][ty][tx] : (T)0;
    out[q] = o;
    s2 += (double)o * (double)o;
  }
  if (inv) {
    const int q = vidx(d, i, j);
    const T o = wmask[q] ? tile[1][ty][tx] : (T)0;
    out[q] = o;
    s2 += (double)o * (double)o;
  }
  double tot[2];
  if (last_block_sum2(s2, 0.0, partials, &st->counter[CNT_A], tot)) {
    if (flat_tid() == 0) st->cg_bnorm = sqrt(tot[0]);
  }
}

// Prolongation (KIND 0, masked by the interior mask).  MODE 0: out = P in.  MODE 1: out += P in.
// MODE 2 (CG direction): first u = r + β u on the tile (β = |r|^2/|r_prev|^2 from the state), written
// back to `dir`, then out = P u.
template <typename T, int TILE, int MODE>
__global__ void __launch_bounds__(TILE* TILE)
    k_prolong(Dims d, int levels, const uint8_t* __restrict__ inner, const T* __restrict__ in, T* __restrict__ out,
              const T* __restrict__ rvec, T* __restrict__ dir, const DevState* __restrict__ st, const int* __restrict__ live) {
  if (live && !*live) return;
  __shared__ T tile[2][TILE][TILE + 1];
  const int bx0 = blockIdx.x * TILE, by0 = blockIdx.y * TILE, tx = threadIdx.x, ty = threadIdx.y;
  const int i = bx0 + tx, j = by0 + ty;
  const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
  if (MODE == 2) {
    const double res = st->cg_res, prev = st->cg_prev;
    const double beta = (res * res) / (prev * prev);
    if (inu) {
      const int q = uidx(d, i, j);
      const T u = (T)((double)rvec[q] + beta * (double)dir[q]);
      dir[q] = u;
      tile[0][ty][tx] = u;
    } else {
      tile[0][ty][tx] = (T)0;
    }
    if (inv) {
      const int q = vidx(d, i, j);
      const T u = (T)((double)rvec[q] + beta * (double)dir[q]);
      dir[q] = u;
      tile[1][ty][tx] = u;
    } else {
      tile[1][ty][tx] = (T)0;
    }
  } else {
    tile[0][ty][tx] = inu ? in[uidx(d, i, j)] : (T)0;
    tile[1][ty][tx] = inv ? in[vidx(d, i, j)] : (T)0;
  }
  __syncthreads();
  haar_tile<TILE, 0>(tile[0], levels, bx0, by0, d.nx + 1, d.ny);
  haar_tile<TILE, 0>(tile[1], levels, bx0, by0, d.nx, d.ny + 1);
  if (inu) {
    const int q = uidx(d, i, j);
    const T o = inner[q] ? tile[0][ty][tx] : (T)0;
    out[q] = MODE == 1 ? (T)(out[q] + o) : o;
  }
  if (inv) {
    const int q = vidx(d, i, j);
    const T o = inner[q] ? tile[1][ty][tx] : (T)0;
    out[q] = MODE == 1 ? (T)(out[q] + o) : o;
  }
}

// Coarse operator application c = R A P u with P u = w given: the operator on a TILE x TILE tile, then
// the Haar restriction of the tile in shared memory (op_coarse_fun!, update_preconditioners.jl:176-193).
// DOT: partial <u, c>; the last block sets α = |r|^2 / <u, c> (cg.jl iterate).  START: instead write
// r = b - c, u = 0, |r|^2, and the last block initialises the CG scalars and its WHILE condition.
template <typename T, int TILE, bool START>
__global__ void __launch_bounds__(TILE* TILE)
    k_coarse_op(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, const T* __restrict__ w,
                T* __restrict__ c, T* __restrict__ u, T* __restrict__ rvec, const T* __restrict__ bvec,
                double* __restrict__ partials, DevState* st, const DevParams* __restrict__ P, CondHandles h,
                const int* __restrict__ live) {
  if (live && !*live) return;
  __shared__ OpTile<T, TILE, TILE> s;
  __shared__ T tile[2][TILE][TILE + 1];
  const int i0 = blockIdx.x * TILE, j0 = blockIdx.y * TILE;
  stage_x(d, i0, j0, s, [&](int q) { return w[q]; });
  __syncthreads();
  stage_stress(d, cf, i0, j0, s);
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y, li = tx + 1, lj = ty + 1, i = i0 + tx, j = j0 + ty;
  const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
  tile[0][ty][tx] = (inu && cf.inner[uidx(d, i, j)]) ? stage_out_u(d, cf, s, li, lj, uidx(d, i, j)) : (T)0;
  tile[1][ty][tx] = (inv && cf.inner[vidx(d, i, j)]) ? stage_out_v(d, cf, s, li, lj, vidx(d, i, j)) : (T)0;
  __syncthreads();
  haar_tile<TILE, 1>(tile[0], levels, i0, j0, d.nx + 1, d.ny);
  haar_tile<TILE, 1>(tile[1], levels, i0, j0, d.nx, d.ny + 1);
  double acc = 0.0;
  auto finish = [&](int q, T cv) {
    cv = wmask[q] ? cv : (T)0;
    if (START) {
      const T rv = bvec[q] - cv;
      rvec[q] = rv;
      u[q] = (T)0;
      acc += (double)rv * (double)rv;
    } else {
      c[q] = cv;
      acc += (double)u[q] * (double)cv;
    }
  };
  if (inu) finish(uidx(d, i, j), tile[0][ty][tx]);
  if (inv) finish(vidx(d, i, j), tile[1][ty][tx]);
  double tot[2];
  if (last_block_sum2(acc, 0.0, partials, &st->counter[START ? CNT_B : CNT_C], tot)) {
    if (flat_tid() == 0) {
      if (START) {
        const double res = sqrt(tot[0]);
        const double abstol = coarse_tolerance(P, st) * st->cg_bnorm;
        st->cg_res = res;
        st->cg_prev = 1.0;
        st->cg_tol = fmax(1.4901161193847656e-08 * res, abstol);  // reltol = sqrt(eps(Float64))
        st->cg_it = 0;
        const bool done = (0 >= P->maxiter_coarse) || res <= st->cg_tol || !(res == res);
        st->cg_continue = done ? 0 : 1;
        if (h.active) cudaGraphSetConditional(h.cg, st->cg_continue);
      } else {
        st->cg_alpha = (st->cg_res * st->cg_res) / tot[0];
      }
    }
  }
}

// x += α u; r -= α c; |r|^2; the last block advances the CG scalars and its WHILE condition.
template <typename T>
__global__ void k_cg_update(int n, const T* __restrict__ u, const T* __restrict__ c, T* __restrict__ x, T* __restrict__ r,
                            double* __restrict__ partials, DevState* st, const DevParams* __restrict__ P, CondHandles h,
                            int* live) {
  if (live && !*live) return;
  const double alpha = st->cg_alpha;
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    x[k] = (T)((double)x[k] + alpha * (double)u[k]);
    const T rv = (T)((double)r[k] - alpha * (double)c[k]);
    r[k] = rv;
    s += (double)rv * (double)rv;
  }
  double tot[2];
  if (last_block_sum2(s, 0.0, partials, &st->counter[CNT_D], tot)) {
    if (flat_tid() == 0) {
      st->cg_prev = st->cg_res;
      const double res = sqrt(tot[0]);
      st->cg_res = res;
      const int it = st->cg_it + 1;
      st->cg_it = it;
      st->cg_total += 1;
      const bool done = it >= P->maxiter_coarse || res <= st->cg_tol || !(res == res);
      st->cg_continue = done ? 0 : 1;
      if (live) *live = st->cg_continue;
      if (h.active) cudaGraphSetConditional(h.cg, st->cg_continue);
    }
  }
}

// End of the V-cycle: x64 += corr; u/v = x at the interior; xc64 = xc (the next coarse solve's warm
// start); |corr|^2 and |x|^2 for the relative update.
//
// In the FP32 coarse solve the warm start is dropped (xc64 = 0) when the coarse CG ended without meeting
// its tolerance.  On a masked grid R A P is singular (Haar basis functions that coincide on the ice);
// FP32 rounding leaves b slightly outside R A P's range, so each solve drifts along the null space, and
// through the warm start the drift accumulates over V-cycles until every coarse solve runs to
// maxiter_coarse and the Picard loop stalls near 1e-6.  A converged coarse solve keeps its warm start,
// so solves that never hit maxiter_coarse are unchanged; the FP64 path keeps the reference's cache.
template <typename T>
__global__ void k_vcycle_finish(int n, const uint8_t* __restrict__ inner, const T* __restrict__ corr, const T* __restrict__ xc,
                                double* __restrict__ x, double* __restrict__ uv, double* __restrict__ xc64,
                                double* __restrict__ partials, DevState* st) {
  const bool keep = sizeof(T) == sizeof(double) || st->cg_res <= st->cg_tol;
  double s0 = 0.0, s1 = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double cv = (double)corr[k];
    const double v = x[k] + cv;
    x[k] = v;
    if (inner[k]) uv[k] = v;
    xc64[k] = keep ? (double)xc[k] : 0.0;
    s0 += cv * cv;
    s1 += v * v;
  }
  double tot[2];
  if (last_block_sum2(s0, s1, partials, &st->counter[CNT_A], tot)) {
    if (flat_tid() == 0) {
      st->du2 = tot[0];
      st->uu2 = tot[1];
      st->rel_update = sqrt(tot[0]) / sqrt(tot[1]);
    }
  }
}

// Solve start: zero the counters and flags.
static __global__ void k_state_init(DevState* st) {
  if (threadIdx.x == 0) {
    DevState z = {};
    z.rel = INFINITY;
    z.rel_update = INFINITY;
    z.picard_continue = 1;
    *st = z;
  }
}

}  // namespace wavi
