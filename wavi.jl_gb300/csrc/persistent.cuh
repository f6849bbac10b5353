// persistent.cuh — the coarse conjugate-gradient solve of one V-cycle as a single persistent kernel.
//
// The coarse solve (IterativeSolvers cg! on R A P, update_preconditioners.jl:54-83) is a long chain of
// small dependent steps: at 640 x 80 one iteration moves ~1 MB, far below what a launch costs.  Here one
// cooperative launch runs every iteration.  Each CTA owns up to MAXT tiles of TILE x TILE points (a tile
// holds whole Haar blocks of both velocity components); each thread keeps, in registers, the CG
// vectors (direction u, residual r, iterate x, and R A P u) of its own point of every owned tile for the
// whole solve.  Per iteration only the prolonged direction w = P u crosses L2 (the operator needs a
// one-point halo of it); three grid barriers separate the phases:
//
//   1. u = r + β u;  w = P u (Haar synthesis of the tile, masked by the interior)  -> barrier
//   2. c = R A w (operator on the tile + halo of w, Haar analysis, wavelet mask); partial <u, c>
//                                                                                  -> barrier + sum
//   3. α = |r|^2/<u,c>;  x += α u;  r -= α c;  partial |r|^2                       -> barrier + sum
//
// Every CTA derives the scalars from the same sums, so all CTAs take the same decisions.  The sums are
// deterministic (the last CTA to arrive adds the per-CTA partials in CTA order).  Every wait is
// bounded: after ~2^22 polls a CTA records WAVI_ERR_WATCHDOG and all CTAs leave the kernel.
#pragma once
#include "fused.cuh"

namespace wavi {

struct GridBar {
  unsigned count;
  unsigned gen;
  int err;
  int pad;
  double sum[2];
};

constexpr long kBarrierSpinLimit = 1L << 22;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier over gridDim.x CTAs.  With REDUCE, (v0, v1) of every thread are summed over the grid
// and returned in out[0..1] to every thread.  Returns false (for every thread of the CTA) if the wait
// gave up or another CTA reported an error.
template <bool REDUCE>
__device__ __forceinline__ bool grid_barrier(GridBar* bar, double* __restrict__ partials, double v0, double v1,
                                             double out[2]) {
  __shared__ double sh[32];
  __shared__ int s_last, s_ok;
  __shared__ unsigned s_gen;
  const int t = flat_tid(), nt = flat_nthreads();
  const unsigned nb = gridDim.x;
  double a0 = 0.0, a1 = 0.0;
  if (REDUCE) {
    a0 = block_sum_any(v0, sh);
    __syncthreads();
    a1 = block_sum_any(v1, sh);
  }
  __syncthreads();
  if (t == 0) {
    if (REDUCE) {
      partials[2 * blockIdx.x] = a0;
      partials[2 * blockIdx.x + 1] = a1;
    }
    s_gen = ld_acquire_u32(&bar->gen);
    __threadfence();
    const unsigned prev = atomicAdd(&bar->count, 1u);
    s_last = (prev == nb - 1u) ? 1 : 0;
    s_ok = 1;
  }
  __syncthreads();
  if (s_last) {
    if (REDUCE) {
      __threadfence();
      double b0 = 0.0, b1 = 0.0;
      for (int k = t; k < (int)nb; k += nt) {
        b0 += __ldcg(partials + 2 * k);
        b1 += __ldcg(partials + 2 * k + 1);
      }
      b0 = block_sum_any(b0, sh);
      __syncthreads();
      b1 = block_sum_any(b1, sh);
      if (t == 0) {
        bar->sum[0] = b0;
        bar->sum[1] = b1;
      }
    }
    if (t == 0) {
      bar->count = 0u;
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    }
  } else if (t == 0) {
    long polls = 0;
    while (ld_acquire_u32(&bar->gen) == s_gen) {
      if (++polls > kBarrierSpinLimit || *(volatile int*)&bar->err) {
        atomicExch(&bar->err, 1);
        s_ok = 0;
        break;
      }
      __nanosleep(64);
    }
  }
  __syncthreads();
  __threadfence();
  if (REDUCE) {
    out[0] = __ldcg(&bar->sum[0]);
    out[1] = __ldcg(&bar->sum[1]);
  }
  return s_ok != 0;
}

// One lifting pass along a 1-D line held one element per lane (lane bits below TILE select the
// position): pairs (o, o + s/2), o a multiple of s, exchanged with warp shuffles.  KIND as haar_tile.
template <int KIND, typename TT>
__device__ __forceinline__ TT lift_lanes(TT v, int pos, int base, int n, bool inside, int levels) {
  const int B = 1 << (levels + 1);
  for (int lv = 0; lv <= levels; ++lv) {
    const int st = (KIND == 0) ? (B >> lv) : (2 << lv);
    const int half = st >> 1;
    const TT p = __shfl_xor_sync(0xffffffffu, v, half);
    const int r = pos & (st - 1);
    if (inside) {
      if (r == 0) {
        if (base + pos + half < n) v = (KIND == 0) ? v - p : (KIND == 1) ? v + p : (TT)0.5 * (v + p);
      } else if (r == half) {
        v = (KIND == 0) ? p + v : (KIND == 1) ? v - p : (TT)0.5 * (v - p);
      }
    }
  }
  return v;
}

// 2-D Haar transform of a TILE x TILE tile held one element per thread (thread (tx, ty) = element
// (bx0 + tx, by0 + ty) of a grid component of extent nxg x nyg): along y through a shared-memory
// transpose, then along x, both with warp shuffles.  Must be called by every thread of the CTA.
template <int TILE, int KIND, typename TT>
__device__ __forceinline__ TT haar2d(TT v, TT (*sm)[TILE + 1], int bx0, int by0, int nxg, int nyg, int levels) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  __syncthreads();
  sm[ty][tx] = v;
  __syncthreads();
  TT w = sm[tx][ty];  // element (bx0 + ty, by0 + tx): its position along y is tx
  w = lift_lanes<KIND>(w, tx, by0, nyg, (bx0 + ty) < nxg && (by0 + tx) < nyg, levels);
  sm[tx][ty] = w;
  __syncthreads();
  v = sm[ty][tx];
  return lift_lanes<KIND>(v, tx, bx0, nxg, (bx0 + tx) < nxg && (by0 + ty) < nyg, levels);
}

template <typename T, int TILE>
struct CGShared {
  OpTile<T, TILE, TILE> op;
  T hs[TILE][TILE + 1];
};

// c = wmask ⊙ R (A w) at this thread's point of the tile with origin (i0, j0); w is read from global
// memory (tile + halo).  Every thread of the CTA must call it.
template <typename T, int TILE>
__device__ __forceinline__ void coarse_apply(const Dims& d, int levels, const OpCoef<T>& cf, const uint8_t* __restrict__ wmask,
                                             const T* __restrict__ w, int i0, int j0, CGShared<T, TILE>& sm, T& cu, T& cv) {
  __syncthreads();  // the previous use of the tile's shared memory is over
  stage_x(d, i0, j0, sm.op, [&](int q) { return __ldcg(w + q); });
  __syncthreads();
  stage_stress(d, cf, i0, j0, sm.op);
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y, i = i0 + tx, j = j0 + ty;
  const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
  T yu = 0, yv = 0;
  if (inu) {
    const int q = uidx(d, i, j);
    if (cf.inner[q]) yu = stage_out_u(d, cf, sm.op, tx + 1, ty + 1, q);
  }
  if (inv) {
    const int q = vidx(d, i, j);
    if (cf.inner[q]) yv = stage_out_v(d, cf, sm.op, tx + 1, ty + 1, q);
  }
  yu = haar2d<TILE, 1>(yu, sm.hs, i0, j0, d.nx + 1, d.ny, levels);
  yv = haar2d<TILE, 1>(yv, sm.hs, i0, j0, d.nx, d.ny + 1, levels);
  cu = (inu && wmask[uidx(d, i, j)]) ? yu : (T)0;
  cv = (inv && wmask[vidx(d, i, j)]) ? yv : (T)0;
}

// w = inner ⊙ P u at this thread's point; written to global memory.
template <typename T, int TILE>
__device__ __forceinline__ void prolong_store(const Dims& d, int levels, const uint8_t* __restrict__ inner, T uu, T uv,
                                              int i0, int j0, CGShared<T, TILE>& sm, T* __restrict__ w) {
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
  const T pu = haar2d<TILE, 0>(uu, sm.hs, i0, j0, d.nx + 1, d.ny, levels);
  const T pv = haar2d<TILE, 0>(uv, sm.hs, i0, j0, d.nx, d.ny + 1, levels);
  if (inu) {
    const int q = uidx(d, i, j);
    __stcg(w + q, inner[q] ? pu : (T)0);
  }
  if (inv) {
    const int q = vidx(d, i, j);
    __stcg(w + q, inner[q] ? pv : (T)0);
  }
}

// The whole coarse CG of one V-cycle: from the warm start xc and right-hand side bc (both global, full
// layout) to the final xc.  Writes the CG statistics into st (CTA 0).
template <typename T, int TILE, int MAXT>
__global__ void __launch_bounds__(TILE* TILE)
    k_cg_persistent(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, T* __restrict__ w,
                    const T* __restrict__ bc, T* __restrict__ xc, double* __restrict__ partials, DevState* st,
                    const DevParams* __restrict__ P, GridBar* bar, int ntx, int nty) {
  __shared__ CGShared<T, TILE> sm;
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y;
  T xu[MAXT], xv[MAXT], ru[MAXT], rv[MAXT], uu[MAXT], uv[MAXT], cu[MAXT], cv[MAXT];
  int i0s[MAXT], j0s[MAXT];
  bool own[MAXT];
#pragma unroll
  for (int k = 0; k < MAXT; ++k) {
    const int t = blockIdx.x + k * gridDim.x;
    own[k] = t < ntiles;
    i0s[k] = own[k] ? (t % ntx) * TILE : 0;
    j0s[k] = own[k] ? (t / ntx) * TILE : 0;
    const int i = i0s[k] + tx, j = j0s[k] + ty;
    xu[k] = (own[k] && i <= d.nx && j < d.ny) ? xc[uidx(d, i, j)] : (T)0;
    xv[k] = (own[k] && i < d.nx && j <= d.ny) ? xc[vidx(d, i, j)] : (T)0;
    uu[k] = uv[k] = cu[k] = cv[k] = ru[k] = rv[k] = (T)0;
  }
  double sums[2];
  // start: w = P xc
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) prolong_store<T, TILE>(d, levels, cf.inner, xu[k], xv[k], i0s[k], j0s[k], sm, w);
  if (!grid_barrier<false>(bar, partials, 0, 0, sums)) return;
  // r = b_c - R A P xc, u = 0;  |r|^2 and |b_c|^2
  double a0 = 0.0, a1 = 0.0;
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) {
      coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0s[k], j0s[k], sm, cu[k], cv[k]);
      const int i = i0s[k] + tx, j = j0s[k] + ty;
      const T bu = (i <= d.nx && j < d.ny) ? bc[uidx(d, i, j)] : (T)0;
      const T bv = (i < d.nx && j <= d.ny) ? bc[vidx(d, i, j)] : (T)0;
      ru[k] = bu - cu[k];
      rv[k] = bv - cv[k];
      a0 += (double)ru[k] * (double)ru[k] + (double)rv[k] * (double)rv[k];
      a1 += (double)bu * (double)bu + (double)bv * (double)bv;
    }
  if (!grid_barrier<true>(bar, partials, a0, a1, sums)) return;
  double res = sqrt(sums[0]);
  const double tol = fmax(1.4901161193847656e-08 * res, P->tol_coarse * sqrt(sums[1]));  // reltol = sqrt(eps)
  double prev = 1.0;
  const int maxit = P->maxiter_coarse;
  int it = 0;
  bool done = (0 >= maxit) || res <= tol || !(res == res);
  while (!done) {
    const double beta = (res * res) / (prev * prev);
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        uu[k] = (T)((double)ru[k] + beta * (double)uu[k]);
        uv[k] = (T)((double)rv[k] + beta * (double)uv[k]);
        prolong_store<T, TILE>(d, levels, cf.inner, uu[k], uv[k], i0s[k], j0s[k], sm, w);
      }
    if (!grid_barrier<false>(bar, partials, 0, 0, sums)) return;
    double dot = 0.0;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0s[k], j0s[k], sm, cu[k], cv[k]);
        dot += (double)uu[k] * (double)cu[k] + (double)uv[k] * (double)cv[k];
      }
    if (!grid_barrier<true>(bar, partials, dot, 0.0, sums)) return;
    const double alpha = (res * res) / sums[0];
    double rr = 0.0;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        xu[k] = (T)((double)xu[k] + alpha * (double)uu[k]);
        xv[k] = (T)((double)xv[k] + alpha * (double)uv[k]);
        ru[k] = (T)((double)ru[k] - alpha * (double)cu[k]);
        rv[k] = (T)((double)rv[k] - alpha * (double)cv[k]);
        rr += (double)ru[k] * (double)ru[k] + (double)rv[k] * (double)rv[k];
      }
    if (!grid_barrier<true>(bar, partials, rr, 0.0, sums)) return;
    prev = res;
    res = sqrt(sums[0]);
    ++it;
    done = it >= maxit || res <= tol || !(res == res);
  }
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) {
      const int i = i0s[k] + tx, j = j0s[k] + ty;
      if (i <= d.nx && j < d.ny) xc[uidx(d, i, j)] = xu[k];
      if (i < d.nx && j <= d.ny) xc[vidx(d, i, j)] = xv[k];
    }
  if (blockIdx.x == 0 && tx == 0 && ty == 0) {
    st->cg_it = it;
    st->cg_total += it;
    st->cg_res = res;
    st->cg_prev = prev;
    st->cg_tol = tol;
  }
}

// Before a persistent CG: an idle barrier (count 0, no error).
static __global__ void k_reset_barrier(GridBar* bar) {
  if (threadIdx.x == 0) {
    bar->count = 0u;
    bar->err = 0;
  }
}

// After a persistent CG: turn a watchdog failure into the solve's status.
static __global__ void k_check_barrier(GridBar* bar, DevState* st, CondHandles h) {
  if (threadIdx.x == 0 && bar->err) {
    st->status = WAVI_ERR_WATCHDOG;
    st->picard_continue = 0;
    if (h.active) cudaGraphSetConditional(h.picard, 0);
  }
}

}  // namespace wavi
