// anderson.cuh — Anderson acceleration of the Picard loop (wavi_options.picard_accel =
// WAVI_PICARD_ANDERSON; not in the reference, whose update_velocities! (update_velocities.jl:11-29) takes
// each relinearised V-cycle correction as it is).
//
// Walker & Ni, "Anderson acceleration for fixed-point iterations", SIAM J. Numer. Anal. 49 (2011).  The
// fixed-point map is one Picard iteration, g(x) = x + V(x)(b(x) - A(x) x): relinearisation, residual and
// one V-cycle.  From the first Picard iteration whose relative residual is below start_rel, each
// iteration keeps f = V(x)(b - A x) (the V-cycle's correction) and g = x + f, stores the differences of
// consecutive f and g as one column of a ring of `depth` columns (dF, dG), and moves to
// x = g - dG gamma, gamma the least-squares solution of min |f - dF gamma|.  The normal equations are
// solved with the columns newest first by Cholesky; at the first pivot below kAAPivot of its diagonal
// entry (a column numerically in the span of the newer ones) that column and every older one are left
// out.  The stopping rule is untouched: the residual test of the next iteration decides on the
// accelerated iterate exactly as on a plain one, so a converged solve meets the reference's criterion.
//
// Two launches after k_vcycle_finish (which has made x = g):
//   k_aa_stage: the new column, f_prev / g_prev, the new Gram row and dF^T f (2 x depth FP64 dot
//               products, one last-block reduction), then thread 0 of the last block solves for gamma;
//   k_aa_apply: x = g - dG gamma on the interior (and into the velocity state), and ||dx|| / ||x|| for
//               the update test (picard_test = 1).
// Both return at once while the acceleration has not started.  FP64 throughout: the columns are
// differences of FP64 iterates (in a mixed context f is the FP32 V-cycle correction widened exactly).
#pragma once

#include "fused.cuh"

namespace wavi {

// Per-solve buffers: depth columns each of dF and dG, and f, g of the previous iteration (N doubles each).
struct AAWork {
  double* dF;     // [depth][N]
  double* dG;     // [depth][N]
  double* fprev;  // [N]
  double* gprev;  // [N]
  double* partials;  // [2 kAAMax][blocks]
};

// Every block contributes K values; the last block to finish gets the K totals, each summed over the
// blocks' partials in block order (deterministic), in tot[0..K) for thread 0, and returns true.  The K
// values go through one shuffle tree per warp each and one shared-memory pass (a single __syncthreads),
// and the last block sums each value's partials with one warp.
template <int K>
__device__ __forceinline__ bool last_block_sumk(const double (&v)[K], double* __restrict__ partials, unsigned* counter,
                                                double (&tot)[K]) {
  __shared__ double sw[32][K];
  __shared__ double stot[K];
  __shared__ int slast;
  const int t = flat_tid(), lane = t & 31, wid = t >> 5, nw = (flat_nthreads() + 31) >> 5;
  const int nb = flat_nblocks(), b = flat_bid();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double s = warp_sum(v[k]);
    if (lane == 0) sw[wid][k] = s;
  }
  __syncthreads();
  if (t < K) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += sw[w][t];
    partials[(size_t)t * nb + b] = s;
    __threadfence();
  }
  __syncthreads();
  if (t == 0) {
    const unsigned prev = atomicAdd(counter, 1u);
    slast = (prev == (unsigned)nb - 1u);
  }
  __syncthreads();
  if (!slast) return false;
  __threadfence();
  for (int k = wid; k < K; k += nw) {
    double a = 0.0;
    for (int q = lane; q < nb; q += 32) a += __ldcg(partials + (size_t)k * nb + q);
    a = warp_sum(a);
    if (lane == 0) stot[k] = a;
  }
  __syncthreads();
  if (t == 0) {
    for (int k = 0; k < K; ++k) tot[k] = stot[k];
    *counter = 0u;
  }
  return true;
}

// The least-squares step of the last block's thread 0: the newest-first Gram matrix from the slot-indexed
// one, Cholesky with the drop rule, gamma.  Returns the columns used.
__device__ __forceinline__ int aa_solve(AAState& a, int depth, const double* rhs) {
  int slot[kAAMax];
  for (int p = 0; p < a.cols; ++p) slot[p] = ((a.head - p) % depth + depth) % depth;  // a.head: the newest
  double L[kAAMax][kAAMax];
  int used = 0;
  for (int p = 0; p < a.cols; ++p) {
    for (int q = 0; q < p; ++q) {
      double s = a.gram[slot[p]][slot[q]];
      for (int k = 0; k < q; ++k) s -= L[p][k] * L[q][k];
      L[p][q] = s / L[q][q];
    }
    const double gpp = a.gram[slot[p]][slot[p]];
    double s = gpp;
    for (int k = 0; k < p; ++k) s -= L[p][k] * L[p][k];
    if (!(s > kAAPivot * gpp)) break;
    L[p][p] = sqrt(s);
    used = p + 1;
  }
  double y[kAAMax];
  for (int p = 0; p < used; ++p) {
    double s = rhs[p];
    for (int k = 0; k < p; ++k) s -= L[p][k] * y[k];
    y[p] = s / L[p][p];
  }
  for (int p = used - 1; p >= 0; --p) {
    double s = y[p];
    for (int k = p + 1; k < used; ++k) s -= L[k][p] * a.gamma[k];
    a.gamma[p] = s / L[p][p];
    a.slot[p] = slot[p];
  }
  return used;
}

template <typename T>
__global__ void __launch_bounds__(256) k_aa_stage(int n, const uint8_t* __restrict__ inner, const double* __restrict__ x,
                                                  const T* __restrict__ corr, AAWork w, DevState* st,
                                                  const DevParams* __restrict__ P) {
  const int depth = P->aa_depth;
  const bool started = st->aa.started || st->rel < P->aa_start_rel;
  if (!started || depth <= 0) return;  // the same decision in every block
  const bool have_prev = st->aa.have_prev != 0;
  const int newest = have_prev ? (st->aa.cols == 0 ? 0 : (st->aa.head + 1) % depth) : 0;
  const int ncols = have_prev ? min(st->aa.cols + 1, depth) : 0;
  // fixed-bound loops with guards keep slot[] and v[] in registers (no dynamic indexing)
  int slot[kAAMax];
#pragma unroll
  for (int p = 0; p < kAAMax; ++p) slot[p] = p < ncols ? ((newest - p) % depth + depth) % depth : 0;
  double v[2 * kAAMax];
#pragma unroll
  for (int k = 0; k < 2 * kAAMax; ++k) v[k] = 0.0;
  const size_t N = (size_t)n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const bool in = inner[k] != 0;  // the unknowns; f, g and the columns are zero elsewhere
    const double f = in ? (double)corr[k] : 0.0, g = in ? x[k] : 0.0;
    if (have_prev) {
      const double cf = f - w.fprev[k], cg = g - w.gprev[k];
      w.dF[(size_t)newest * N + k] = cf;
      w.dG[(size_t)newest * N + k] = cg;
      v[0] += cf * cf;
      v[kAAMax] += cf * f;
#pragma unroll
      for (int p = 1; p < kAAMax; ++p)
        if (p < ncols) {
          const double o = w.dF[(size_t)slot[p] * N + k];
          v[p] += cf * o;
          v[kAAMax + p] += o * f;
        }
    }
    w.fprev[k] = f;
    w.gprev[k] = g;
  }
  double tot[2 * kAAMax];
  if (last_block_sumk<2 * kAAMax>(v, w.partials, &st->counter[CNT_AA_STAGE], tot)) {
    if (flat_tid() == 0) {
      AAState& a = st->aa;
      a.started = 1;
      a.used = 0;
      if (have_prev) {
        for (int p = 0; p < ncols; ++p) a.gram[newest][slot[p]] = a.gram[slot[p]][newest] = tot[p];
        a.head = newest;
        a.cols = ncols;
        a.used = aa_solve(a, depth, tot + kAAMax);
        if (a.used > 0) a.steps++;
      }
      a.have_prev = 1;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_aa_apply(int n, const uint8_t* __restrict__ inner, double* __restrict__ x,
                                                  const T* __restrict__ corr, AAWork w, double* __restrict__ uv,
                                                  DevState* st, const DevParams* __restrict__ P) {
  if (P->aa_depth <= 0 || !st->aa.started || st->aa.used == 0) return;  // the same decision in every block
  const int used = st->aa.used;
  double gam[kAAMax];
  const double* col[kAAMax];
#pragma unroll
  for (int p = 0; p < kAAMax; ++p) {
    gam[p] = p < used ? st->aa.gamma[p] : 0.0;
    col[p] = w.dG + (size_t)(p < used ? st->aa.slot[p] : 0) * (size_t)n;
  }
  double v[2] = {0.0, 0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    if (!inner[k]) continue;
    double xn = x[k], dx = (double)corr[k];
#pragma unroll
    for (int p = 0; p < kAAMax; ++p)
      if (p < used) {
        const double c = gam[p] * col[p][k];
        xn -= c;
        dx -= c;
      }
    x[k] = xn;
    uv[k] = xn;
    v[0] += dx * dx;
    v[1] += xn * xn;
  }
  double tot[2];
  if (last_block_sumk<2>(v, w.partials, &st->counter[CNT_AA_APPLY], tot)) {
    if (flat_tid() == 0) {
      st->du2 = tot[0];
      st->uu2 = tot[1];
      st->rel_update = sqrt(tot[0]) / sqrt(tot[1]);
    }
  }
}

}  // namespace wavi
