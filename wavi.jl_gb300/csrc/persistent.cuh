// persistent.cuh — the coarse conjugate-gradient solve of one V-cycle as a single persistent kernel,
// and the smoother pass as another.
//
// The coarse solve (IterativeSolvers cg! on R A P, update_preconditioners.jl:54-83) is a long chain of
// small dependent steps: at 640 x 80 one iteration moves ~1 MB, far below what a launch costs.  Here one
// cooperative launch runs every iteration.  Each CTA owns up to MAXT tiles of TILE x TILE points (a tile
// holds whole Haar blocks of both velocity components); each thread keeps, in registers, the CG vectors
// of its own point of every owned tile for the whole solve.  Per operator application only a prolonged
// vector w = P u crosses L2 (the operator needs a one-point halo of it).  Two kernels:
//
//   k_cg_persistent   the reference's cg! recurrence: u = r + β u; w = P u; c = R A w; <u, c>;
//                     α; x, r; |r|^2 — two grid reductions per iteration
//   k_srcg_persistent single-reduction CG (Chronopoulos & Gear 1989), preconditioned by nothing, by
//                     the Jacobi diagonal, or by Chebyshev-accelerated Jacobi steps: both inner products
//                     of an iteration follow its operator application, one grid reduction per iteration
//   k_pcg_persistent  pipelined CG with the Chebyshev preconditioner, restarted from the true residual
//                     after every hundredfold fall of |r| (FP32 fast path only; opt-in): the grid
//                     reduction of an iteration completes while its preconditioner and operator run
//
// The FP64 and global-memory instantiations separate the prolongation from the operator by a grid
// barrier.  The FP32 instantiations on 16 x 16 tiles (the fast path) keep the tiles' coefficients in
// shared memory, transform u and v together (idwt2d_pair, idwt2dT_pair), exchange only tile boundaries
// through tagged words that the neighbours wait for (stage_tagged), and carry the grid reductions and
// CG scalars in float-float arithmetic (GB300 executes FP64 at a small fraction of its FP32 rate).
// k_smooth_persistent runs a smoother pass on the same machinery.
//
// Grid sums are deterministic and identical in every CTA: each CTA publishes its partials, and after
// the barrier every CTA adds all partials in the same fixed order.  Every wait is bounded: after ~2^22
// polls a CTA records WAVI_ERR_WATCHDOG and all CTAs leave the kernel.
#pragma once
#include <type_traits>

#include "fused.cuh"

namespace wavi {

struct GridBar {
  unsigned count;  // arrivals since the launch began (monotonic; epoch e is complete at e * gridDim.x)
  unsigned gen;    // launch generation: the tags of the FP32 kernels' tagged words (advanced before each launch)
  int err;
  int pad;
  double sum[4];
};

constexpr long kBarrierSpinLimit = 1L << 22;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// Tagged words of the FP32 register-resident kernels: a 32-bit value and the 32-bit tag of the exchange
// that wrote it, in one naturally aligned 64-bit word (single-copy atomic), so a reader that sees the
// expected tag sees that exchange's value.  Writers store relaxed and need no fence: a word is rewritten
// only after its readers have consumed it (the kernel's reductions order that).
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" : : "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long tagged(unsigned tag, float x) {
  return ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(x);
}
__device__ __forceinline__ unsigned tag_of(unsigned long long w) { return (unsigned)(w >> 32); }
__device__ __forceinline__ float value_of(unsigned long long w) { return __uint_as_float((unsigned)w); }

// ------------------------------------------------------------------------------------------------
// Float-float arithmetic for the FP32 kernels' reductions and CG scalars.  GB300 executes FP64 at a
// small fraction of its FP32 rate (a warp's FP64 instruction costs tens of cycles, with one lane active
// or all), and the grid sums and scalar recurrences are serial chains on every CG iteration's critical
// path.  A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2 (~48-bit
// significand), built from Knuth's TwoSum and the FMA TwoProduct (Dekker 1971; the double-double
// algorithms of Hida, Li & Bailey 2001 carried over to floats).  The __f*_rn intrinsics keep the
// compiler from contracting the error terms into FMAs.  The range is float's, as for the FP32 kernels'
// per-thread products.
// ------------------------------------------------------------------------------------------------
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff ff_quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff operator+(ff x, ff y) {
  ff s = ff_two_sum(x.hi, y.hi);
  const ff t = ff_two_sum(x.lo, y.lo);
  s = ff_quick_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return ff_quick_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ ff operator-(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff operator-(ff x, ff y) { return x + (-y); }
__device__ __forceinline__ ff operator*(ff x, ff y) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p)));
  return ff_quick_two_sum(p, e);
}
__device__ __forceinline__ ff operator/(ff x, ff y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const ff r = x - y * ff{q1, 0.0f};
  return ff_quick_two_sum(q1, __fdiv_rn(r.hi, y.hi));
}
__device__ __forceinline__ bool operator<=(ff x, ff y) { return x.hi < y.hi || (x.hi == y.hi && x.lo <= y.lo); }
__device__ __forceinline__ ff ff_of(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double dbl_of(ff v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ double dbl_of(double v) { return v; }

// The type in which a kernel of vector type T sums its grid reductions and keeps its CG scalars.
template <typename T>
struct CGReal {
  using type = double;
};
template <>
struct CGReal<float> {
  using type = ff;
};
__device__ __forceinline__ double real_term(double x) { return x; }
__device__ __forceinline__ ff real_term(float x) { return {x, 0.0f}; }
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ ff shfl_xor(ff v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ ff ld_cg(const ff* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}

// Shared memory of the grid synchronisation.
struct SyncShared {
  double warp[32][4];  // warp sums (CGReal of the kernel's vector type: double, or ff in the same 8 bytes)
  double tot[4];       // grid totals (the same type)
  int ok;
};

// Grid-wide barrier over gridDim.x CTAs.  v[0..NS) are this thread's terms (type A: float or double);
// they are summed over the warp and the CTA in A, over the grid in S = CGReal<A> (double, or float-float
// for float), and after the barrier tot[0..NS) (type S, in shared memory) hold the grid sums and
// `scalars(tot)` has run in thread 0 (it derives the CG scalars once per CTA); the barrier ends with a
// __syncthreads, so its results are visible to the whole CTA.  `epoch` counts this thread's barriers
// since the launch (the same in every thread); partials holds 2 x 4 x gridDim.x 8-byte slots (the two
// parities of the epoch, so a slot is rewritten only after every CTA has read it).  Arrival is a
// red.release by thread 0 after the CTA barrier (release is cumulative: it publishes the CTA's stores
// ordered before it by the __syncthreads); the wait is an ld.acquire poll followed by a __syncthreads.
// Returns false (in every thread of the CTA) if the wait gave up or another CTA reported an error.
template <int NS, typename A, typename F>
__device__ __forceinline__ bool grid_sync(GridBar* bar, double* __restrict__ partials, unsigned& epoch, SyncShared& ss,
                                          const A (&v)[4], F&& scalars) {
  using S = typename CGReal<A>::type;
  static_assert(sizeof(S) == sizeof(double), "partial slots are 8 bytes");
  const int t = flat_tid(), lane = t & 31, wid = t >> 5, nw = (flat_nthreads() + 31) >> 5;
  const unsigned nb = gridDim.x;
  ++epoch;
  S* slot = reinterpret_cast<S*>(partials + (size_t)(epoch & 1u) * 4u * nb);
  S(*wsum)[4] = reinterpret_cast<S(*)[4]>(ss.warp);
  S* tot = reinterpret_cast<S*>(ss.tot);
  if (NS > 0) {
    A x[4];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      x[q] = v[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x[q] += __shfl_xor_sync(0xffffffffu, x[q], o);
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < NS; ++q) wsum[wid][q] = real_term(x[q]);
  }
  __syncthreads();  // the CTA's writes (halo vector, warp sums) precede the arrival
  if (wid == 0 && NS > 0) {
    // lane l adds the sums of warps l/4, l/4 + 8, ... for quantity l%4, then a butterfly over the lanes
    // of equal l%4 (the same order in every CTA)
    const int q = lane & 3;
    S s{};
    if constexpr (std::is_same<A, float>::value) {
      // FP32 kernels: the CTA's eight warp sums in FP32 as well (float-float from the CTA partials on;
      // measured 1.7 % faster per solve than a float-float CTA sum)
      float f = 0.f;
      if (q < NS)
        for (int k = lane >> 2; k < nw; k += 8) f += wsum[k][q].hi;
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
      s = real_term(f);
    } else {
      if (q < NS)
        for (int k = lane >> 2; k < nw; k += 8) s = s + wsum[k][q];
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) s = s + shfl_xor(s, o);
    }
    if (lane < NS) slot[lane * nb + blockIdx.x] = s;
    __syncwarp();
  }
  if (t == 0) {
    red_release_add_u32(&bar->count, 1u);
    const unsigned target = epoch * nb;
    int ok = 1;
    long polls = 0;
    while ((int)(ld_acquire_u32(&bar->count) - target) < 0) {
      if (++polls > kBarrierSpinLimit || ((polls & 255) == 0 && *(volatile int*)&bar->err)) {
        ok = 0;
        break;
      }
      if (polls > 8) __nanosleep(32);
    }
    if (!ok) atomicExch(&bar->err, 1);
    ss.ok = ok;
  }
  __syncthreads();
  if (!ss.ok) return false;
  if (NS > 0) {
    // warp q adds partial q of every CTA: eight slots per lane and round, added as a tree, then a
    // butterfly (a fixed order, so every CTA obtains the same bits)
    if (wid < NS) {
      const S* src = slot + wid * nb;
      S s{};
      for (unsigned k0 = 0; k0 < nb; k0 += 256) {
        S b[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const unsigned k = k0 + lane + 32u * e;
          b[e] = k < nb ? ld_cg(src + k) : S{};
        }
        s = s + (((b[0] + b[1]) + (b[2] + b[3])) + ((b[4] + b[5]) + (b[6] + b[7])));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s = s + shfl_xor(s, o);
      if (lane == 0) tot[wid] = s;
    }
    __syncthreads();
    if (t == 0) scalars(static_cast<const S*>(tot));
    __syncthreads();
  }
  return true;
}

// grid_sync in two halves, for a kernel with work to do while the grid sum completes (k_pcg_persistent):
// grid_arrive publishes this CTA's partials and arrives, as the first half of grid_sync does; grid_wait
// waits for every CTA's arrival, adds the partials and runs `scalars` in thread 0, as the second half
// does, and ends with a __syncthreads.  Between the halves a CTA may exchange tagged words with its
// neighbours, but it starts no other grid reduction or barrier and leaves ss alone.  The parity argument
// of grid_sync holds unchanged: a CTA reaches the arrival of epoch e + 2 only after the wait of e + 1,
// which needs every CTA's arrival at e + 1, which each CTA makes after its own wait of e.
template <int NS, typename A>
__device__ __forceinline__ void grid_arrive(GridBar* bar, double* __restrict__ partials, unsigned& epoch, SyncShared& ss,
                                            const A (&v)[4]) {
  using S = typename CGReal<A>::type;
  static_assert(sizeof(S) == sizeof(double), "partial slots are 8 bytes");
  const int t = flat_tid(), lane = t & 31, wid = t >> 5, nw = (flat_nthreads() + 31) >> 5;
  const unsigned nb = gridDim.x;
  ++epoch;
  S* slot = reinterpret_cast<S*>(partials + (size_t)(epoch & 1u) * 4u * nb);
  S(*wsum)[4] = reinterpret_cast<S(*)[4]>(ss.warp);
  if (NS > 0) {
    A x[4];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      x[q] = v[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x[q] += __shfl_xor_sync(0xffffffffu, x[q], o);
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < NS; ++q) wsum[wid][q] = real_term(x[q]);
  }
  __syncthreads();
  if (wid == 0 && NS > 0) {
    const int q = lane & 3;
    S s{};
    if constexpr (std::is_same<A, float>::value) {
      float f = 0.f;
      if (q < NS)
        for (int k = lane >> 2; k < nw; k += 8) f += wsum[k][q].hi;
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
      s = real_term(f);
    } else {
      if (q < NS)
        for (int k = lane >> 2; k < nw; k += 8) s = s + wsum[k][q];
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) s = s + shfl_xor(s, o);
    }
    if (lane < NS) slot[lane * nb + blockIdx.x] = s;
    __syncwarp();
  }
  if (t == 0) red_release_add_u32(&bar->count, 1u);
}
template <int NS, typename A, typename F>
__device__ __forceinline__ bool grid_wait(GridBar* bar, double* __restrict__ partials, unsigned epoch, SyncShared& ss,
                                          F&& scalars) {
  using S = typename CGReal<A>::type;
  const int t = flat_tid(), lane = t & 31, wid = t >> 5;
  const unsigned nb = gridDim.x;
  const S* slot = reinterpret_cast<const S*>(partials + (size_t)(epoch & 1u) * 4u * nb);
  S* tot = reinterpret_cast<S*>(ss.tot);
  if (t == 0) {
    const unsigned target = epoch * nb;
    int ok = 1;
    long polls = 0;
    while ((int)(ld_acquire_u32(&bar->count) - target) < 0) {
      if (++polls > kBarrierSpinLimit || ((polls & 255) == 0 && *(volatile int*)&bar->err)) {
        ok = 0;
        break;
      }
      if (polls > 8) __nanosleep(32);
    }
    if (!ok) atomicExch(&bar->err, 1);
    ss.ok = ok;
  }
  __syncthreads();
  if (!ss.ok) return false;
  if (NS > 0) {
    if (wid < NS) {
      const S* src = slot + wid * nb;
      S s{};
      for (unsigned k0 = 0; k0 < nb; k0 += 256) {
        S b[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const unsigned k = k0 + lane + 32u * e;
          b[e] = k < nb ? ld_cg(src + k) : S{};
        }
        s = s + (((b[0] + b[1]) + (b[2] + b[3])) + ((b[4] + b[5]) + (b[6] + b[7])));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s = s + shfl_xor(s, o);
      if (lane == 0) tot[wid] = s;
    }
    __syncthreads();
    if (t == 0) scalars(static_cast<const S*>(tot));
    __syncthreads();
  }
  return true;
}

template <typename A>
__device__ __forceinline__ bool grid_barrier(GridBar* bar, double* __restrict__ partials, unsigned& epoch, SyncShared& ss) {
  const A v[4] = {A(0), A(0), A(0), A(0)};
  return grid_sync<0>(bar, partials, epoch, ss, v, [](const typename CGReal<A>::type*) {});
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

// P on a TILE x TILE tile, u and v together: the idwt lifting (haar_tile KIND 0) along y, then along x,
// written as a gather.  The output at in-block position j is the block's scaling coefficient plus, per
// level l (half = B >> (l + 1)), minus or plus the detail coefficient at (j rounded down to 2 half) + half:
// plus when j lies in the upper half of its pair.  These are the lifting's additions in the same order,
// so the result is the lifting's; positions off the grid hold zeros, which stands for the steps the
// lifting skips at a ragged edge.  Along y the terms come from shared memory, along x by shuffles within
// the row's lanes.  One __syncthreads (after the shared-memory writes; a leading one protects the buffers).
template <int TILE, typename TT>
__device__ __forceinline__ void idwt2d_pair(TT& u, TT& v, TT (*su)[TILE + 1], TT (*sv)[TILE + 1], int levels) {
  constexpr int MAXL = TILE == 16 ? 4 : 5;  // levels + 1 <= log2(TILE)
  const int tx = threadIdx.x, ty = threadIdx.y, B = 1 << (levels + 1);
  __syncthreads();
  su[ty][tx] = u;
  sv[ty][tx] = v;
  __syncthreads();
  TT au = su[ty & ~(B - 1)][tx], av = sv[ty & ~(B - 1)][tx];
#pragma unroll
  for (int l = 0; l < MAXL; ++l)
    if (l <= levels) {
      const int half = B >> (l + 1), q = (ty & ~(2 * half - 1)) + half;
      const TT pu = su[q][tx], pv = sv[q][tx];
      if (ty & half) {
        au = pu + au;
        av = pv + av;
      } else {
        au = au - pu;
        av = av - pv;
      }
    }
  const int row0 = ((tx + TILE * ty) & 31) - tx;  // lane of the row's element 0
  TT bu = __shfl_sync(0xffffffffu, au, row0 + (tx & ~(B - 1)));
  TT bv = __shfl_sync(0xffffffffu, av, row0 + (tx & ~(B - 1)));
#pragma unroll
  for (int l = 0; l < MAXL; ++l) {
    const int half = B >> (l + 1), q = (tx & ~(2 * half - 1)) + half;
    const TT pu = __shfl_sync(0xffffffffu, au, row0 + q), pv = __shfl_sync(0xffffffffu, av, row0 + q);
    if (l <= levels) {
      if (tx & half) {
        bu = pu + bu;
        bv = pv + bv;
      } else {
        bu = bu - pu;
        bv = bv - pv;
      }
    }
  }
  u = bu;
  v = bv;
}

// Sum of m (a power of two <= MAXM) consecutive entries of column col from row r0, as a pairwise tree
// (the order in which the idwtᵀ lifting accumulates them); absent entries are zeros.
template <int MAXM, int TILE, typename TT>
__device__ __forceinline__ TT column_tree_sum(const TT (*s)[TILE + 1], int r0, int m, int col) {
  TT a[MAXM];
#pragma unroll
  for (int k = 0; k < MAXM; ++k) a[k] = k < m ? s[r0 + k][col] : (TT)0;
#pragma unroll
  for (int w = 1; w < MAXM; w <<= 1)
#pragma unroll
    for (int k = 0; k < MAXM; k += 2 * w) a[k] = a[k] + a[k + w];
  return a[0];
}

// Pᵀ (= R) on a TILE x TILE tile, u and v together: the idwtᵀ lifting (haar_tile KIND 1) along y, then
// along x.  Along y each output is a difference of two tree sums of its column (upper half minus lower
// half of its pair at its own level; the scaling coefficient is the sum of both halves of the block),
// read from shared memory; along x the lifting runs on the row's lanes with shuffles.  Inputs off the
// grid must be zero (they stand for the partners the lifting skips at a ragged edge).
template <int TILE, typename TT>
__device__ __forceinline__ void idwt2dT_pair(TT& u, TT& v, TT (*su)[TILE + 1], TT (*sv)[TILE + 1], int levels) {
  constexpr int MAXL = TILE == 16 ? 4 : 5;
  const int tx = threadIdx.x, ty = threadIdx.y, B = 1 << (levels + 1);
  __syncthreads();
  su[ty][tx] = u;
  sv[ty][tx] = v;
  __syncthreads();
  const int jj = ty & (B - 1);
  const int m = jj == 0 ? (B >> 1) : (jj & -jj);
  const int r0 = jj == 0 ? ty : ty - m;
  const TT fu = column_tree_sum<TILE / 2, TILE>(su, r0, m, tx), gu = column_tree_sum<TILE / 2, TILE>(su, r0 + m, m, tx);
  const TT fv = column_tree_sum<TILE / 2, TILE>(sv, r0, m, tx), gv = column_tree_sum<TILE / 2, TILE>(sv, r0 + m, m, tx);
  TT bu = jj == 0 ? fu + gu : gu - fu, bv = jj == 0 ? fv + gv : gv - fv;
#pragma unroll
  for (int l = 0; l < MAXL; ++l)
    if (l <= levels) {
      const int half = 1 << l;
      const TT pu = __shfl_xor_sync(0xffffffffu, bu, half), pv = __shfl_xor_sync(0xffffffffu, bv, half);
      const int r = tx & (2 * half - 1);
      if (r == 0) {
        bu = bu + pu;
        bv = bv + pv;
      } else if (r == half) {
        bu = bu - pu;
        bv = bv - pv;
      }
    }
  u = bu;
  v = bv;
}

template <typename T, int TILE>
struct CGShared {
  OpTile<T, TILE, TILE> op;
  T hs[TILE][TILE + 1];
  T hs2[std::is_same<T, float>::value ? TILE : 1][TILE + 1];  // FP32: the second buffer of the paired transforms
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
  if constexpr (std::is_same<T, float>::value) {
    idwt2dT_pair<TILE>(yu, yv, sm.hs, sm.hs2, levels);
  } else {
    yu = haar2d<TILE, 1>(yu, sm.hs, i0, j0, d.nx + 1, d.ny, levels);
    yv = haar2d<TILE, 1>(yv, sm.hs, i0, j0, d.nx, d.ny + 1, levels);
  }
  cu = (inu && wmask[uidx(d, i, j)]) ? yu : (T)0;
  cv = (inv && wmask[vidx(d, i, j)]) ? yv : (T)0;
}

// w = inner ⊙ P u at this thread's point; written to global memory.
template <typename T, int TILE>
__device__ __forceinline__ void prolong_store(const Dims& d, int levels, const uint8_t* __restrict__ inner, T uu, T uv,
                                              int i0, int j0, CGShared<T, TILE>& sm, T* __restrict__ w) {
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
  T pu, pv;
  if constexpr (std::is_same<T, float>::value) {
    pu = inu ? uu : (T)0;
    pv = inv ? uv : (T)0;
    idwt2d_pair<TILE>(pu, pv, sm.hs, sm.hs2, levels);
  } else {
    pu = haar2d<TILE, 0>(uu, sm.hs, i0, j0, d.nx + 1, d.ny, levels);
    pv = haar2d<TILE, 0>(uv, sm.hs, i0, j0, d.nx, d.ny + 1, levels);
  }
  if (inu) {
    const int q = uidx(d, i, j);
    __stcg(w + q, inner[q] ? pu : (T)0);
  }
  if (inv) {
    const int q = vidx(d, i, j);
    __stcg(w + q, inner[q] ? pv : (T)0);
  }
}

// ------------------------------------------------------------------------------------------------
// The FP32 register-resident kernels (TILE = 16) keep the operator's coefficients on chip for the whole
// launch and transform u and v together.
//
// CoefTile: the coefficients that the tile's stress stage reads (h cells and c points of the tile and
// its one-cell halo, h_m at the u and v points around them), staged once per launch in shared memory;
// PointCoef: the thread's own point (β, h_m and the inner / coarse-space flags) in registers.  Per CG
// iteration the operator then reads only the prolonged vector from L2.
// ------------------------------------------------------------------------------------------------
template <typename T, int TILE>
struct CoefTile {
  T he2[TILE + 1][TILE + 1];  // 2 hη at h cell (i0 - 1 + a, j0 - 1 + b); 0 off the grid
  T dm[TILE + 1][TILE + 1];   // dimp at the h cells
  T hc[TILE + 1][TILE + 1];   // hη_c at c point (i0 - 1 + a, j0 - 1 + b)
  T hmu[TILE + 1][TILE + 2];  // h_m at u point (i0 - 1 + a, j0 - 1 + b)
  T hmv[TILE + 2][TILE + 1];  // h_m at v point (i0 - 1 + a, j0 - 1 + b)
};
template <typename T>
struct PointCoef {
  T beta_u, beta_v, hm_u, hm_v;
  bool inu, inv, inner_u, inner_v, wm_u, wm_v;  // on the grid; interior; in the coarse space
};

template <typename T, int TILE>
__device__ __forceinline__ void load_coef_tile(const Dims& d, const OpCoef<T>& cf, const uint8_t* __restrict__ wmask,
                                               int i0, int j0, CoefTile<T, TILE>& ct, PointCoef<T>& pc) {
  for (int p = flat_tid(); p < (TILE + 1) * (TILE + 1); p += flat_nthreads()) {
    const int la = p % (TILE + 1), lb = p / (TILE + 1), a = i0 - 1 + la, b = j0 - 1 + lb;
    const bool hin = a >= 0 && a < d.nx && b >= 0 && b < d.ny;
    ct.he2[lb][la] = hin ? (T)2 * cf.heta_h[hidx(d, a, b)] : (T)0;
    ct.dm[lb][la] = hin ? cf.dimp[hidx(d, a, b)] : (T)0;
    ct.hc[lb][la] = (a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1) ? cf.heta_c[cidx(d, a, b)] : (T)0;
  }
  for (int p = flat_tid(); p < (TILE + 1) * (TILE + 2); p += flat_nthreads()) {
    const int la = p % (TILE + 2), lb = p / (TILE + 2), a = i0 - 1 + la, b = j0 - 1 + lb;
    ct.hmu[lb][la] = (a >= 0 && a <= d.nx && b >= 0 && b < d.ny) ? cf.h_m[uidx(d, a, b)] : (T)0;
  }
  for (int p = flat_tid(); p < (TILE + 2) * (TILE + 1); p += flat_nthreads()) {
    const int la = p % (TILE + 1), lb = p / (TILE + 1), a = i0 - 1 + la, b = j0 - 1 + lb;
    ct.hmv[lb][la] = (a >= 0 && a < d.nx && b >= 0 && b <= d.ny) ? cf.h_m[vidx(d, a, b)] : (T)0;
  }
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  pc.inu = i <= d.nx && j < d.ny;
  pc.inv = i < d.nx && j <= d.ny;
  const int qu = pc.inu ? uidx(d, i, j) : 0, qv = pc.inv ? vidx(d, i, j) : 0;
  pc.beta_u = pc.inu ? cf.beta_m[qu] : (T)0;
  pc.hm_u = pc.inu ? cf.h_m[qu] : (T)0;
  pc.inner_u = pc.inu && cf.inner[qu];
  pc.wm_u = pc.inu && wmask[qu];
  pc.beta_v = pc.inv ? cf.beta_m[qv] : (T)0;
  pc.hm_v = pc.inv ? cf.h_m[qv] : (T)0;
  pc.inner_v = pc.inv && cf.inner[qv];
  pc.wm_v = pc.inv && wmask[qv];
}

// One stress cell (la, lb) of stage_stress with the coefficients from the CoefTile (the same operations).
template <typename T, int TX, int TY, int TILE>
__device__ __forceinline__ void stress_cell_ct(const Dims& d, const CoefTile<T, TILE>& ct, int i0, int j0,
                                               OpTile<T, TX, TY>& s, int la, int lb) {
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  const int a = i0 - 1 + la, b = j0 - 1 + lb;
  T rxx = 0, ryy = 0, e = 0, rxy = 0;
  if (a >= 0 && a < d.nx && b >= 0 && b < d.ny) {
    const T u0 = s.xu[lb][la], u1 = s.xu[lb][la + 1], v0 = s.xv[lb][la], v1 = s.xv[lb + 1][la];
    const T ux = (u1 - u0) * rdx, vy = (v1 - v0) * rdy;
    const T he2 = ct.he2[lb][la];
    rxx = he2 * ((T)2 * ux + vy);
    ryy = he2 * ((T)2 * vy + ux);
    const T dm = ct.dm[lb][la];
    if (dm != (T)0) {
      const T divq = (ct.hmu[lb][la + 1] * u1 - ct.hmu[lb][la] * u0) * rdx +
                     (ct.hmv[lb + 1][la] * v1 - ct.hmv[lb][la] * v0) * rdy;
      e = dm * divq;
    }
  }
  if (a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1) {
    const T hc = ct.hc[lb][la];
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

// Tagged halo exchange of the FP32 register-resident kernels.  The prolonged vector of a tile never
// leaves the chip except its boundary: each tile publishes its first/last column and row (u and v) as
// tagged words in its halo box, and a tile's operator reads its one-point halo ring from the neighbours'
// boxes, waiting (bounded) for the current exchange's tag.  No grid barrier and no fence separate the
// prolongation from the operator, and a CTA waits only for its neighbours.  Ordering: a tile rewrites its
// box only after the next grid reduction, which needs every CTA's partial, computed from the halo values
// it read.  Tags are (gen << 21) + exchange, gen advanced by k_reset_barrier before each launch past the
// previous launch's range, so no word left by an earlier launch carries a current tag.  (Tagged words
// for the reductions as well, every CTA polling every CTA's partial, were measured slower than the
// counter barrier: the polls crowd the few L2 lines that the partials occupy.)
struct TagState {
  unsigned long long* halo;  // [parity][tile][u, v][west column, east column, south row, north row][TILE]
  unsigned base;             // gen << 21
  unsigned hx;               // exchanges so far in this launch
  size_t parity_stride;      // words per parity (0: one box set, the coarse CG's; its reductions order the rewrites)
  __device__ __forceinline__ unsigned long long* box(int tile, int TILE) const {
    return halo + (size_t)(hx & 1u) * parity_stride + (size_t)tile * (8 * TILE);
  }
};

// Bounded wait for a tagged word.  On a timeout (or another CTA's error) sets fail and bar->err.
__device__ __forceinline__ unsigned long long wait_tagged(const unsigned long long* p, unsigned tag, GridBar* bar,
                                                          volatile int* fail) {
  unsigned long long w = ld_relaxed_u64(p);
  long polls = 0;
  while (tag_of(w) != tag) {
    if (++polls > kBarrierSpinLimit || ((polls & 255) == 0 && *(volatile int*)&bar->err)) {
      *fail = 1;
      atomicExch(&bar->err, 1);
      break;
    }
    if (polls > 8) __nanosleep(32);
    w = ld_relaxed_u64(p);
  }
  return w;
}

// The tile's boundary values (this thread's hu, hv if it lies on the first/last row or column) as
// tagged words of exchange ts.hx.
template <typename T, int TILE>
__device__ __forceinline__ void publish_boundary(T hu, T hv, int tile, const TagState& ts) {
  const unsigned tag = ts.base + ts.hx;
  unsigned long long* box = ts.box(tile, TILE);
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (tx == 0) {
    st_relaxed_u64(box + 0 * TILE + ty, tagged(tag, hu));
    st_relaxed_u64(box + 4 * TILE + ty, tagged(tag, hv));
  }
  if (tx == TILE - 1) {
    st_relaxed_u64(box + 1 * TILE + ty, tagged(tag, hu));
    st_relaxed_u64(box + 5 * TILE + ty, tagged(tag, hv));
  }
  if (ty == 0) {
    st_relaxed_u64(box + 2 * TILE + tx, tagged(tag, hu));
    st_relaxed_u64(box + 6 * TILE + tx, tagged(tag, hv));
  }
  if (ty == TILE - 1) {
    st_relaxed_u64(box + 3 * TILE + tx, tagged(tag, hu));
    st_relaxed_u64(box + 7 * TILE + tx, tagged(tag, hv));
  }
}

// P on the tile (paired Haar transform); the prolonged values stay in the thread's registers (hu, hv:
// inner ⊙ P u, zero off the grid) and the tile's boundary is published for exchange ts.hx.
template <typename T, int TILE>
__device__ __forceinline__ void prolong_publish(int levels, const PointCoef<T>& pc, T uu, T uv, int tile,
                                                CGShared<T, TILE>& sm, T (*hs2)[TILE + 1], const TagState& ts, T& hu,
                                                T& hv) {
  T pu = pc.inu ? uu : (T)0, pv = pc.inv ? uv : (T)0;
  idwt2d_pair<TILE>(pu, pv, sm.hs, hs2, levels);
  hu = pc.inner_u ? pu : (T)0;
  hv = pc.inner_v ? pv : (T)0;
  publish_boundary<T, TILE>(hu, hv, tile, ts);
}

// The operator's staging on the fast path: the tile's x (this thread's hu, hv) into shared memory, its
// one-point halo ring from the neighbours' boxes of exchange ts.hx, and the stresses.  The ring loads are
// issued first and their tags checked after the 15 x 15 interior stress cells (which need no halo value),
// so that the L2 round trip overlaps them; then the 4 TILE boundary cells.  Returns false (in every
// thread) if a wait gave up.
template <typename T, int TILE>
__device__ __forceinline__ bool stage_tagged(const Dims& d, const CoefTile<T, TILE>& ct, T hu, T hv, int i0, int j0, int ntx,
                                             OpTile<T, TILE, TILE>& op, const TagState& ts, GridBar* bar,
                                             volatile int* fail) {
  constexpr int RING = 4 * TILE + 4;
  __syncthreads();  // the previous use of the tile's shared memory is over
  const int tx = threadIdx.x, ty = threadIdx.y, t = tx + TILE * ty;
  op.xu[ty + 1][tx + 1] = hu;
  op.xv[ty + 1][tx + 1] = hv;
  const unsigned tag = ts.base + ts.hx;
  const unsigned long long* src = nullptr;
  int li_r = 0, lj_r = 0, c_r = 0;
  unsigned long long w = 0;
  if (t < 2 * RING) {
    // ring position p: the row below (lj = 0), the row above (lj = TILE + 1), then the two columns
    c_r = t >= RING;
    const int p = t - c_r * RING;
    if (p < TILE + 2) {
      li_r = p;
      lj_r = 0;
    } else if (p < 2 * (TILE + 2)) {
      li_r = p - (TILE + 2);
      lj_r = TILE + 1;
    } else {
      const int q = p - 2 * (TILE + 2);
      li_r = (q & 1) ? TILE + 1 : 0;
      lj_r = 1 + (q >> 1);
    }
    const int i = i0 - 1 + li_r, j = j0 - 1 + lj_r;
    const bool on = c_r == 0 ? (i >= 0 && i <= d.nx && j >= 0 && j < d.ny) : (i >= 0 && i < d.nx && j >= 0 && j <= d.ny);
    if (on) {
      // the owning tile and the edge of its box that holds (i, j)
      const int ti = i / TILE, tj = j / TILE;
      const int e = li_r == 0 ? 1 : li_r == TILE + 1 ? 0 : lj_r == 0 ? 3 : 2;
      const int k = (li_r == 0 || li_r == TILE + 1) ? j - tj * TILE : i - ti * TILE;
      src = ts.box(tj * ntx + ti, TILE) + (c_r * 4 + e) * TILE + k;
      w = ld_relaxed_u64(src);
    }
  }
  __syncthreads();  // the interior of x is in shared memory
  for (int p = t; p < (TILE - 1) * (TILE - 1); p += TILE * TILE)
    stress_cell_ct(d, ct, i0, j0, op, 1 + p % (TILE - 1), 1 + p / (TILE - 1));
  if (t < 2 * RING) {
    T val = 0;
    if (src) {
      long polls = 0;
      while (tag_of(w) != tag) {
        if (++polls > kBarrierSpinLimit || ((polls & 255) == 0 && *(volatile int*)&bar->err)) {
          *fail = 1;
          atomicExch(&bar->err, 1);
          break;
        }
        if (polls > 8) __nanosleep(32);
        w = ld_relaxed_u64(src);
      }
      val = value_of(w);
    }
    if (c_r == 0)
      op.xu[lj_r][li_r] = val;
    else
      op.xv[lj_r][li_r] = val;
  }
  __syncthreads();
  if (*fail) return false;
  // the stress cells on the tile's boundary (17 x 17 - 15 x 15 = 4 TILE)
  if (t < 4 * TILE) {
    int la, lb;
    if (t < TILE + 1) {
      la = t;
      lb = 0;
    } else if (t < 2 * (TILE + 1)) {
      la = t - (TILE + 1);
      lb = TILE;
    } else {
      const int q = t - 2 * (TILE + 1);
      la = (q & 1) ? TILE : 0;
      lb = 1 + (q >> 1);
    }
    stress_cell_ct(d, ct, i0, j0, op, la, lb);
  }
  __syncthreads();
  return true;
}

// (A x) at this thread's u and v points from the staged stresses (stage_out_u / stage_out_v with the
// coefficients from registers); zero off the interior.
template <typename T, int TILE>
__device__ __forceinline__ void out_tagged(const Dims& d, const PointCoef<T>& pc, const OpTile<T, TILE, TILE>& s, T& yu,
                                           T& yv) {
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  const int li = threadIdx.x + 1, lj = threadIdx.y + 1;
  yu = 0;
  yv = 0;
  if (pc.inner_u)
    yu = (s.rxx[lj][li] - s.rxx[lj][li - 1]) * rdx + (s.rxy[lj][li - 1] - s.rxy[lj - 1][li - 1]) * rdy -
         pc.beta_u * s.xu[lj][li] - pc.hm_u * ((s.e[lj][li] - s.e[lj][li - 1]) * rdx);
  if (pc.inner_v)
    yv = (s.ryy[lj][li] - s.ryy[lj - 1][li]) * rdy + (s.rxy[lj - 1][li] - s.rxy[lj - 1][li - 1]) * rdx -
         pc.beta_v * s.xv[lj][li] - pc.hm_v * ((s.e[lj][li] - s.e[lj - 1][li]) * rdy);
}

// coarse_apply of the fast path: stage_tagged, the operator, the paired Pᵀ.  Returns false (in every
// thread) if a wait gave up.
template <typename T, int TILE>
__device__ __forceinline__ bool apply_tagged(const Dims& d, int levels, const CoefTile<T, TILE>& ct, const PointCoef<T>& pc,
                                             T hu, T hv, int i0, int j0, int ntx, CGShared<T, TILE>& sm,
                                             T (*hs2)[TILE + 1], const TagState& ts, GridBar* bar, volatile int* fail,
                                             T& cu, T& cv) {
  if (!stage_tagged<T, TILE>(d, ct, hu, hv, i0, j0, ntx, sm.op, ts, bar, fail)) return false;
  T yu, yv;
  out_tagged<T, TILE>(d, pc, sm.op, yu, yv);
  idwt2dT_pair<TILE>(yu, yv, sm.hs, hs2, levels);
  cu = pc.wm_u ? yu : (T)0;
  cv = pc.wm_v ? yv : (T)0;
  return true;
}

// ------------------------------------------------------------------------------------------------
// The smoother as one persistent launch per pass (FP32, 16 x 16 tiles): gauss_seidel_smoother!
// (update_preconditioners.jl:133-150), nsweeps sweeps over the four colours, each colour step the Jacobi
// update x += ω r / diag of that colour's interior points followed by r = b - A x, as the per-step
// k_smooth launches compute it (the same arithmetic in the same order).  A tile keeps x, r, b and diag
// in registers and its coefficients in shared memory; after each update it publishes its boundary as
// tagged words and the operator waits for its neighbours' ring only.  The boxes alternate parity by
// step: a tile rewrites parity p two steps later, after computing r of the step in between, which needs
// every neighbour's values of that step, which each neighbour publishes only after it has read this
// tile's parity-p words.  residual_first: a first step without update (r = b - A x of the input x; r
// is not read).  order: the four colours of a sweep, 3 bits each.
// ------------------------------------------------------------------------------------------------
template <int MAXT>
struct SmoothShared {
  OpTile<float, 16, 16> op;
  CoefTile<float, 16> ct[MAXT];
  int fail;
};

template <int MAXT>
__global__ void __launch_bounds__(256, MAXT <= 2 ? 2 : 1)
    k_smooth_persistent(Dims d, OpCoef<float> cf, const DevParams* __restrict__ P, const float* __restrict__ b,
                        const float* __restrict__ diag, float* __restrict__ x, float* __restrict__ r, int residual_first,
                        int nsweeps, int order, GridBar* bar, unsigned long long* __restrict__ halo, int ntx, int nty) {
  constexpr int TILE = 16;
  __shared__ SmoothShared<MAXT> sh;
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y;
  float xu[MAXT], xv[MAXT], ru[MAXT], rv[MAXT], bu[MAXT], bv[MAXT], du[MAXT], dv[MAXT];
  int colu[MAXT], colv[MAXT], i0s[MAXT], j0s[MAXT];
  bool own[MAXT];
  PointCoef<float> pc[MAXT] = {};
  TagState ts{halo, 0u, 0u, (size_t)ntiles * 8 * TILE};
  ts.base = *(volatile unsigned*)&bar->gen << 21;
  if (tx == 0 && ty == 0) sh.fail = 0;
  const float omega = (float)P->omega;
#pragma unroll
  for (int k = 0; k < MAXT; ++k) {
    const int t = blockIdx.x + k * gridDim.x;
    own[k] = t < ntiles;
    i0s[k] = own[k] ? (t % ntx) * TILE : 0;
    j0s[k] = own[k] ? (t / ntx) * TILE : 0;
    if (own[k]) load_coef_tile<float, TILE>(d, cf, cf.inner, i0s[k], j0s[k], sh.ct[k], pc[k]);
    const int i = i0s[k] + tx, j = j0s[k] + ty;
    const bool inu = own[k] && pc[k].inu, inv = own[k] && pc[k].inv;
    const int qu = inu ? uidx(d, i, j) : 0, qv = inv ? vidx(d, i, j) : 0;
    xu[k] = inu ? x[qu] : 0.f;
    xv[k] = inv ? x[qv] : 0.f;
    ru[k] = (inu && !residual_first) ? r[qu] : 0.f;
    rv[k] = (inv && !residual_first) ? r[qv] : 0.f;
    bu[k] = inu ? b[qu] : 0.f;
    bv[k] = inv ? b[qv] : 0.f;
    du[k] = inu ? diag[qu] : 1.f;
    dv[k] = inv ? diag[qv] : 1.f;
    const int par = ((i - j) % 2 + 2) % 2;
    colu[k] = 1 + par;
    colv[k] = 3 + par;
  }
  const int nsteps = (residual_first ? 1 : 0) + 4 * nsweeps;
  for (int step = 0; step < nsteps; ++step) {
    const int sw = step - residual_first;
    const int colour = sw < 0 ? 0 : (order >> (3 * (sw & 3))) & 7;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k] && colour) {
        if (pc[k].inner_u && colu[k] == colour) xu[k] = xu[k] + omega * ru[k] / du[k];
        if (pc[k].inner_v && colv[k] == colour) xv[k] = xv[k] + omega * rv[k] / dv[k];
      }
    ++ts.hx;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) publish_boundary<float, TILE>(xu[k], xv[k], blockIdx.x + k * gridDim.x, ts);
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        if (!stage_tagged<float, TILE>(d, sh.ct[k], xu[k], xv[k], i0s[k], j0s[k], ntx, sh.op, ts, bar, &sh.fail)) return;
        float yu, yv;
        out_tagged<float, TILE>(d, pc[k], sh.op, yu, yv);
        ru[k] = pc[k].inner_u ? bu[k] - yu : 0.f;
        rv[k] = pc[k].inner_v ? bv[k] - yv : 0.f;
      }
  }
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) {
      const int i = i0s[k] + tx, j = j0s[k] + ty;
      if (pc[k].inu) {
        const int q = uidx(d, i, j);
        x[q] = xu[k];
        r[q] = ru[k];
      }
      if (pc[k].inv) {
        const int q = vidx(d, i, j);
        x[q] = xv[k];
        r[q] = rv[k];
      }
    }
}

// Shared memory of the FP32 fast path: the coefficient tiles, the second Haar buffer, the failure flag.
template <typename T, int TILE, int MAXT>
struct FastShared {
  CoefTile<T, TILE> ct[MAXT];
  T hs2[TILE][TILE + 1];
  int fail;
};
template <typename T, int TILE, int MAXT>
using FastSharedFor = typename std::conditional<std::is_same<T, float>::value && TILE == 16, FastShared<T, TILE, MAXT>, char>::type;

// The fixed perturbation of the power iteration's start vector at full-layout index q: a value in [-1, 1)
// from a multiplicative hash (the oracle's coarse_srcg_chebyshev uses the same).
__device__ __forceinline__ float cheb_start(int q) {
  const unsigned h = (unsigned)q * 2654435761u;
  return (float)((h >> 8) & 0xffffu) * (1.0f / 32768.0f) - 1.0f;
}

// CG scalars broadcast to the CTA (written by thread 0 inside grid_sync).  R = CGReal<T>: the FP64
// kernels keep the reference's FP64 scalars; the FP32 kernels keep squared norms and the recurrence
// scalars in float-float (no FP64 arithmetic per iteration; res and tol are FP64, set once per solve).
template <typename T, typename RR = typename CGReal<T>::type>
struct CGScalars {
  using R = RR;      // the type of the sums and scalars: double, or float-float (FP32 kernels' default)
  double res, tol;   // |r| and the stopping tolerance
  double alpha_prev; // cg!'s "prev" (FP64 kernels)
  R rr, tol2;        // |r|^2 and tol^2
  R alpha, beta, gamma_prev;
  T alpha_t, beta_t;
  int stop;
};

template <typename T>
__device__ __forceinline__ T fmul_add(T a, T b, T c) {
  return a * b + c;
}
template <>
__device__ __forceinline__ float fmul_add<float>(float a, float b, float c) {
  return fmaf(a, b, c);
}

// a b + c d in the accumulation type A of a reduction (the FP32 kernels' default A = float: the same
// expression as written in float; A = double: every product and the sum in FP64)
template <typename A, typename T>
__device__ __forceinline__ A dot2(T a, T b, T c, T d) {
  return (A)a * (A)b + (A)c * (A)d;
}

__device__ __forceinline__ float to_vec(ff v) { return v.hi; }
__device__ __forceinline__ double to_vec(double v) { return v; }
__device__ __forceinline__ bool is_nan(ff v) { return !(v.hi == v.hi); }
__device__ __forceinline__ bool is_nan(double v) { return !(v == v); }
__device__ __forceinline__ bool not_finite(ff v) { return !(v.hi == v.hi) || isinf(v.hi); }
__device__ __forceinline__ bool not_finite(double v) { return !(v == v) || isinf(v); }

// cg! scalars (IterativeSolvers cg!, the reference's coarse solver).  Start: |r0|^2 and |b_c|^2 give the
// tolerance max(sqrt(eps) |r0|, tol_coarse |b_c|); the first direction is r (β = 0).
template <typename T>
__device__ __forceinline__ void cg_start(CGScalars<T>& sc, const typename CGReal<T>::type* tot, int maxit,
                                         double tol_coarse) {
  sc.res = sqrt(dbl_of(tot[0]));
  sc.rr = tot[0];
  sc.tol = fmax(1.4901161193847656e-08 * sc.res, tol_coarse * sqrt(dbl_of(tot[1])));  // reltol = sqrt(eps)
  if constexpr (std::is_same<T, float>::value)
    sc.tol2 = ff_of(sc.tol * sc.tol);
  else
    sc.tol2 = sc.tol * sc.tol;
  sc.alpha_prev = 1.0;  // prev
  sc.stop = (0 >= maxit) || sc.res <= sc.tol || !(sc.res == sc.res);
  sc.beta_t = (T)0;  // u = 0: the first direction is r
}
// α = |r|^2 / (u, c) with c = R A P u
template <typename T>
__device__ __forceinline__ void cg_alpha(CGScalars<T>& sc, const typename CGReal<T>::type* tot) {
  if constexpr (std::is_same<T, float>::value)
    sc.alpha = sc.rr / tot[0];
  else
    sc.alpha = (sc.res * sc.res) / tot[0];
  sc.alpha_t = (T)to_vec(sc.alpha);
}
// new |r|^2: stopping test and β = |r|^2 / |r_prev|^2
template <typename T>
__device__ __forceinline__ void cg_next(CGScalars<T>& sc, const typename CGReal<T>::type* tot, int it, int maxit) {
  if constexpr (std::is_same<T, float>::value) {  // squared norms: no square root per iteration
    const ff rr_prev = sc.rr;
    sc.rr = tot[0];
    sc.stop = it >= maxit || sc.rr <= sc.tol2 || is_nan(sc.rr);
    sc.beta = sc.rr / rr_prev;
  } else {
    sc.alpha_prev = sc.res;  // prev
    sc.res = sqrt(tot[0]);
    sc.stop = it >= maxit || sc.res <= sc.tol || !(sc.res == sc.res);
    sc.beta = (sc.res * sc.res) / (sc.alpha_prev * sc.alpha_prev);
  }
  sc.beta_t = (T)to_vec(sc.beta);
}
// Single-reduction CG scalars from γ = (r, z), δ = (w, z), |r|^2 (and |b_c|^2 in the first pass):
// β = γ/γ',  α = γ / (δ - β γ / α')  (the oracle's coarse_srcg in FP64, the same order).  With float-float
// sums (R = ff) the stopping test compares squared norms; with FP64 sums it is the FP64 kernels' test.
template <typename T, typename R = typename CGReal<T>::type>
__device__ __forceinline__ void srcg_scalars(CGScalars<T, R>& sc, const R* tot, bool first, int it, int maxit,
                                             double tol_coarse) {
  constexpr bool f32 = std::is_same<R, ff>::value;
  const R gamma = tot[0], delta = tot[1];
  sc.rr = tot[2];
  if (!f32 || first) sc.res = sqrt(dbl_of(tot[2]));
  int stop;
  if (first) {
    sc.tol = fmax(1.4901161193847656e-08 * sc.res, tol_coarse * sqrt(dbl_of(tot[3])));  // reltol = sqrt(eps)
    if constexpr (f32)
      sc.tol2 = ff_of(sc.tol * sc.tol);
    else
      sc.tol2 = sc.tol * sc.tol;
    sc.beta = R{};
    sc.alpha = gamma / delta;
    stop = (0 >= maxit) || sc.res <= sc.tol || is_nan(sc.rr);
  } else {
    if constexpr (f32)
      stop = it >= maxit || sc.rr <= sc.tol2 || is_nan(sc.rr);
    else
      stop = it >= maxit || sc.res <= sc.tol || is_nan(sc.rr);
    if (!stop) {
      sc.beta = gamma / sc.gamma_prev;
      sc.alpha = gamma / (delta - sc.beta * gamma / sc.alpha);
    }
  }
  if (!stop && not_finite(sc.alpha)) stop = 1;
  sc.gamma_prev = gamma;
  sc.alpha_t = (T)to_vec(sc.alpha);
  sc.beta_t = (T)to_vec(sc.beta);
  sc.stop = stop;
}
// The CG scalars of k_pcg_persistent: srcg_scalars' (the pipelined iteration has the same α and β), except
// that a restart (the recursively updated vectors replaced by recomputed ones) takes the first
// iteration's β = 0, α = γ/δ while keeping the tolerance and the iteration limit; and the decision to
// restart the next iteration: once |r| has fallen below kPcgRestartFactor times its value at the start or
// the last restart.  (In an FP32 simulation on assembled coarse systems this kept the iteration counts
// within 0.97-1.10x of single-reduction CG's, with two restarts per solve, where a fixed period of 25
// cost up to 29 % more iterations in FP64 and replacing r, u, w without restarting broke convergence.)
constexpr double kPcgRestartFactor = 1e-2;
template <typename T>
struct PcgScalars : CGScalars<T> {
  typename CGReal<T>::type rr_ref;  // |r|² at the start or the last restart
  int restart_next;
};
template <typename T>
__device__ __forceinline__ void pcg_scalars(PcgScalars<T>& sc, const typename CGReal<T>::type* tot, bool first,
                                            bool restart, int it, int maxit, double tol_coarse) {
  using R = typename CGReal<T>::type;
  constexpr bool f32 = std::is_same<T, float>::value;
  if (first) {
    srcg_scalars<T>(sc, tot, true, it, maxit, tol_coarse);
    sc.rr_ref = sc.rr;
    sc.restart_next = 0;
    return;
  }
  const R gamma = tot[0], delta = tot[1];
  sc.rr = tot[2];
  if (!f32) sc.res = sqrt(dbl_of(tot[2]));
  int stop;
  if constexpr (f32)
    stop = it >= maxit || sc.rr <= sc.tol2 || is_nan(sc.rr);
  else
    stop = it >= maxit || sc.res <= sc.tol || is_nan(sc.rr);
  if (!stop) {
    if (restart) {
      sc.beta = R{};
      sc.alpha = gamma / delta;
    } else {
      sc.beta = gamma / sc.gamma_prev;
      sc.alpha = gamma / (delta - sc.beta * gamma / sc.alpha);
    }
  }
  if (!stop && not_finite(sc.alpha)) stop = 1;
  if (restart) sc.rr_ref = sc.rr;
  sc.restart_next = !stop && dbl_of(sc.rr) < kPcgRestartFactor * kPcgRestartFactor * dbl_of(sc.rr_ref);
  sc.gamma_prev = gamma;
  sc.alpha_t = (T)to_vec(sc.alpha);
  sc.beta_t = (T)to_vec(sc.beta);
  sc.stop = stop;
}
// |r| of the final iterate for the statistics
template <typename T, typename R>
__device__ __forceinline__ double cg_final_res(const CGScalars<T, R>& sc) {
  if constexpr (std::is_same<R, ff>::value)
    return sqrt(dbl_of(sc.rr));
  else
    return sc.res;
}

// The whole coarse CG of one V-cycle with the reference's cg! recurrence: from the warm start xc and
// right-hand side bc (both global, full layout) to the final xc.  Writes the CG statistics into st (CTA 0).
// Stopping rule of cg!: |r| <= max(sqrt(eps) |r0|, abstol) with abstol = tol_coarse |b_c|, or maxiter.
template <typename T, int TILE, int MAXT>
__global__ void __launch_bounds__(TILE* TILE, (TILE == 16 && MAXT <= 2) ? 2 : 1)
    k_cg_persistent(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, T* __restrict__ w,
                    const T* __restrict__ bc, T* __restrict__ xc, double* __restrict__ partials, DevState* st,
                    const DevParams* __restrict__ P, GridBar* bar, unsigned long long* __restrict__ halo, int ntx,
                    int nty) {
  __shared__ CGShared<T, TILE> sm;
  __shared__ SyncShared ss;
  __shared__ CGScalars<T> sc;
  __shared__ FastSharedFor<T, TILE, MAXT> fs;
  PointCoef<T> pc[MAXT] = {};
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
  unsigned epoch = 0;
  int it = 0;
  const int maxit = P->maxiter_coarse;
  const double tol_coarse = coarse_tolerance(P, st);
  constexpr bool kFast = !std::is_same<FastSharedFor<T, TILE, MAXT>, char>::value;
  T hu[MAXT], hv[MAXT];  // fast path: the tiles' prolonged vectors (inner ⊙ P u)
  TagState ts{halo, 0u, 0u};
  volatile int* fail = nullptr;
  if constexpr (kFast) {
    ts.base = *(volatile unsigned*)&bar->gen << 21;
    fail = &fs.fail;
    if (tx == 0 && ty == 0) fs.fail = 0;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) load_coef_tile<T, TILE>(d, cf, wmask, i0s[k], j0s[k], fs.ct[k], pc[k]);
  }  // (all of it is read after a __syncthreads)
  // w = inner ⊙ P (a, b) for tile k: published (fast path) or stored to w
  auto prolong = [&](int k, T a, T b) {
    if constexpr (kFast)
      prolong_publish<T, TILE>(levels, pc[k], a, b, blockIdx.x + k * gridDim.x, sm, fs.hs2, ts, hu[k], hv[k]);
    else
      prolong_store<T, TILE>(d, levels, cf.inner, a, b, i0s[k], j0s[k], sm, w);
  };
  // between the prolongation and the operator: a grid barrier, except on the fast path, whose operator
  // waits for its halo ring
  auto halo_ready = [&]() -> bool {
    if constexpr (kFast)
      return true;
    else
      return grid_barrier<T>(bar, partials, epoch, ss);
  };
  // (c1, c2) = wmask ⊙ R A w on tile k
  auto apply = [&](int k, T& c1, T& c2) -> bool {
    if constexpr (kFast) {
      return apply_tagged<T, TILE>(d, levels, fs.ct[k], pc[k], hu[k], hv[k], i0s[k], j0s[k], ntx, sm, fs.hs2, ts, bar,
                                   fail, c1, c2);
    } else {
      coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0s[k], j0s[k], sm, c1, c2);
      return true;
    }
  };
  // start: w = P xc
  ++ts.hx;  // a new exchange
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) prolong(k, xu[k], xv[k]);
  if (!halo_ready()) return;
  // r = b_c - R A P xc, u = 0;  |r|^2 and |b_c|^2
  {
    T a[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        if (!apply(k, cu[k], cv[k])) return;
        const int i = i0s[k] + tx, j = j0s[k] + ty;
        const T bu = (i <= d.nx && j < d.ny) ? bc[uidx(d, i, j)] : (T)0;
        const T bv = (i < d.nx && j <= d.ny) ? bc[vidx(d, i, j)] : (T)0;
        ru[k] = bu - cu[k];
        rv[k] = bv - cv[k];
        a[0] += ru[k] * ru[k] + rv[k] * rv[k];
        a[1] += bu * bu + bv * bv;
      }
    if (!grid_sync<2>(bar, partials, epoch, ss, a, [&](const typename CGReal<T>::type* tot) { cg_start<T>(sc, tot, maxit, tol_coarse); }))
      return;
  }
  while (!sc.stop) {
    const T beta = sc.beta_t;
    ++ts.hx;  // a new exchange
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        uu[k] = fmul_add(beta, uu[k], ru[k]);
        uv[k] = fmul_add(beta, uv[k], rv[k]);
        prolong(k, uu[k], uv[k]);
      }
    if (!halo_ready()) return;
    T dot[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        if (!apply(k, cu[k], cv[k])) return;
        dot[0] += uu[k] * cu[k] + uv[k] * cv[k];
      }
    if (!grid_sync<1>(bar, partials, epoch, ss, dot, [&](const typename CGReal<T>::type* tot) { cg_alpha<T>(sc, tot); }))
      return;
    const T alpha = sc.alpha_t;
    T rr[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        xu[k] = fmul_add(alpha, uu[k], xu[k]);
        xv[k] = fmul_add(alpha, uv[k], xv[k]);
        ru[k] = fmul_add(-alpha, cu[k], ru[k]);
        rv[k] = fmul_add(-alpha, cv[k], rv[k]);
        rr[0] += ru[k] * ru[k] + rv[k] * rv[k];
      }
    ++it;
    if (!grid_sync<1>(bar, partials, epoch, ss, rr, [&](const typename CGReal<T>::type* tot) { cg_next<T>(sc, tot, it, maxit); }))
      return;
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
    st->cg_res = cg_final_res(sc);
    st->cg_prev = sc.alpha_prev;
    st->cg_tol = sc.tol;
  }
}

// Single-reduction CG (Chronopoulos & Gear, "s-step iterative methods for symmetric linear systems",
// J. Comput. Appl. Math. 25 (1989)) on R A P x = b_c, an opt-in alternative to the reference's cg!, with
// M = diag(R A P) (dcoarse) or M = I (dcoarse == nullptr), and cg!'s stopping rule on the
// unpreconditioned residual.  Both inner products of an iteration follow its one operator application,
// so an iteration costs one reduction barrier (cg! needs two reductions) besides its operator application:
//   x += α p;  r -= α s;  z = M⁻¹ r;  w = P z                                       -> barrier
//   w = R A w;  partial (r,z), (w,z), |r|^2                                         -> barrier + sums
//   β = γ/γ';  α = γ/(δ - β γ/α');  p = z + β p;  s = w + β s
// In FP32 this form keeps the attainable accuracy of standard CG (unlike the pipelined variants, whose
// recursively updated residual drifts by ~1e-3 in FP32).  The oracle's coarse_srcg states the same
// iteration in FP64.  cheb > 1 replaces M⁻¹ by the Chebyshev-accelerated Jacobi iteration (precond
// below): cheb - 1 more operator applications per iteration and ~0.4 of the iterations (and grid
// reductions) for cheb = 3 on the channel workloads.
template <typename T, int TILE, int MAXT, bool ACC64 = false>
__global__ void __launch_bounds__(TILE* TILE, (TILE == 16 && MAXT <= 2) ? 2 : 1)
    k_srcg_persistent(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, const T* __restrict__ dcoarse,
                      T* __restrict__ w, const T* __restrict__ bc, T* __restrict__ xc, double* __restrict__ partials,
                      DevState* st, const DevParams* __restrict__ P, GridBar* bar, unsigned long long* __restrict__ halo,
                      int cheb, float cheb_ratio, T* __restrict__ eig, int ntx, int nty) {
  // Acc: the type of the per-thread dot-product terms (T, or FP64 with ACC64: every product and sum of the
  // reductions in FP64, from the FP32 vectors); S: that of the grid sums and CG scalars
  using Acc = typename std::conditional<ACC64, double, T>::type;
  using S = typename CGReal<Acc>::type;
  __shared__ CGShared<T, TILE> sm;
  __shared__ SyncShared ss;
  __shared__ CGScalars<T, S> sc;
  __shared__ FastSharedFor<T, TILE, MAXT> fs;
  PointCoef<T> pc[MAXT] = {};
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y;
  T xu[MAXT], xv[MAXT], ru[MAXT], rv[MAXT], zu[MAXT], zv[MAXT], wu[MAXT], wv[MAXT];
  T pu[MAXT], pv[MAXT], su[MAXT], sv[MAXT], iu[MAXT], iv[MAXT];  // iu, iv: M⁻¹ (0 off the coarse space)
  T cdu[MAXT], cdv[MAXT];  // Chebyshev direction (cheb > 1)
  __shared__ T cheb_s[3];  // θ, δ, σ of the Chebyshev interval
  int i0s[MAXT], j0s[MAXT];
  bool own[MAXT];
#pragma unroll
  for (int k = 0; k < MAXT; ++k) {
    const int t = blockIdx.x + k * gridDim.x;
    own[k] = t < ntiles;
    i0s[k] = own[k] ? (t % ntx) * TILE : 0;
    j0s[k] = own[k] ? (t / ntx) * TILE : 0;
    const int i = i0s[k] + tx, j = j0s[k] + ty;
    const bool inu = own[k] && i <= d.nx && j < d.ny, inv = own[k] && i < d.nx && j <= d.ny;
    xu[k] = inu ? xc[uidx(d, i, j)] : (T)0;
    xv[k] = inv ? xc[vidx(d, i, j)] : (T)0;
    if (dcoarse) {
      const T du = inu ? dcoarse[uidx(d, i, j)] : (T)0, dv = inv ? dcoarse[vidx(d, i, j)] : (T)0;
      iu[k] = du != (T)0 ? (T)1 / du : (T)0;
      iv[k] = dv != (T)0 ? (T)1 / dv : (T)0;
    } else {
      iu[k] = iv[k] = (T)1;
    }
    ru[k] = rv[k] = zu[k] = zv[k] = wu[k] = wv[k] = pu[k] = pv[k] = su[k] = sv[k] = cdu[k] = cdv[k] = (T)0;
  }
  unsigned epoch = 0;
  int it = 0;
  const int maxit = P->maxiter_coarse;
  const double tol_coarse = coarse_tolerance(P, st);
  constexpr bool kFast = !std::is_same<FastSharedFor<T, TILE, MAXT>, char>::value;
  T hu[MAXT], hv[MAXT];  // fast path: the tiles' prolonged vectors (inner ⊙ P u)
  // two box sets (by exchange parity): the Chebyshev steps exchange without a grid reduction in between
  TagState ts{halo, 0u, 0u, (size_t)ntiles * 8 * TILE};
  volatile int* fail = nullptr;
  if constexpr (kFast) {
    ts.base = *(volatile unsigned*)&bar->gen << 21;
    fail = &fs.fail;
    if (tx == 0 && ty == 0) fs.fail = 0;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) load_coef_tile<T, TILE>(d, cf, wmask, i0s[k], j0s[k], fs.ct[k], pc[k]);
  }  // (all of it is read after a __syncthreads)
  // w = inner ⊙ P (a, b) for tile k: published (fast path) or stored to w
  auto prolong = [&](int k, T a, T b) {
    if constexpr (kFast)
      prolong_publish<T, TILE>(levels, pc[k], a, b, blockIdx.x + k * gridDim.x, sm, fs.hs2, ts, hu[k], hv[k]);
    else
      prolong_store<T, TILE>(d, levels, cf.inner, a, b, i0s[k], j0s[k], sm, w);
  };
  // between the prolongation and the operator: a grid barrier, except on the fast path, whose operator
  // waits for its halo ring
  auto halo_ready = [&]() -> bool {
    if constexpr (kFast)
      return true;
    else
      return grid_barrier<T>(bar, partials, epoch, ss);
  };
  // (c1, c2) = wmask ⊙ R A w on tile k
  auto apply = [&](int k, T& c1, T& c2) -> bool {
    if constexpr (kFast) {
      return apply_tagged<T, TILE>(d, levels, fs.ct[k], pc[k], hu[k], hv[k], i0s[k], j0s[k], ntx, sm, fs.hs2, ts, bar,
                                   fail, c1, c2);
    } else {
      coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0s[k], j0s[k], sm, c1, c2);
      return true;
    }
  };
  // z = M⁻¹ r: Jacobi, or (cheb > 1) the Jacobi-preconditioned Chebyshev iteration of cheb steps on
  // D⁻¹ R A P z = D⁻¹ r from z = 0 (a fixed polynomial in D⁻¹ R A P times D⁻¹, symmetric positive
  // definite for any interval when cheb is odd), cheb - 1 operator applications and no reduction
  auto precond = [&]() -> bool {
#pragma unroll
    for (int k = 0; k < MAXT; ++k) {
      zu[k] = iu[k] * ru[k];
      zv[k] = iv[k] * rv[k];
    }
    if (cheb <= 1) return true;
    const T th = cheb_s[0], de = cheb_s[1], sg = cheb_s[2];
#pragma unroll
    for (int k = 0; k < MAXT; ++k) {
      zu[k] = zu[k] / th;
      zv[k] = zv[k] / th;
      cdu[k] = zu[k];
      cdv[k] = zv[k];
    }
    T rho = (T)1 / sg;
    for (int stp = 1; stp < cheb; ++stp) {
      ++ts.hx;  // a new exchange
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) prolong(k, zu[k], zv[k]);
      if (!halo_ready()) return false;
      const T rn = (T)1 / ((T)2 * sg - rho), c1 = rn * rho, c2 = (T)2 * rn / de;
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) {
          T tu, tv;
          if (!apply(k, tu, tv)) return false;
          cdu[k] = c1 * cdu[k] + c2 * (iu[k] * (ru[k] - tu));
          cdv[k] = c1 * cdv[k] + c2 * (iv[k] * (rv[k] - tv));
          zu[k] = zu[k] + cdu[k];
          zv[k] = zv[k] + cdv[k];
        }
      rho = rn;
    }
    return true;
  };
  if (cheb > 1) {
    // λmax of D⁻¹ R A P by power steps from the previous V-cycle's vector (eig, zeroed at each solve's
    // start) plus a small fixed perturbation: 12 in a solve's first V-cycle, 4 after it; the interval
    // [b / cheb_ratio, b], b = 1.15 λmax
    T eu[MAXT], ev[MAXT];
#pragma unroll
    for (int k = 0; k < MAXT; ++k) {
      const int i = i0s[k] + tx, j = j0s[k] + ty;
      const bool inu = own[k] && i <= d.nx && j < d.ny, inv = own[k] && i < d.nx && j <= d.ny;
      const int qu = inu ? uidx(d, i, j) : 0, qv = inv ? vidx(d, i, j) : 0;
      eu[k] = iu[k] != (T)0 ? eig[qu] + (T)1e-3 * cheb_start(qu) : (T)0;
      ev[k] = iv[k] != (T)0 ? eig[qv] + (T)1e-3 * cheb_start(qv) : (T)0;
    }
    const int npow = st->picard_it <= 1 ? 12 : 4;
    for (int pstep = 0; pstep < npow; ++pstep) {
      ++ts.hx;  // a new exchange
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) prolong(k, eu[k], ev[k]);
      if (!halo_ready()) return;
      Acc a2[4] = {Acc(0), Acc(0), Acc(0), Acc(0)};
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) {
          T tu, tv;
          if (!apply(k, tu, tv)) return;
          tu = iu[k] * tu;
          tv = iv[k] * tv;
          a2[0] += dot2<Acc>(tu, tu, tv, tv);
          a2[1] += dot2<Acc>(eu[k], eu[k], ev[k], ev[k]);
          eu[k] = tu;
          ev[k] = tv;
        }
      if (!grid_sync<2>(bar, partials, epoch, ss, a2, [&](const S* tot) {
            const double tt = dbl_of(tot[0]), vv = dbl_of(tot[1]);
            const double lam = (vv > 0.0 && tt > 0.0) ? sqrt(tt / vv) : 1.0;
            const double bmax = 1.15 * lam, amin = bmax / (double)cheb_ratio;
            cheb_s[0] = (T)(0.5 * (bmax + amin));
            cheb_s[1] = (T)(0.5 * (bmax - amin));
            cheb_s[2] = (T)((bmax + amin) / (bmax - amin));
            sc.alpha_t = (T)(tt > 0.0 ? 1.0 / sqrt(tt) : 0.0);  // the normalisation of the power vector
          }))
        return;
      const T nrm = sc.alpha_t;
#pragma unroll
      for (int k = 0; k < MAXT; ++k) {
        eu[k] = eu[k] * nrm;
        ev[k] = ev[k] * nrm;
      }
    }
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        const int i = i0s[k] + tx, j = j0s[k] + ty;
        if (i <= d.nx && j < d.ny) eig[uidx(d, i, j)] = eu[k];
        if (i < d.nx && j <= d.ny) eig[vidx(d, i, j)] = ev[k];
      }
  }
  // r = b_c - R A P xc;  z = M⁻¹ r
  ++ts.hx;  // a new exchange
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) prolong(k, xu[k], xv[k]);
  if (!halo_ready()) return;
  Acc bb = 0;
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) {
      T cu, cv;
      if (!apply(k, cu, cv)) return;
      const int i = i0s[k] + tx, j = j0s[k] + ty;
      const T bu = (i <= d.nx && j < d.ny) ? bc[uidx(d, i, j)] : (T)0;
      const T bv = (i < d.nx && j <= d.ny) ? bc[vidx(d, i, j)] : (T)0;
      ru[k] = bu - cu;
      rv[k] = bv - cv;
      bb += dot2<Acc>(bu, bu, bv, bv);
    }
  if (!precond()) return;
  // (every CTA has read the prolonged vector, from w or from the halo boxes: the barrier below orders the
  // rewrite)
  if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
  bool first = true;
  for (;;) {
    if (!first) {
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) {
          const T alpha = sc.alpha_t;
          xu[k] = fmul_add(alpha, pu[k], xu[k]);
          xv[k] = fmul_add(alpha, pv[k], xv[k]);
          ru[k] = fmul_add(-alpha, su[k], ru[k]);
          rv[k] = fmul_add(-alpha, sv[k], rv[k]);
        }
      if (!precond()) return;
      ++it;
    }
    // w = R A P z
    ++ts.hx;  // a new exchange
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) prolong(k, zu[k], zv[k]);
    if (!halo_ready()) return;
    Acc a[4] = {Acc(0), Acc(0), Acc(0), first ? bb : Acc(0)};
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        if (!apply(k, wu[k], wv[k])) return;
        a[0] += dot2<Acc>(ru[k], zu[k], rv[k], zv[k]);
        a[1] += dot2<Acc>(wu[k], zu[k], wv[k], zv[k]);
        a[2] += dot2<Acc>(ru[k], ru[k], rv[k], rv[k]);
      }
    if (!grid_sync<4>(bar, partials, epoch, ss, a, [&](const S* tot) { srcg_scalars(sc, tot, first, it, maxit, tol_coarse); }))
      return;
    if (sc.stop) break;
    const T beta = sc.beta_t;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        pu[k] = fmul_add(beta, pu[k], zu[k]);
        pv[k] = fmul_add(beta, pv[k], zv[k]);
        su[k] = fmul_add(beta, su[k], wu[k]);
        sv[k] = fmul_add(beta, sv[k], wv[k]);
      }
    first = false;
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
    st->cg_res = cg_final_res(sc);
    st->cg_tol = sc.tol;
  }
}

// ------------------------------------------------------------------------------------------------
// Pipelined CG (Ghysels & Vanroose, "Hiding global synchronization latency in the preconditioned
// Conjugate Gradient algorithm", Parallel Computing 40 (2014) 224-238) on the FP32 fast path, with
// k_srcg_persistent's Chebyshev-accelerated Jacobi preconditioner M and cg!'s stopping rule.  The same
// iterates as k_srcg_persistent in exact arithmetic; each iteration's one grid reduction (arrived at by
// grid_arrive) completes while the CTA applies M and A, which need only neighbour exchanges:
//   γ = (r,u), δ = (w,u), |r|²  → arrive;  m = M⁻¹ w;  n = A m;  wait;  stop?
//   z = n + β z;  q = m + β q;  s = w + β s;  p = u + β p;  x += α p;  r −= α s;  u −= α q;  w −= α z
// from r = b − A x, u = M⁻¹ r, w = A u.  In FP32 the recursively updated r, u, w drift from b − A x, so the
// iteration restarts from x (r, u, w recomputed, β = 0) once |r| has fallen by kPcgRestartFactor since the
// start or the last restart (pcg_scalars decides it from the previous iteration's reduction).  The
// oracle's coarse_pipelined_chebyshev states the same iteration, restarts included, in FP64.  x, r, u, w
// and the preconditioner's vectors stay in registers; p, s, q, z live in shared memory (each thread
// touches only its own points of them).

template <typename T, int TILE, int MAXT>
struct PcgShared {
  T v[4][MAXT][2][TILE * TILE];  // p, s, q, z: [vector][tile][u, v][thread]
};

template <typename T, int TILE, int MAXT>
__global__ void __launch_bounds__(TILE* TILE, (TILE == 16 && MAXT <= 2) ? 2 : 1)
    k_pcg_persistent(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, const T* __restrict__ dcoarse,
                     const T* __restrict__ bc, T* __restrict__ xc, double* __restrict__ partials, DevState* st,
                     const DevParams* __restrict__ P, GridBar* bar, unsigned long long* __restrict__ halo, int cheb,
                     float cheb_ratio, T* __restrict__ eig, int ntx, int nty) {
  static_assert(!std::is_same<FastSharedFor<T, TILE, MAXT>, char>::value, "the pipelined CG needs the FP32 fast path");
  __shared__ CGShared<T, TILE> sm;
  __shared__ SyncShared ss;
  __shared__ PcgScalars<T> sc;
  __shared__ FastSharedFor<T, TILE, MAXT> fs;
  __shared__ PcgShared<T, TILE, MAXT> pv;
  __shared__ T cheb_s[3];  // θ, δ, σ of the Chebyshev interval
  enum { VP = 0, VS = 1, VQ = 2, VZ = 3 };
  PointCoef<T> pc[MAXT] = {};
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y, lin = ty * TILE + tx;
  T xu[MAXT], xv[MAXT], ru[MAXT], rv[MAXT], uu[MAXT], uv[MAXT], wu[MAXT], wv[MAXT];
  T mu[MAXT], mv[MAXT], nu[MAXT], nv[MAXT], iu[MAXT], iv[MAXT];  // iu, iv: D⁻¹ (0 off the coarse space)
  T cdu[MAXT], cdv[MAXT];                                        // Chebyshev direction
  T hu[MAXT], hv[MAXT];                                          // the tiles' prolonged vectors
  int i0s[MAXT], j0s[MAXT];
  bool own[MAXT];
#pragma unroll
  for (int k = 0; k < MAXT; ++k) {
    const int t = blockIdx.x + k * gridDim.x;
    own[k] = t < ntiles;
    i0s[k] = own[k] ? (t % ntx) * TILE : 0;
    j0s[k] = own[k] ? (t / ntx) * TILE : 0;
    const int i = i0s[k] + tx, j = j0s[k] + ty;
    const bool inu = own[k] && i <= d.nx && j < d.ny, inv = own[k] && i < d.nx && j <= d.ny;
    xu[k] = inu ? xc[uidx(d, i, j)] : (T)0;
    xv[k] = inv ? xc[vidx(d, i, j)] : (T)0;
    const T du = inu ? dcoarse[uidx(d, i, j)] : (T)0, dv = inv ? dcoarse[vidx(d, i, j)] : (T)0;
    iu[k] = du != (T)0 ? (T)1 / du : (T)0;
    iv[k] = dv != (T)0 ? (T)1 / dv : (T)0;
    ru[k] = rv[k] = uu[k] = uv[k] = wu[k] = wv[k] = mu[k] = mv[k] = nu[k] = nv[k] = cdu[k] = cdv[k] = (T)0;
#pragma unroll
    for (int q = 0; q < 4; ++q) pv.v[q][k][0][lin] = pv.v[q][k][1][lin] = (T)0;
  }
  unsigned epoch = 0;
  int it = 0;
  const int maxit = P->maxiter_coarse;
  const double tol_coarse = coarse_tolerance(P, st);
  TagState ts{halo, 0u, 0u, (size_t)ntiles * 8 * TILE};
  ts.base = *(volatile unsigned*)&bar->gen << 21;
  volatile int* fail = &fs.fail;
  if (tx == 0 && ty == 0) fs.fail = 0;
#pragma unroll
  for (int k = 0; k < MAXT; ++k)
    if (own[k]) load_coef_tile<T, TILE>(d, cf, wmask, i0s[k], j0s[k], fs.ct[k], pc[k]);
  // (all of it is read after a __syncthreads)
  auto prolong = [&](int k, T a, T b) {
    prolong_publish<T, TILE>(levels, pc[k], a, b, blockIdx.x + k * gridDim.x, sm, fs.hs2, ts, hu[k], hv[k]);
  };
  auto apply = [&](int k, T& c1, T& c2) -> bool {
    return apply_tagged<T, TILE>(d, levels, fs.ct[k], pc[k], hu[k], hv[k], i0s[k], j0s[k], ntx, sm, fs.hs2, ts, bar,
                                 fail, c1, c2);
  };
  // (ou, ov) = R A P (au, av): one neighbour exchange
  auto op = [&](const T (&au)[MAXT], const T (&av)[MAXT], T (&ou)[MAXT], T (&ov)[MAXT]) -> bool {
    ++ts.hx;  // a new exchange
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) prolong(k, au[k], av[k]);
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k] && !apply(k, ou[k], ov[k])) return false;
    return true;
  };
  // (ou, ov) = M⁻¹ (au, av): cheb steps of the Chebyshev iteration on D⁻¹ R A P z = D⁻¹ a from z = 0, as
  // k_srcg_persistent's precond (cheb - 1 exchanges, no reduction)
  auto precond = [&](const T (&au)[MAXT], const T (&av)[MAXT], T (&ou)[MAXT], T (&ov)[MAXT]) -> bool {
    const T th = cheb_s[0], de = cheb_s[1], sg = cheb_s[2];
#pragma unroll
    for (int k = 0; k < MAXT; ++k) {
      ou[k] = iu[k] * au[k];
      ov[k] = iv[k] * av[k];
      ou[k] = ou[k] / th;
      ov[k] = ov[k] / th;
      cdu[k] = ou[k];
      cdv[k] = ov[k];
    }
    T rho = (T)1 / sg;
    for (int stp = 1; stp < cheb; ++stp) {
      ++ts.hx;  // a new exchange
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) prolong(k, ou[k], ov[k]);
      const T rn = (T)1 / ((T)2 * sg - rho), c1 = rn * rho, c2 = (T)2 * rn / de;
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) {
          T tu, tv;
          if (!apply(k, tu, tv)) return false;
          cdu[k] = c1 * cdu[k] + c2 * (iu[k] * (au[k] - tu));
          cdv[k] = c1 * cdv[k] + c2 * (iv[k] * (av[k] - tv));
          ou[k] = ou[k] + cdu[k];
          ov[k] = ov[k] + cdv[k];
        }
      rho = rn;
    }
    return true;
  };
  // λmax of D⁻¹ R A P by power steps, as in k_srcg_persistent
  {
    T eu[MAXT], ev[MAXT];
#pragma unroll
    for (int k = 0; k < MAXT; ++k) {
      const int i = i0s[k] + tx, j = j0s[k] + ty;
      const bool inu = own[k] && i <= d.nx && j < d.ny, inv = own[k] && i < d.nx && j <= d.ny;
      const int qu = inu ? uidx(d, i, j) : 0, qv = inv ? vidx(d, i, j) : 0;
      eu[k] = iu[k] != (T)0 ? eig[qu] + (T)1e-3 * cheb_start(qu) : (T)0;
      ev[k] = iv[k] != (T)0 ? eig[qv] + (T)1e-3 * cheb_start(qv) : (T)0;
    }
    const int npow = st->picard_it <= 1 ? 12 : 4;
    for (int pstep = 0; pstep < npow; ++pstep) {
      ++ts.hx;  // a new exchange
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) prolong(k, eu[k], ev[k]);
      T a2[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
      for (int k = 0; k < MAXT; ++k)
        if (own[k]) {
          T tu, tv;
          if (!apply(k, tu, tv)) return;
          tu = iu[k] * tu;
          tv = iv[k] * tv;
          a2[0] += tu * tu + tv * tv;
          a2[1] += eu[k] * eu[k] + ev[k] * ev[k];
          eu[k] = tu;
          ev[k] = tv;
        }
      if (!grid_sync<2>(bar, partials, epoch, ss, a2, [&](const typename CGReal<T>::type* tot) {
            const double tt = dbl_of(tot[0]), vv = dbl_of(tot[1]);
            const double lam = (vv > 0.0 && tt > 0.0) ? sqrt(tt / vv) : 1.0;
            const double bmax = 1.15 * lam, amin = bmax / (double)cheb_ratio;
            cheb_s[0] = (T)(0.5 * (bmax + amin));
            cheb_s[1] = (T)(0.5 * (bmax - amin));
            cheb_s[2] = (T)((bmax + amin) / (bmax - amin));
            sc.alpha_t = (T)(tt > 0.0 ? 1.0 / sqrt(tt) : 0.0);  // the normalisation of the power vector
          }))
        return;
      const T nrm = sc.alpha_t;
#pragma unroll
      for (int k = 0; k < MAXT; ++k) {
        eu[k] = eu[k] * nrm;
        ev[k] = ev[k] * nrm;
      }
    }
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        const int i = i0s[k] + tx, j = j0s[k] + ty;
        if (i <= d.nx && j < d.ny) eig[uidx(d, i, j)] = eu[k];
        if (i < d.nx && j <= d.ny) eig[vidx(d, i, j)] = ev[k];
      }
  }
  // r = b_c − R A P x (and |b_c|² for the tolerance); u = M⁻¹ r; w = R A P u
  T bb = 0;
  auto residual = [&]() -> bool {
    if (!op(xu, xv, nu, nv)) return false;
    bb = 0;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        const int i = i0s[k] + tx, j = j0s[k] + ty;
        const T bu = (i <= d.nx && j < d.ny) ? bc[uidx(d, i, j)] : (T)0;
        const T bv = (i < d.nx && j <= d.ny) ? bc[vidx(d, i, j)] : (T)0;
        ru[k] = bu - nu[k];
        rv[k] = bv - nv[k];
        bb += bu * bu + bv * bv;
      }
    if (!precond(ru, rv, uu, uv)) return false;
    return op(uu, uv, wu, wv);
  };
  if (!residual()) return;
  bool first = true;
  for (;;) {
    // restart (decided by the previous iteration's scalars): r, u, w recomputed from x; β = 0 below
    const bool restart = !first && sc.restart_next;
    if (restart && !residual()) return;
    T a[4] = {T(0), T(0), T(0), first ? bb : T(0)};
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        a[0] += ru[k] * uu[k] + rv[k] * uv[k];
        a[1] += wu[k] * uu[k] + wv[k] * uv[k];
        a[2] += ru[k] * ru[k] + rv[k] * rv[k];
      }
    grid_arrive<4>(bar, partials, epoch, ss, a);
    // m = M⁻¹ w and n = R A P m while the grid sum completes
    if (!precond(wu, wv, mu, mv)) return;
    if (!op(mu, mv, nu, nv)) return;
    if (!grid_wait<4, T>(bar, partials, epoch, ss, [&](const typename CGReal<T>::type* tot) {
          pcg_scalars<T>(sc, tot, first, restart, it, maxit, tol_coarse);
        }))
      return;
    if (sc.stop) break;
    const T alpha = sc.alpha_t, beta = sc.beta_t;
#pragma unroll
    for (int k = 0; k < MAXT; ++k)
      if (own[k]) {
        T z0 = pv.v[VZ][k][0][lin], z1 = pv.v[VZ][k][1][lin];
        T q0 = pv.v[VQ][k][0][lin], q1 = pv.v[VQ][k][1][lin];
        T s0 = pv.v[VS][k][0][lin], s1 = pv.v[VS][k][1][lin];
        T p0 = pv.v[VP][k][0][lin], p1 = pv.v[VP][k][1][lin];
        z0 = fmul_add(beta, z0, nu[k]);
        z1 = fmul_add(beta, z1, nv[k]);
        q0 = fmul_add(beta, q0, mu[k]);
        q1 = fmul_add(beta, q1, mv[k]);
        s0 = fmul_add(beta, s0, wu[k]);
        s1 = fmul_add(beta, s1, wv[k]);
        p0 = fmul_add(beta, p0, uu[k]);
        p1 = fmul_add(beta, p1, uv[k]);
        xu[k] = fmul_add(alpha, p0, xu[k]);
        xv[k] = fmul_add(alpha, p1, xv[k]);
        ru[k] = fmul_add(-alpha, s0, ru[k]);
        rv[k] = fmul_add(-alpha, s1, rv[k]);
        uu[k] = fmul_add(-alpha, q0, uu[k]);
        uv[k] = fmul_add(-alpha, q1, uv[k]);
        wu[k] = fmul_add(-alpha, z0, wu[k]);
        wv[k] = fmul_add(-alpha, z1, wv[k]);
        pv.v[VZ][k][0][lin] = z0;
        pv.v[VZ][k][1][lin] = z1;
        pv.v[VQ][k][0][lin] = q0;
        pv.v[VQ][k][1][lin] = q1;
        pv.v[VS][k][0][lin] = s0;
        pv.v[VS][k][1][lin] = s1;
        pv.v[VP][k][0][lin] = p0;
        pv.v[VP][k][1][lin] = p1;
      }
    ++it;
    first = false;
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
    st->cg_res = cg_final_res(sc);
    st->cg_tol = sc.tol;
  }
}

// ------------------------------------------------------------------------------------------------
// Grids whose tiles outnumber the device's resident CTAs: the same two solvers with the CG vectors in
// global memory (L2-resident up to ~10^7 unknowns), each CTA looping over tiles t = blockIdx.x + k·gridDim.x
// in every phase.  The arithmetic and its order are those of the register-resident kernels above.  Their
// tile passes wait on L2 loads (ncu at 2560x320: long-scoreboard stalls first, 25 % of warps active at two
// CTAs per SM), so the 16 x 16 instantiations are held to 64 registers for four resident CTAs per SM.
// Vectors (full layout, N entries): xc (iterate, in place), gr (residual), gz (z = M⁻¹ r, or cg!'s
// direction u), gp, gs (C-G recurrences, or cg!'s c = R A u in gp), gw (R A z), w (prolonged vector).
// ------------------------------------------------------------------------------------------------
template <typename T>
struct GlobalCG {
  T *gr, *gz, *gp, *gs, *gw;
};

template <typename T, int TILE>
__global__ void __launch_bounds__(TILE* TILE, TILE == 16 ? 4 : 1)
    k_srcg_global(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, const T* __restrict__ dcoarse,
                  T* __restrict__ w, const T* __restrict__ bc, T* __restrict__ xc, GlobalCG<T> g,
                  double* __restrict__ partials, DevState* st, const DevParams* __restrict__ P, GridBar* bar, int ntx,
                  int nty) {
  __shared__ CGShared<T, TILE> sm;
  __shared__ SyncShared ss;
  __shared__ CGScalars<T> sc;
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y;
  unsigned epoch = 0;
  int it = 0;
  const int maxit = P->maxiter_coarse;
  const double tol_coarse = coarse_tolerance(P, st);
  const bool use_m = dcoarse != nullptr;
  auto minv = [&](int q) -> T {
    if (!use_m) return (T)1;
    const T dq = dcoarse[q];
    return dq != (T)0 ? (T)1 / dq : (T)0;
  };
  // w = P xc
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
    const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
    prolong_store<T, TILE>(d, levels, cf.inner, inu ? xc[uidx(d, i, j)] : (T)0, inv ? xc[vidx(d, i, j)] : (T)0, i0,
                           j0, sm, w);
  }
  if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
  // r = b_c - R A w;  z = M⁻¹ r;  p = s = 0
  T bb = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
    const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
    T cu, cv;
    coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0, j0, sm, cu, cv);
    if (inu) {
      const int q = uidx(d, i, j);
      const T bu = bc[q], ru = bu - cu;
      g.gr[q] = ru;
      g.gz[q] = minv(q) * ru;
      g.gp[q] = g.gs[q] = (T)0;
      bb += bu * bu;
    }
    if (inv) {
      const int q = vidx(d, i, j);
      const T bv = bc[q], rv = bv - cv;
      g.gr[q] = rv;
      g.gz[q] = minv(q) * rv;
      g.gp[q] = g.gs[q] = (T)0;
      bb += bv * bv;
    }
  }
  if (!grid_barrier<T>(bar, partials, epoch, ss)) return;  // every CTA has read w
  bool first = true;
  for (;;) {
    // (after the first pass) p = z + β p;  s = R A z + β s;  x += α p;  r -= α s;  z = M⁻¹ r;  w = P z
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
      T zz[2] = {(T)0, (T)0};
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        if (comp == 0 ? !inu : !inv) continue;
        const int q = comp == 0 ? uidx(d, i, j) : vidx(d, i, j);
        T z = g.gz[q];
        if (!first) {
          const T alpha = sc.alpha_t, beta = sc.beta_t;
          const T p = fmul_add(beta, g.gp[q], z), s = fmul_add(beta, g.gs[q], g.gw[q]);
          const T x = fmul_add(alpha, p, xc[q]), r = fmul_add(-alpha, s, g.gr[q]);
          z = minv(q) * r;
          g.gp[q] = p;
          g.gs[q] = s;
          xc[q] = x;
          g.gr[q] = r;
          g.gz[q] = z;
        }
        zz[comp] = z;
      }
      prolong_store<T, TILE>(d, levels, cf.inner, zz[0], zz[1], i0, j0, sm, w);
    }
    if (!first) ++it;
    if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
    T a[4] = {T(0), T(0), T(0), first ? bb : T(0)};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      T wu, wv;
      coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0, j0, sm, wu, wv);
      if (i <= d.nx && j < d.ny) {
        const int q = uidx(d, i, j);
        const T r = g.gr[q], z = g.gz[q];
        a[0] += r * z;
        a[1] += wu * z;
        a[2] += r * r;
        g.gw[q] = wu;
      }
      if (i < d.nx && j <= d.ny) {
        const int q = vidx(d, i, j);
        const T r = g.gr[q], z = g.gz[q];
        a[0] += r * z;
        a[1] += wv * z;
        a[2] += r * r;
        g.gw[q] = wv;
      }
    }
    if (!grid_sync<4>(bar, partials, epoch, ss, a, [&](const typename CGReal<T>::type* tot) { srcg_scalars(sc, tot, first, it, maxit, tol_coarse); }))
      return;
    if (sc.stop) break;
    first = false;
  }
  if (blockIdx.x == 0 && tx == 0 && ty == 0) {
    st->cg_it = it;
    st->cg_total += it;
    st->cg_res = cg_final_res(sc);
    st->cg_tol = sc.tol;
  }
}

// The single-reduction CG with the Chebyshev-accelerated Jacobi preconditioner (k_srcg_persistent with
// cheb > 1) for grids whose tiles outnumber the resident CTAs: the vectors in global memory, each CTA
// looping over tiles.  The same arithmetic per point as the register-resident kernel: λmax by npow power
// steps from the previous V-cycle's vector (eig), then per iteration cheb - 1 Chebyshev steps and one
// operator application with its two inner products and |r|² in one grid reduction.  Each Chebyshev step
// applies the operator to the prolonged vector of the previous one and prolongs its own result in the
// same tile pass, into the other of two prolongation buffers (w, w2), so that a step needs one grid barrier:
// a buffer is rewritten only after the barrier that follows the pass in which every CTA read it.
// gcd holds the Chebyshev direction.
template <typename T, int TILE>
__global__ void __launch_bounds__(TILE* TILE, TILE == 16 ? 4 : 1)
    k_srcg_cheb_global(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask,
                       const T* __restrict__ dcoarse, T* __restrict__ w, T* __restrict__ w2, const T* __restrict__ bc,
                       T* __restrict__ xc, GlobalCG<T> g, T* __restrict__ gcd, T* __restrict__ eig, int cheb,
                       float cheb_ratio, double* __restrict__ partials, DevState* st, const DevParams* __restrict__ P,
                       GridBar* bar, int ntx, int nty) {
  __shared__ CGShared<T, TILE> sm;
  __shared__ SyncShared ss;
  __shared__ CGScalars<T> sc;
  __shared__ T cheb_s[3];  // θ, δ, σ of the Chebyshev interval
  using S = typename CGReal<T>::type;
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y;
  unsigned epoch = 0;
  int it = 0;
  const int maxit = P->maxiter_coarse;
  const double tol_coarse = coarse_tolerance(P, st);
  T* const wbuf[2] = {w, w2};
  int wsel = 0;
  auto minv = [&](int q) -> T {
    const T dq = dcoarse[q];
    return dq != (T)0 ? (T)1 / dq : (T)0;
  };
  // λmax of D⁻¹ R A P: power steps from eig (plus a small fixed perturbation), normalised by the grid sum
  {
    T scale = (T)1;
    const int npow = st->picard_it <= 1 ? 12 : 4;
    for (int pstep = 0; pstep < npow; ++pstep) {
      auto e_of = [&](int q) -> T {
        if (pstep > 0) return eig[q] * scale;
        return minv(q) != (T)0 ? eig[q] + (T)1e-3 * cheb_start(q) : (T)0;
      };
      T* wo = wbuf[wsel];
      wsel ^= 1;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
        const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
        prolong_store<T, TILE>(d, levels, cf.inner, inu ? e_of(uidx(d, i, j)) : (T)0, inv ? e_of(vidx(d, i, j)) : (T)0,
                               i0, j0, sm, wo);
      }
      if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
      T a2[4] = {T(0), T(0), T(0), T(0)};
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
        T tu, tv;
        coarse_apply<T, TILE>(d, levels, cf, wmask, wo, i0, j0, sm, tu, tv);
        if (i <= d.nx && j < d.ny) {
          const int q = uidx(d, i, j);
          const T e = e_of(q), tq = minv(q) * tu;
          a2[0] += tq * tq;
          a2[1] += e * e;
          eig[q] = tq;
        }
        if (i < d.nx && j <= d.ny) {
          const int q = vidx(d, i, j);
          const T e = e_of(q), tq = minv(q) * tv;
          a2[0] += tq * tq;
          a2[1] += e * e;
          eig[q] = tq;
        }
      }
      if (!grid_sync<2>(bar, partials, epoch, ss, a2, [&](const S* tot) {
            const double tt = dbl_of(tot[0]), vv = dbl_of(tot[1]);
            const double lam = (vv > 0.0 && tt > 0.0) ? sqrt(tt / vv) : 1.0;
            const double bmax = 1.15 * lam, amin = bmax / (double)cheb_ratio;
            cheb_s[0] = (T)(0.5 * (bmax + amin));
            cheb_s[1] = (T)(0.5 * (bmax - amin));
            cheb_s[2] = (T)((bmax + amin) / (bmax - amin));
            sc.alpha_t = (T)(tt > 0.0 ? 1.0 / sqrt(tt) : 0.0);  // the normalisation of the power vector
          }))
        return;
      scale = sc.alpha_t;
    }
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      if (i <= d.nx && j < d.ny) eig[uidx(d, i, j)] *= scale;
      if (i < d.nx && j <= d.ny) eig[vidx(d, i, j)] *= scale;
    }
  }
  // z = M⁻¹ r (gr into gz): cheb steps of the Jacobi-preconditioned Chebyshev iteration on D⁻¹ R A P z = D⁻¹ r
  // from z = 0; ends with z prolonged into wbuf[wsel ^ 1] (returned), which a grid barrier must precede
  // any read of
  auto precond = [&](T*& wout) -> bool {
    const T th = cheb_s[0], de = cheb_s[1], sg = cheb_s[2];
    T* wo = wbuf[wsel];
    wsel ^= 1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      T zz[2] = {(T)0, (T)0};
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        if (comp == 0 ? !(i <= d.nx && j < d.ny) : !(i < d.nx && j <= d.ny)) continue;
        const int q = comp == 0 ? uidx(d, i, j) : vidx(d, i, j);
        const T z = minv(q) * g.gr[q] / th;
        g.gz[q] = z;
        gcd[q] = z;
        zz[comp] = z;
      }
      prolong_store<T, TILE>(d, levels, cf.inner, zz[0], zz[1], i0, j0, sm, wo);
    }
    T rho = (T)1 / sg;
    for (int stp = 1; stp < cheb; ++stp) {
      if (!grid_barrier<T>(bar, partials, epoch, ss)) return false;
      const T rn = (T)1 / ((T)2 * sg - rho), c1 = rn * rho, c2 = (T)2 * rn / de;
      T* wn = wbuf[wsel];
      wsel ^= 1;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
        T tt[2];
        coarse_apply<T, TILE>(d, levels, cf, wmask, wo, i0, j0, sm, tt[0], tt[1]);
        T zz[2] = {(T)0, (T)0};
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          if (comp == 0 ? !(i <= d.nx && j < d.ny) : !(i < d.nx && j <= d.ny)) continue;
          const int q = comp == 0 ? uidx(d, i, j) : vidx(d, i, j);
          const T cd = c1 * gcd[q] + c2 * (minv(q) * (g.gr[q] - tt[comp]));
          const T z = g.gz[q] + cd;
          gcd[q] = cd;
          g.gz[q] = z;
          zz[comp] = z;
        }
        prolong_store<T, TILE>(d, levels, cf.inner, zz[0], zz[1], i0, j0, sm, wn);
      }
      wo = wn;
      rho = rn;
    }
    wout = wo;
    return true;
  };
  // r = b_c - R A P xc;  p = s = 0
  T* wcur = wbuf[wsel];
  wsel ^= 1;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
    const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
    prolong_store<T, TILE>(d, levels, cf.inner, inu ? xc[uidx(d, i, j)] : (T)0, inv ? xc[vidx(d, i, j)] : (T)0, i0,
                           j0, sm, wcur);
  }
  if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
  T bb = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
    T cu, cv;
    coarse_apply<T, TILE>(d, levels, cf, wmask, wcur, i0, j0, sm, cu, cv);
    if (i <= d.nx && j < d.ny) {
      const int q = uidx(d, i, j);
      const T bu = bc[q];
      g.gr[q] = bu - cu;
      g.gp[q] = g.gs[q] = (T)0;
      bb += bu * bu;
    }
    if (i < d.nx && j <= d.ny) {
      const int q = vidx(d, i, j);
      const T bv = bc[q];
      g.gr[q] = bv - cv;
      g.gp[q] = g.gs[q] = (T)0;
      bb += bv * bv;
    }
  }
  if (!precond(wcur)) return;
  if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
  bool first = true;
  for (;;) {
    // w = R A P z with γ = (r, z), δ = (w, z), |r|²
    T a[4] = {T(0), T(0), T(0), first ? bb : T(0)};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      T wu, wv;
      coarse_apply<T, TILE>(d, levels, cf, wmask, wcur, i0, j0, sm, wu, wv);
      if (i <= d.nx && j < d.ny) {
        const int q = uidx(d, i, j);
        const T r = g.gr[q], z = g.gz[q];
        a[0] += r * z;
        a[1] += wu * z;
        a[2] += r * r;
        g.gw[q] = wu;
      }
      if (i < d.nx && j <= d.ny) {
        const int q = vidx(d, i, j);
        const T r = g.gr[q], z = g.gz[q];
        a[0] += r * z;
        a[1] += wv * z;
        a[2] += r * r;
        g.gw[q] = wv;
      }
    }
    if (!grid_sync<4>(bar, partials, epoch, ss, a, [&](const S* tot) { srcg_scalars(sc, tot, first, it, maxit, tol_coarse); }))
      return;
    if (sc.stop) break;
    // p = z + β p;  s = w + β s;  x += α p;  r -= α s;  then z = M⁻¹ r
    const T alpha = sc.alpha_t, beta = sc.beta_t;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        if (comp == 0 ? !(i <= d.nx && j < d.ny) : !(i < d.nx && j <= d.ny)) continue;
        const int q = comp == 0 ? uidx(d, i, j) : vidx(d, i, j);
        const T pq = fmul_add(beta, g.gp[q], g.gz[q]), sq = fmul_add(beta, g.gs[q], g.gw[q]);
        g.gp[q] = pq;
        g.gs[q] = sq;
        xc[q] = fmul_add(alpha, pq, xc[q]);
        g.gr[q] = fmul_add(-alpha, sq, g.gr[q]);
      }
    }
    ++it;
    if (!precond(wcur)) return;
    if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
    first = false;
  }
  if (blockIdx.x == 0 && tx == 0 && ty == 0) {
    st->cg_it = it;
    st->cg_total += it;
    st->cg_res = cg_final_res(sc);
    st->cg_tol = sc.tol;
  }
}

// cg! with global vectors: gz holds the direction u, gp holds c = R A u.
template <typename T, int TILE>
__global__ void __launch_bounds__(TILE* TILE, TILE == 16 ? 4 : 1)
    k_cg_global(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, T* __restrict__ w,
                const T* __restrict__ bc, T* __restrict__ xc, GlobalCG<T> g, double* __restrict__ partials, DevState* st,
                const DevParams* __restrict__ P, GridBar* bar, int ntx, int nty) {
  __shared__ CGShared<T, TILE> sm;
  __shared__ SyncShared ss;
  __shared__ CGScalars<T> sc;
  const int ntiles = ntx * nty;
  const int tx = threadIdx.x, ty = threadIdx.y;
  unsigned epoch = 0;
  int it = 0;
  const int maxit = P->maxiter_coarse;
  const double tol_coarse = coarse_tolerance(P, st);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
    const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
    prolong_store<T, TILE>(d, levels, cf.inner, inu ? xc[uidx(d, i, j)] : (T)0, inv ? xc[vidx(d, i, j)] : (T)0, i0,
                           j0, sm, w);
  }
  if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
  {
    T a[4] = {T(0), T(0), T(0), T(0)};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      T cu, cv;
      coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0, j0, sm, cu, cv);
      if (i <= d.nx && j < d.ny) {
        const int q = uidx(d, i, j);
        const T bu = bc[q], ru = bu - cu;
        g.gr[q] = ru;
        g.gz[q] = (T)0;
        a[0] += ru * ru;
        a[1] += bu * bu;
      }
      if (i < d.nx && j <= d.ny) {
        const int q = vidx(d, i, j);
        const T bv = bc[q], rv = bv - cv;
        g.gr[q] = rv;
        g.gz[q] = (T)0;
        a[0] += rv * rv;
        a[1] += bv * bv;
      }
    }
    if (!grid_sync<2>(bar, partials, epoch, ss, a, [&](const typename CGReal<T>::type* tot) { cg_start<T>(sc, tot, maxit, tol_coarse); }))
      return;
  }
  while (!sc.stop) {
    const T beta = sc.beta_t;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      const bool inu = i <= d.nx && j < d.ny, inv = i < d.nx && j <= d.ny;
      T uu = 0, uv = 0;
      if (inu) {
        const int q = uidx(d, i, j);
        uu = fmul_add(beta, g.gz[q], g.gr[q]);
        g.gz[q] = uu;
      }
      if (inv) {
        const int q = vidx(d, i, j);
        uv = fmul_add(beta, g.gz[q], g.gr[q]);
        g.gz[q] = uv;
      }
      prolong_store<T, TILE>(d, levels, cf.inner, uu, uv, i0, j0, sm, w);
    }
    if (!grid_barrier<T>(bar, partials, epoch, ss)) return;
    T dot[4] = {T(0), T(0), T(0), T(0)};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
      T cu, cv;
      coarse_apply<T, TILE>(d, levels, cf, wmask, w, i0, j0, sm, cu, cv);
      if (i <= d.nx && j < d.ny) {
        const int q = uidx(d, i, j);
        dot[0] += g.gz[q] * cu;
        g.gp[q] = cu;
      }
      if (i < d.nx && j <= d.ny) {
        const int q = vidx(d, i, j);
        dot[0] += g.gz[q] * cv;
        g.gp[q] = cv;
      }
    }
    if (!grid_sync<1>(bar, partials, epoch, ss, dot, [&](const typename CGReal<T>::type* tot) { cg_alpha<T>(sc, tot); }))
      return;
    const T alpha = sc.alpha_t;
    T rr[4] = {T(0), T(0), T(0), T(0)};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int i0 = (t % ntx) * TILE, j0 = (t / ntx) * TILE, i = i0 + tx, j = j0 + ty;
#pragma unroll
      for (int comp = 0; comp < 2; ++comp) {
        if (comp == 0 ? !(i <= d.nx && j < d.ny) : !(i < d.nx && j <= d.ny)) continue;
        const int q = comp == 0 ? uidx(d, i, j) : vidx(d, i, j);
        xc[q] = fmul_add(alpha, g.gz[q], xc[q]);
        const T r = fmul_add(-alpha, g.gp[q], g.gr[q]);
        g.gr[q] = r;
        rr[0] += r * r;
      }
    }
    ++it;
    if (!grid_sync<1>(bar, partials, epoch, ss, rr, [&](const typename CGReal<T>::type* tot) { cg_next<T>(sc, tot, it, maxit); }))
      return;
  }
  if (blockIdx.x == 0 && tx == 0 && ty == 0) {
    st->cg_it = it;
    st->cg_total += it;
    st->cg_res = cg_final_res(sc);
    st->cg_prev = sc.alpha_prev;
    st->cg_tol = sc.tol;
  }
}

// ------------------------------------------------------------------------------------------------
// Exact diagonal of the coarse operator R A P (a Jacobi preconditioner for the mixed-precision coarse
// solve).  With P e_k = inner ⊙ (φ ⊗ ψ) a Haar basis function and A symmetric, summation by parts of the
// operator's differences gives its quadratic form
//   xᵀ A x = -Σ_h 4 hη (u_x² + v_y² + u_x v_y) - Σ_c hη_c (u_y + v_x)² - Σ β x² + Σ_h dimp (div q)²,
// so diag_k = E(P e_k) is a sum over the cells touching the basis function's support.  One thread per
// basis function of a TILE x TILE block (u and v component each).
// ------------------------------------------------------------------------------------------------
// The 1-D reverse Haar basis function of in-block offset k for a block of `len` existing points
// (len < B at a ragged grid edge): the lifting of the unit vector, as wavelet_matrix builds it.
template <int B>
__device__ __forceinline__ void basis_1d(int k, int len, int levels, float (&phi)[B]) {
#pragma unroll
  for (int p = 0; p < B; ++p) phi[p] = (p == k) ? 1.f : 0.f;
  const int Bl = 1 << (levels + 1);
  for (int lv = 0; lv <= levels; ++lv) {
    const int st = Bl >> lv, half = st >> 1;
#pragma unroll
    for (int o = 0; o < B; ++o) {
      if ((o % st) == 0 && o + half < len) {
        const float xo = phi[o], xe = phi[o + half];
        phi[o + half] = xe + xo;
        phi[o] = xo - xe;
      }
    }
  }
}

template <typename T, int TILE>
__global__ void __launch_bounds__(TILE* TILE)
    k_coarse_diag(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, T* __restrict__ dc) {
  __shared__ T s_heh[TILE + 1][TILE + 1], s_hec[TILE + 1][TILE + 1], s_dim[TILE + 1][TILE + 1];
  const int bx0 = blockIdx.x * TILE, by0 = blockIdx.y * TILE, tx = threadIdx.x, ty = threadIdx.y;
  // h cells / c points [bx0-1, bx0+TILE) x [by0-1, by0+TILE) at local index +1
  for (int p = tx + TILE * ty; p < (TILE + 1) * (TILE + 1); p += TILE * TILE) {
    const int la = p % (TILE + 1), lb = p / (TILE + 1), a = bx0 - 1 + la, b = by0 - 1 + lb;
    const bool hv = a >= 0 && a < d.nx && b >= 0 && b < d.ny;
    const bool cv = a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1;
    s_heh[lb][la] = hv ? cf.heta_h[hidx(d, a, b)] : (T)0;
    s_dim[lb][la] = hv ? cf.dimp[hidx(d, a, b)] : (T)0;
    s_hec[lb][la] = cv ? cf.heta_c[cidx(d, a, b)] : (T)0;
  }
  __syncthreads();
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  for (int comp = 0; comp < 2; ++comp) {
    const int nxg = comp == 0 ? d.nx + 1 : d.nx, nyg = comp == 0 ? d.ny : d.ny + 1;
    const int i = bx0 + tx, j = by0 + ty;
    if (i >= nxg || j >= nyg) continue;
    const int lenx = min(TILE, nxg - bx0), leny = min(TILE, nyg - by0);
    float phi[TILE], psi[TILE];
    basis_1d<TILE>(tx, lenx, levels, phi);
    basis_1d<TILE>(ty, leny, levels, psi);
    auto gq = [&](int gi, int gj) { return comp == 0 ? uidx(d, gi, gj) : vidx(d, gi, gj); };
    // x at block-local (p, r); zero outside the block, off the grid, or off the interior
    auto xval = [&](int p, int r) -> T {
      if (p < 0 || p >= lenx || r < 0 || r >= leny) return (T)0;
      const float s = phi[p] * psi[r];
      if (s == 0.f) return (T)0;
      return cf.inner[gq(bx0 + p, by0 + r)] ? (T)s : (T)0;
    };
    auto hm = [&](int p, int r) -> T {  // h_m at block-local (p, r) (0 off the block: x is 0 there)
      if (p < 0 || p >= lenx || r < 0 || r >= leny) return (T)0;
      return cf.h_m[gq(bx0 + p, by0 + r)];
    };
    int p0 = TILE, p1 = -1, r0 = TILE, r1 = -1;  // support bounds
    for (int p = 0; p < lenx; ++p)
      if (phi[p] != 0.f) { p0 = min(p0, p); p1 = max(p1, p); }
    for (int r = 0; r < leny; ++r)
      if (psi[r] != 0.f) { r0 = min(r0, r); r1 = max(r1, r); }
    T e = (T)0;
    if (comp == 0) {
      // h cells (a, r) with a = bx0 + p - 1 .. : u_x = x(p) - x(p-1) over the cell between u points p-1, p
      for (int r = r0; r <= r1; ++r)
        for (int p = p0; p <= p1 + 1; ++p) {  // cell between u points p-1 and p  (h index bx0 + p - 1)
          const T ux = (xval(p, r) - xval(p - 1, r)) * rdx;
          const T dq = (hm(p, r) * xval(p, r) - hm(p - 1, r) * xval(p - 1, r)) * rdx;
          const int la = p, lb = r + 1;  // smem index of h cell (bx0 + p - 1, by0 + r)
          e += s_dim[lb][la] * dq * dq - (T)4 * s_heh[lb][la] * ux * ux;
        }
      // c points (a, b) = (bx0 + p - 1, by0 + r - 1): u_y = x(p, r) - x(p, r-1)
      for (int r = r0; r <= r1 + 1; ++r)
        for (int p = p0; p <= p1; ++p) {
          const T uy = (xval(p, r) - xval(p, r - 1)) * rdy;
          e -= s_hec[r][p] * uy * uy;
        }
    } else {
      // h cells (p, b) between v points r-1 and r: v_y
      for (int r = r0; r <= r1 + 1; ++r)
        for (int p = p0; p <= p1; ++p) {
          const T vy = (xval(p, r) - xval(p, r - 1)) * rdy;
          const T dq = (hm(p, r) * xval(p, r) - hm(p, r - 1) * xval(p, r - 1)) * rdy;
          const int la = p + 1, lb = r;  // h cell (bx0 + p, by0 + r - 1)
          e += s_dim[lb][la] * dq * dq - (T)4 * s_heh[lb][la] * vy * vy;
        }
      // c points (a, b) = (bx0 + p - 1, by0 + r - 1): v_x = y(p, r) - y(p-1, r)
      for (int r = r0; r <= r1; ++r)
        for (int p = p0; p <= p1 + 1; ++p) {
          const T vx = (xval(p, r) - xval(p - 1, r)) * rdx;
          e -= s_hec[r][p] * vx * vx;
        }
    }
    for (int r = r0; r <= r1; ++r)
      for (int p = p0; p <= p1; ++p) {
        const T x = xval(p, r);
        if (x != (T)0) e -= cf.beta_m[gq(bx0 + p, by0 + r)] * x * x;
      }
    const int q = gq(i, j);
    dc[q] = wmask[q] ? e : (T)0;
  }
}

// k_coarse_diag for 16 x 16 tiles, separated.  A basis function is x = inner ⊙ (φ ⊗ ψ) on its block, so
// a difference along x is ψ(r) (inner φ)(p) - ψ(r) (inner φ)(p-1) and one along y is φ(p) times the
// difference of inner ψ; every term of the quadratic form is therefore ψ(r)² times a sum over the row r
// that depends on φ alone, or φ(p)² times a sum over the column p that depends on ψ alone:
//   diag(φ_kx ⊗ ψ_ky) = Σ_r ψ_ky(r)² X[kx][r] + Σ_p φ_kx(p)² Y[ky][p].
// u: X holds the u_x, div q and β terms, Y the u_y term; v: Y holds v_y and div q, X the v_x and β terms.
// Each thread builds one entry of X and one of Y (sums over 17 positions), then evaluates its own basis
// function (32 terms): O(TILE) work per function instead of k_coarse_diag's O(support area), the same
// terms added in another order.
template <typename T, int TILE>
__global__ void __launch_bounds__(TILE* TILE)
    k_coarse_diag_sep(Dims d, int levels, OpCoef<T> cf, const uint8_t* __restrict__ wmask, T* __restrict__ dc) {
  __shared__ T s_heh[TILE + 1][TILE + 1], s_hec[TILE + 1][TILE + 1], s_dim[TILE + 1][TILE + 1];
  __shared__ float s_basis[2][TILE][TILE + 1];  // [along x, along y][offset][position]
  __shared__ T s_in[TILE][TILE + 1], s_hm[TILE][TILE + 1], s_beta[TILE][TILE + 1];  // [r][p] on the block
  __shared__ T s_x[TILE][TILE + 1], s_y[TILE][TILE + 1];                           // X[kx][r], Y[ky][p]
  const int bx0 = blockIdx.x * TILE, by0 = blockIdx.y * TILE, tx = threadIdx.x, ty = threadIdx.y;
  for (int p = tx + TILE * ty; p < (TILE + 1) * (TILE + 1); p += TILE * TILE) {
    const int la = p % (TILE + 1), lb = p / (TILE + 1), a = bx0 - 1 + la, b = by0 - 1 + lb;
    const bool hv = a >= 0 && a < d.nx && b >= 0 && b < d.ny;
    const bool cv = a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1;
    s_heh[lb][la] = hv ? cf.heta_h[hidx(d, a, b)] : (T)0;
    s_dim[lb][la] = hv ? cf.dimp[hidx(d, a, b)] : (T)0;
    s_hec[lb][la] = cv ? cf.heta_c[cidx(d, a, b)] : (T)0;
  }
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d), rdx2 = rdx * rdx, rdy2 = rdy * rdy;
  for (int comp = 0; comp < 2; ++comp) {
    const int nxg = comp == 0 ? d.nx + 1 : d.nx, nyg = comp == 0 ? d.ny : d.ny + 1;
    const int lenx = min(TILE, nxg - bx0), leny = min(TILE, nyg - by0);
    auto gq = [&](int gi, int gj) { return comp == 0 ? uidx(d, gi, gj) : vidx(d, gi, gj); };
    __syncthreads();  // the previous component's tables are no longer read
    if (ty < 2) {
      float b[TILE];
      basis_1d<TILE>(tx, ty == 0 ? lenx : leny, levels, b);
#pragma unroll
      for (int p = 0; p < TILE; ++p) s_basis[ty][tx][p] = b[p];
    }
    {
      const bool on = tx < lenx && ty < leny;
      const int q = on ? gq(bx0 + tx, by0 + ty) : 0;
      s_in[ty][tx] = (on && cf.inner[q]) ? (T)1 : (T)0;
      s_hm[ty][tx] = on ? cf.h_m[q] : (T)0;
      s_beta[ty][tx] = on ? cf.beta_m[q] : (T)0;
    }
    __syncthreads();
    // (inner φ_k)(p) in row r and (inner ψ_k)(r) in column p; zero off the block
    auto ix = [&](int k, int p, int r) -> T {
      return (p >= 0 && p < lenx && r >= 0 && r < leny) ? s_in[r][p] * (T)s_basis[0][k][p] : (T)0;
    };
    auto iy = [&](int k, int p, int r) -> T {
      return (p >= 0 && p < lenx && r >= 0 && r < leny) ? s_in[r][p] * (T)s_basis[1][k][r] : (T)0;
    };
    auto hmb = [&](int p, int r) -> T { return (p >= 0 && p < lenx && r >= 0 && r < leny) ? s_hm[r][p] : (T)0; };
    {
      // thread (tx, ty): X[kx = tx][r = ty] and Y[ky = tx][p = ty]
      const int k = tx;
      T xs = 0, ys = 0;
      if (comp == 0) {
        const int r = ty;
        T a = 0, bsum = 0;
        for (int p = 0; p <= TILE; ++p) {  // h cell between u points p-1, p of row r
          const T dxv = ix(k, p, r) - ix(k, p - 1, r);
          const T dqv = hmb(p, r) * ix(k, p, r) - hmb(p - 1, r) * ix(k, p - 1, r);
          a += s_dim[r + 1][p] * dqv * dqv - (T)4 * s_heh[r + 1][p] * dxv * dxv;
        }
        for (int p = 0; p < TILE; ++p) {
          const T f = (T)s_basis[0][k][p];
          bsum += (r < leny && p < lenx) ? s_beta[r][p] * s_in[r][p] * f * f : (T)0;
        }
        xs = rdx2 * a - bsum;
        const int p = ty;
        T c = 0;
        for (int rr = 0; rr <= TILE; ++rr) {  // c point between u points (p, rr-1), (p, rr)
          const T dyv = iy(k, p, rr) - iy(k, p, rr - 1);
          c += s_hec[rr][p] * dyv * dyv;
        }
        ys = -rdy2 * c;
      } else {
        const int p = ty;
        T a = 0;
        for (int rr = 0; rr <= TILE; ++rr) {  // h cell between v points (p, rr-1), (p, rr)
          const T dyv = iy(k, p, rr) - iy(k, p, rr - 1);
          const T dqv = hmb(p, rr) * iy(k, p, rr) - hmb(p, rr - 1) * iy(k, p, rr - 1);
          a += s_dim[rr][p + 1] * dqv * dqv - (T)4 * s_heh[rr][p + 1] * dyv * dyv;
        }
        ys = rdy2 * a;
        const int r = ty;
        T c = 0, bsum = 0;
        for (int pp = 0; pp <= TILE; ++pp) {  // c point between v points (pp-1, r), (pp, r)
          const T dxv = ix(k, pp, r) - ix(k, pp - 1, r);
          c += s_hec[r][pp] * dxv * dxv;
        }
        for (int pp = 0; pp < TILE; ++pp) {
          const T f = (T)s_basis[0][k][pp];
          bsum += (r < leny && pp < lenx) ? s_beta[r][pp] * s_in[r][pp] * f * f : (T)0;
        }
        xs = -rdx2 * c - bsum;
      }
      s_x[k][ty] = xs;
      s_y[k][ty] = ys;
    }
    __syncthreads();
    const int i = bx0 + tx, j = by0 + ty;
    if (i >= nxg || j >= nyg) continue;  // (no __syncthreads below in this component)
    T e = 0;
    for (int r = 0; r < TILE; ++r) {
      const T ps = (T)s_basis[1][ty][r];
      e += ps * ps * s_x[tx][r];
    }
    for (int p = 0; p < TILE; ++p) {
      const T ph = (T)s_basis[0][tx][p];
      e += ph * ph * s_y[ty][p];
    }
    const int q = gq(i, j);
    dc[q] = wmask[q] ? e : (T)0;
  }
}

// Self-test of the bounded waits: one thread waits, with wait_tagged, for a word that nothing writes;
// out = 1 if the wait gave up (it also sets bar->err, which the caller clears).
static __global__ void k_selftest_wait(GridBar* bar, const unsigned long long* __restrict__ word, int* out) {
  __shared__ int fail;
  if (threadIdx.x == 0) {
    fail = 0;
    wait_tagged(word, 1u, bar, &fail);
    *out = fail;
  }
}

// Before a persistent CG: an idle barrier (count 0, no error).
// Before each persistent launch: restart the arrival counter, clear the error, and advance the tag
// generation past every tag the previous launch can have written (at most ~cheb (maxiter_coarse + 1) + 5
// tagged exchanges, cheb <= 8; 2^21 tags per generation step).
static __global__ void k_reset_barrier(GridBar* bar, const DevParams* __restrict__ P) {
  if (threadIdx.x == 0) {
    bar->count = 0u;
    bar->err = 0;
    bar->gen += 1u + ((unsigned)max(P->maxiter_coarse, 0) >> 16);
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
