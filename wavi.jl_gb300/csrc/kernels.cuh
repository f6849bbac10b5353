// kernels.cuh — sm_103a kernels of the WAVI velocity solve.
//
// Data layout (HBM): every field is a full rectangle, column-major with x fastest, exactly the
// reference's Julia layout (src/Fields/*.jl): h grid nx*ny, u grid (nx+1)*ny, v grid nx*(ny+1),
// c grid (nx-1)*(ny-1).  Solver vectors are one buffer [u part (Nu) | v part (Nv)] of full rectangles
// that are zero off the interior mask, which replaces the reference's sampled vectors
// (samp_inner / spread_inner, src/Fields/UGrid.jl:79-82) without any gather or scatter.  The adaptive
// wavelet coarse space is the same layout with the wavelet mask (src/Wavelets/UWavelets.jl).
//
// Precision: templates on T (float or double) for everything inside the V-cycle; reductions always
// accumulate in double.  The Picard residual uses the double instantiation.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace wavi {

constexpr int OP_TX = 32;  // operator tile: 32 x 8 points of the (nx+1) x (ny+1) index space
constexpr int OP_TY = 8;
constexpr int RED_THREADS = 256;

struct Dims {
  int nx, ny, ns;
  int Nh, Nu, Nv, Nc, N;
  double dx, dy, rdx, rdy;
  float rdx_f, rdy_f;  // FP32 copies: a per-thread FP64 -> FP32 conversion runs on GB300's slow FP64 pipe
};

// 1/dx and 1/dy in the kernel's arithmetic type.
template <typename T>
__device__ __forceinline__ T rdx_of(const Dims& d) {
  return (T)d.rdx;
}
template <>
__device__ __forceinline__ float rdx_of<float>(const Dims& d) {
  return d.rdx_f;
}
template <typename T>
__device__ __forceinline__ T rdy_of(const Dims& d) {
  return (T)d.rdy;
}
template <>
__device__ __forceinline__ float rdy_of<float>(const Dims& d) {
  return d.rdy_f;
}

__device__ __forceinline__ int hidx(const Dims& d, int i, int j) { return i + d.nx * j; }
__device__ __forceinline__ int uidx(const Dims& d, int i, int j) { return i + (d.nx + 1) * j; }
__device__ __forceinline__ int vidx(const Dims& d, int i, int j) { return d.Nu + i + d.nx * j; }  // in uv buffers
__device__ __forceinline__ int cidx(const Dims& d, int i, int j) { return i + (d.nx - 1) * j; }

// Coefficients of the linearised operator (update_rheological_operators!, update_velocities.jl:374-383),
// with the reference's crops folded in:  heta_h = h_mask*h*ηav,  heta_c = c_mask*cent_xy(h*ηav),
// dimp = h_mask*(-ρ g θ dt dsdh),  beta_m = mask*βeff (u|v),  h_m = mask*h (u|v),  inner = mask_inner (u|v).
template <typename T>
struct OpCoef {
  const T* heta_h;
  const T* heta_c;
  const T* dimp;
  const T* beta_m;
  const T* h_m;
  const uint8_t* inner;
};

// ------------------------------------------------------------------------------------------------
// Block reduction (deterministic for a fixed launch shape)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// Sum over the block; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < nw ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}
__device__ __forceinline__ double block_sum_2d(double v, double* sh) {
  // flattened thread index for 2-D blocks
  const int t = threadIdx.x + blockDim.x * threadIdx.y;
  const int nt = blockDim.x * blockDim.y;
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
  return r;
}

// Sum partials[0..n) into *out (one block, fixed order).
static __global__ void k_reduce(const double* __restrict__ partials, int n, double* __restrict__ out) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partials[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = s;
}

// ------------------------------------------------------------------------------------------------
// The matrix-free momentum operator (op_fun!, src/utilities.jl:61-145), tiled.
//
// Output point (i,j) of the (nx+1) x (ny+1) index space holds fx at u(i,j) (j < ny) and fy at v(i,j)
// (i < nx).  Phase 1 computes, for the tile plus a one-point halo on the low side, the h-cell stresses
// Rxx = 2hη(2u_x+v_y), Ryy = 2hη(2v_y+u_x), the Schur-complement term E = dimp*div(h u), and the c-point
// shear stress Rxy = hη_c (u_y+v_x), into shared memory.  Phase 2 takes the divergences:
//   fx = (Rxx(i)-Rxx(i-1))/dx + (Rxy(i-1,j)-Rxy(i-1,j-1))/dy - β_u u - h_u (E(i)-E(i-1))/dx
//   fy = (Ryy(j)-Ryy(j-1))/dy + (Rxy(i,j-1)-Rxy(i-1,j-1))/dx - β_v v - h_v (E(j)-E(j-1))/dy
// sampled at the interior mask.  Terms outside the grid are zero, as in the reference's sparse
// transposes.  MODE 0: y = A x.  MODE 1: y = b - A x with a partial sum of y^2 per block.
// ------------------------------------------------------------------------------------------------
template <typename T, typename TI, int MODE>
__global__ void __launch_bounds__(OP_TX* OP_TY)
    k_op(Dims d, OpCoef<T> cf, const TI* __restrict__ x, const T* __restrict__ b, T* __restrict__ y,
         double* __restrict__ partials, const int* __restrict__ skip) {
  if (skip && *skip) return;
  __shared__ T sRxx[OP_TY + 1][OP_TX + 1];
  __shared__ T sRyy[OP_TY + 1][OP_TX + 1];
  __shared__ T sE[OP_TY + 1][OP_TX + 1];
  __shared__ T sRxy[OP_TY + 1][OP_TX + 1];
  const int i0 = blockIdx.x * OP_TX, j0 = blockIdx.y * OP_TY;
  const int tid = threadIdx.x + OP_TX * threadIdx.y;
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d);
  const TI* xu = x;
  for (int p = tid; p < (OP_TX + 1) * (OP_TY + 1); p += OP_TX * OP_TY) {
    const int li = p % (OP_TX + 1), lj = p / (OP_TX + 1);
    const int a = i0 - 1 + li, bb = j0 - 1 + lj;
    T rxx = 0, ryy = 0, e = 0, rxy = 0;
    if (a >= 0 && a < d.nx && bb >= 0 && bb < d.ny) {
      const int hc = hidx(d, a, bb);
      const T u0 = (T)xu[uidx(d, a, bb)], u1 = (T)xu[uidx(d, a + 1, bb)];
      const T v0 = (T)xu[vidx(d, a, bb)], v1 = (T)xu[vidx(d, a, bb + 1)];
      const T ux = (u1 - u0) * rdx, vy = (v1 - v0) * rdy;
      const T he2 = (T)2 * cf.heta_h[hc];
      rxx = he2 * ((T)2 * ux + vy);
      ryy = he2 * ((T)2 * vy + ux);
      const T divq = (cf.h_m[uidx(d, a + 1, bb)] * u1 - cf.h_m[uidx(d, a, bb)] * u0) * rdx +
                     (cf.h_m[vidx(d, a, bb + 1)] * v1 - cf.h_m[vidx(d, a, bb)] * v0) * rdy;
      e = cf.dimp[hc] * divq;
    }
    if (a >= 0 && a < d.nx - 1 && bb >= 0 && bb < d.ny - 1) {
      const T hc = cf.heta_c[cidx(d, a, bb)];
      if (hc != (T)0) {
        const T uy = ((T)xu[uidx(d, a + 1, bb + 1)] - (T)xu[uidx(d, a + 1, bb)]) * rdy;
        const T vx = ((T)xu[vidx(d, a + 1, bb + 1)] - (T)xu[vidx(d, a, bb + 1)]) * rdx;
        rxy = hc * (uy + vx);
      }
    }
    sRxx[lj][li] = rxx;
    sRyy[lj][li] = ryy;
    sE[lj][li] = e;
    sRxy[lj][li] = rxy;
  }
  __syncthreads();
  const int li = threadIdx.x + 1, lj = threadIdx.y + 1;
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  double acc = 0.0;
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    T f = 0;
    if (cf.inner[q]) {
      f = (sRxx[lj][li] - sRxx[lj][li - 1]) * rdx + (sRxy[lj][li - 1] - sRxy[lj - 1][li - 1]) * rdy -
          cf.beta_m[q] * (T)xu[q] - cf.h_m[q] * ((sE[lj][li] - sE[lj][li - 1]) * rdx);
      if (MODE == 1) f = b[q] - f;
    }
    y[q] = f;
    if (MODE == 1) acc += (double)f * (double)f;
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    T f = 0;
    if (cf.inner[q]) {
      f = (sRyy[lj][li] - sRyy[lj - 1][li]) * rdy + (sRxy[lj - 1][li] - sRxy[lj - 1][li - 1]) * rdx -
          cf.beta_m[q] * (T)xu[q] - cf.h_m[q] * ((sE[lj][li] - sE[lj - 1][li]) * rdy);
      if (MODE == 1) f = b[q] - f;
    }
    y[q] = f;
    if (MODE == 1) acc += (double)f * (double)f;
  }
  if (MODE == 1) {
    __shared__ double sh[32];
    double s = block_sum_2d(acc, sh);
    if (tid == 0) partials[blockIdx.x + gridDim.x * blockIdx.y] = s;
  }
}

// Diagonal of the operator at the interior points (closed form of op_fun! applied to a unit vector;
// replaces the coloured probing of get_op_diag, update_preconditioners.jl:92-109).
template <typename T>
__global__ void k_op_diag(Dims d, OpCoef<T> cf, T* __restrict__ diag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const T rdx = rdx_of<T>(d), rdy = rdy_of<T>(d), rdx2 = rdx * rdx, rdy2 = rdy * rdy;
  auto heh = [&](int a, int b) -> T { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny) ? cf.heta_h[hidx(d, a, b)] : (T)0; };
  auto dim = [&](int a, int b) -> T { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny) ? cf.dimp[hidx(d, a, b)] : (T)0; };
  auto hec = [&](int a, int b) -> T {
    return (a >= 0 && a < d.nx - 1 && b >= 0 && b < d.ny - 1) ? cf.heta_c[cidx(d, a, b)] : (T)0;
  };
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
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
    T v = 0;
    if (cf.inner[q]) {
      const T hv = cf.h_m[q];
      v = -(T)4 * rdy2 * (heh(i, j) + heh(i, j - 1)) - rdx2 * (hec(i, j - 1) + hec(i - 1, j - 1)) - cf.beta_m[q] +
          hv * hv * rdy2 * (dim(i, j) + dim(i, j - 1));
    }
    diag[q] = v;
  }
}

// ------------------------------------------------------------------------------------------------
// Relinearisation on the h grid (inner_update!, update_velocities.jl:32-45): strain rate :202-209,
// depth-averaged speed :216-220, bed speed :227-231, Weertman β :238-243, basal drag :251-255,
// two fixed-point sweeps of the σ-level Glen viscosity :264-283, quadratures :292-328, βeff :335-339,
// and the h-grid operator coefficients :374-383.  TR is the arithmetic type of the viscosity sweeps.
// ------------------------------------------------------------------------------------------------
// Device-side copy of the per-solve scalars, read by the kernels through a pointer so that a captured
// CUDA graph never freezes a parameter value (Params.jl / SolverParams.jl members used by the solve).
struct DevParams {
  double weertman_m, weertman_reg_speed, glen_n, glen_reg_strain_rate;
  double c0;        // -ρ g θ dt  (update_rheological_operators!, update_velocities.jl:381)
  double rho_i, rho_w, g, sea_level, theta_dt;
  double tol_picard, tol_coarse, omega;
  int maxiter_picard, maxiter_coarse, nsmooth, n_iter_viscosity;
  int picard_test;
  int aa_depth;         // Anderson acceleration of the Picard loop: columns (0: the reference's iteration)
  int coarse_forcing;   // 1: the coarse CG's relative tolerance follows the Picard residual (coarse_tolerance)
  double aa_start_rel;  // ... from the first Picard iteration whose relative residual is below this
  // the float relinearisation's uniform constants, rounded once on the host: 1/m - 1, 1/n - 1 (the
  // exponents of β and of the viscosity), the squared strain-rate regularisation, the speed regularisation
  float weertman_ex_f, glen_ex_f, glen_er2_f, weertman_reg_speed_f;
};

// IEEE 754 conversions between binary64 and binary32 by integer operations: binary64 -> binary32 rounds to
// nearest, ties to even (subnormal results, overflow to infinity, NaN stays NaN); binary32 -> binary64 is
// exact.  GB300 runs the hardware conversions (cvt.rn.f32.f64, cvt.f64.f32) on its FP64 pipe at about one
// per SM and cycle, where these take a dozen integer operations on the integer pipes; the float
// relinearisation converts ~50 values per cell between the caller's FP64 fields and float.  Their results
// equal the hardware conversions bit for bit (NaN: any NaN), checked by wavi_selftest_conversions.
static __device__ __noinline__ float f32_rn_bits_general(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu);
  const unsigned long long m = b & 0xfffffffffffffull;
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));  // ±inf, NaN
  const int ef = e - 1023 + 127;  // the binary32 biased exponent of a normal result
  if (ef >= 0xff) return __uint_as_float(sign | 0x7f800000u);
  if (ef <= 0) {
    // below 2^-126: a subnormal binary32 (or zero), k·2^-149 with k < 2^23, from the 53-bit significand
    if (ef < -24) return __uint_as_float(sign);  // below 2^-150: rounds to zero
    const unsigned long long sig = m | (1ull << 52);
    const int drop = 30 - ef;  // 30..54 bits dropped
    const unsigned long long rem = sig & ((1ull << drop) - 1ull), half = 1ull << (drop - 1);
    unsigned k = (unsigned)(sig >> drop);
    if (rem > half || (rem == half && (k & 1u))) ++k;  // a carry into bit 23 gives the smallest normal
    return __uint_as_float(sign | k);
  }
  unsigned r = ((unsigned)ef << 23) | (unsigned)(m >> 29);
  const unsigned rem = (unsigned)(m & 0x1fffffffull);
  if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ++r;  // a carry may reach the exponent (or inf)
  return __uint_as_float(sign | r);
}
static __device__ __noinline__ double f64_exact_bits_general(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  unsigned long long r;
  if (e == 0xffu) {
    r = sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29);  // ±inf, NaN (payload kept)
  } else if (e != 0u) {
    r = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
  } else if (m == 0u) {
    r = sign;  // ±0
  } else {
    // subnormal binary32 m·2^-149 with its leading one at bit p: a normal binary64 1.f·2^(p-149)
    const int p = 31 - __clz((int)m);
    const unsigned f = (m << (23 - p)) & 0x7fffffu;
    r = sign | ((unsigned long long)(1023 + p - 149) << 52) | ((unsigned long long)f << 29);
  }
  return __longlong_as_double((long long)r);
}

struct RelinIn {
  const double* uv;      // velocities (u | v), full rectangles
  const uint8_t* mask;   // u mask | v mask
  const uint8_t* h_mask;
  const uint8_t* c_mask;
  const double* h;
  const double* wc;      // weertman_c (C * grounded fraction)
  const double* glen_b;  // nx*ny*ns
  const double* dsdh;
  const double* zeta;    // ns (device)
  const double* qw;      // ns (device)
  const DevParams* P;
  const float* zeta_f;   // ns: zeta and qw rounded to float (the float relinearisation)
  const float* qw_f;
};
struct RelinOut {
  double *shelf_strain_rate, *av_speed, *bed_speed, *beta, *tau_bed, *eta, *eta_av, *quad_f1, *quad_f2, *beta_eff;
  double* heta_h64;  // h_mask*h*ηav
  double* dimp64;
  float* heta_h32;
  float* dimp32;
  double* hn;        // h*ηav (all cells) for the c-grid centring
};

// The conversions a kernel calls: the common cases (results in binary32's normal range, zeros) on the two
// 32-bit halves of the binary64 pattern in a few integer operations, the rest (subnormal, infinite and NaN
// results, overflow) in the general forms above.
__device__ __forceinline__ float f32_rn_bits(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ahi = hi & 0x7fffffffu;
  if (ahi - 0x38100000u < 0x47f00000u - 0x38100000u) {  // biased exponent 897..1150: a normal binary32
    // (e - 896) << 23 | the top 23 mantissa bits, rounded to nearest even on the 29 dropped bits (a carry
    // may reach the exponent, up to infinity)
    unsigned r = ((ahi - 0x38000000u) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    r += (rem + (r & 1u)) > 0x10000000u;
    return __uint_as_float(r | (hi & 0x80000000u));
  }
  if ((ahi | lo) == 0u) return __uint_as_float(hi & 0x80000000u);  // ±0
  return f32_rn_bits_general(x);
}
__device__ __forceinline__ double f64_exact_bits(float x) {
  const unsigned b = __float_as_uint(x), e = (b >> 23) & 0xffu;
  if (e - 1u < 254u)  // normal: the exponent rebiased by 1023 - 127 = 896, the mantissa moved up by 29 bits
    return __hiloint2double((int)((b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + 0x38000000u)), (int)(b << 29));
  if ((b & 0x7fffffffu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);  // ±0
  return f64_exact_bits_general(x);
}

// Self-test of f32_rn_bits and f64_exact_bits against the hardware conversions over n hashed bit patterns
// of each width: binary64 patterns over every exponent, every other one with its exponent within binary32's
// range ± 30 binades (subnormal, normal and overflowing results) and every fourth an exact rounding tie;
// binary32 patterns over every exponent.  Adds the mismatches (two NaNs agree) to *bad.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {  // SplitMix64's finaliser
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static __global__ void k_selftest_conversions(long long n, unsigned long long* bad) {
  unsigned long long local = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const unsigned long long h = mix64(0x9e3779b97f4a7c15ull * (unsigned long long)(k + 1));
    unsigned long long b = h;
    if (k & 1) {
      const unsigned long long e = 1023 - 160 + mix64(h) % 290;
      b = (b & 0x800fffffffffffffull) | (e << 52);
      if (k & 2) b = (b & ~0x1fffffffull) | 0x10000000ull;
    }
    const double x = __longlong_as_double((long long)b);
    const float a = f32_rn_bits(x), hw = __double2float_rn(x);
    local += !(__float_as_uint(a) == __float_as_uint(hw) || (isnan(a) && isnan(hw)));
    const float f = __uint_as_float((unsigned)(h >> 17));
    const double a2 = f64_exact_bits(f), hw2 = (double)f;
    local += !(__double_as_longlong(a2) == __double_as_longlong(hw2) || (isnan(a2) && isnan(hw2)));
  }
  if (local) atomicAdd(bad, local);
}

template <typename TR>
__device__ __forceinline__ TR powT(TR a, TR b);
template <>
__device__ __forceinline__ double powT<double>(double a, double b) { return pow(a, b); }
template <>
__device__ __forceinline__ float powT<float>(float a, float b) { return powf(a, b); }

// The float relinearisation of one h cell after its strain rate ssr and centred speed avs (both zero off
// the ice): drag (update_β!, update_basal_drag!), the σ-level viscosity sweeps (update_viscosity!), the
// quadratures (update_av_viscosity!, update_quadrature_f1/f2!) and βeff, with the FP64 fields converted by
// integer operations.
__device__ __forceinline__ void relin_h_float_cell(const Dims& d, const RelinIn& in, const RelinOut& out, int c,
                                                   float ssr, float avs, bool hm) {
  const DevParams* P = in.P;
  const float f2_prev = f32_rn_bits(out.quad_f2[c]), beta_prev = f32_rn_bits(out.beta[c]);
  const float bs = avs / (1.0f + f2_prev * beta_prev);
  const float ur = P->weertman_reg_speed_f;
  const float beta = f32_rn_bits(in.wc[c]) * powf(sqrtf(bs * bs + ur * ur), P->weertman_ex_f);
  const float tau = beta * bs;
  out.shelf_strain_rate[c] = f64_exact_bits(ssr);
  out.av_speed[c] = f64_exact_bits(avs);
  out.bed_speed[c] = f64_exact_bits(bs);
  out.beta[c] = f64_exact_bits(beta);
  out.tau_bed[c] = f64_exact_bits(tau);
  const float hh = f32_rn_bits(in.h[c]);
  float eav = 0.0f, f1 = 0.0f, f2 = 0.0f;
  if (hm) {
    const float ex = P->glen_ex_f, er2 = P->glen_er2_f;
    const int n_iter_viscosity = P->n_iter_viscosity;
    const float e2 = ssr * ssr;
    for (int k = 0; k < d.ns; ++k) {
      const size_t q = (size_t)c + (size_t)d.Nh * k;
      float eta = f32_rn_bits(out.eta[q]);
      const float B = f32_rn_bits(in.glen_b[q]), zk = in.zeta_f[k], wk = in.qw_f[k];
      const float tz = tau * zk;
      for (int it = 0; it < n_iter_viscosity; ++it) {
        const float t = tz / eta;
        eta = 0.5f * B * powf(sqrtf(e2 + 0.25f * (t * t) + er2), ex);
      }
      out.eta[q] = f64_exact_bits(eta);
      const float ie = 1.0f / eta, hz = wk * hh * zk * ie;
      eav += wk * eta;
      f1 += hz;
      f2 += hz * zk;
    }
  }
  out.eta_av[c] = f64_exact_bits(eav);
  out.quad_f1[c] = f64_exact_bits(f1);
  out.quad_f2[c] = f64_exact_bits(f2);
  out.beta_eff[c] = f64_exact_bits(beta / (1.0f + f2 * beta));
  const float hn = hh * eav;
  out.hn[c] = f64_exact_bits(hn);
  const float hh_m = hm ? hn : 0.0f;
  const double dm = hm ? P->c0 * in.dsdh[c] : 0.0;
  out.heta_h64[c] = f64_exact_bits(hh_m);
  out.dimp64[c] = dm;
  if (out.heta_h32) {
    out.heta_h32[c] = hh_m;
    out.dimp32[c] = f32_rn_bits(dm);
  }
}

template <typename TR>
__global__ void k_relin_h(Dims d, RelinIn in, RelinOut out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const int i = c % d.nx, j = c / d.nx;
  const double* U = in.uv;
  auto um = [&](int a, int b) { int q = uidx(d, a, b); return in.mask[q] ? U[q] : 0.0; };
  auto vm = [&](int a, int b) { int q = vidx(d, a, b); return in.mask[q] ? U[q] : 0.0; };
  const bool hm = in.h_mask[c];
  // strain-rate components (masked velocities: gu.crop*gu.u)
  const double u0 = um(i, j), u1 = um(i + 1, j), v0 = vm(i, j), v1 = vm(i, j + 1);
  if constexpr (std::is_same<TR, float>::value) {
    // FP32 viscosity sweeps (mixed precision): η carries float precision, so everything after the velocity
    // differences runs in float too — speeds, β (powf), the sweeps, one reciprocal of η per level for the
    // quadratures, βeff.  FP64 arithmetic is left only where float would lose the result: the differences
    // of neighbouring velocities (each rounded to float afterwards) and the FP64 coefficient c0·∂s/∂h.
    // Every load and store of an FP64 field converts by integer operations (f32_rn_bits, f64_exact_bits):
    // GB300's FP64 pipe, which the hardware conversions use, bounded this kernel.
    if (hm) {
      const float rdx = f32_rn_bits(d.rdx), rdy = f32_rn_bits(d.rdy);
      const float fx = f32_rn_bits(u1 - u0) * rdx, fy = f32_rn_bits(v1 - v0) * rdy;
      float sx[2] = {0.0f, 0.0f};
      for (int tb = 0; tb < 2; ++tb) {
        const int cb = j - 1 + tb;
        float acc = 0.0f;
        for (int ta = 0; ta < 2; ++ta) {
          const int ca = i - 1 + ta;
          if (ca < 0 || ca >= d.nx - 1 || cb < 0 || cb >= d.ny - 1) continue;
          if (!in.c_mask[cidx(d, ca, cb)]) continue;
          const float uy = f32_rn_bits(um(ca + 1, cb + 1) - um(ca + 1, cb)) * rdy;
          const float vx = f32_rn_bits(vm(ca + 1, cb + 1) - vm(ca, cb + 1)) * rdx;
          acc += 0.5f * (uy + vx);
        }
        sx[tb] = acc;
      }
      const float fs = 0.5f * sx[0] + 0.5f * sx[1];
      const float ssr = sqrtf(fx * fx + fy * fy + fx * fy + 0.25f * (fs * fs));
      const float uc = 0.5f * f32_rn_bits(u0 + u1), vc = 0.5f * f32_rn_bits(v0 + v1);
      relin_h_float_cell(d, in, out, c, ssr, sqrtf(uc * uc + vc * vc), true);
    } else {
      relin_h_float_cell(d, in, out, c, 0.0f, 0.0f, false);
    }
    return;
  }
  const double ux = hm ? (u1 * d.rdx - u0 * d.rdx) : 0.0;
  const double vy = hm ? (v1 * d.rdy - v0 * d.rdy) : 0.0;
  // c -> h average of the c-masked shear at the up-to-four surrounding corners (CGrid.jl:45)
  double shear = 0.0;
  if (hm) {
    double sx[2] = {0.0, 0.0};
    for (int tb = 0; tb < 2; ++tb) {
      const int cb = j - 1 + tb;
      double acc = 0.0;
      for (int ta = 0; ta < 2; ++ta) {
        const int ca = i - 1 + ta;
        if (ca < 0 || ca >= d.nx - 1 || cb < 0 || cb >= d.ny - 1) continue;
        if (!in.c_mask[cidx(d, ca, cb)]) continue;
        const double uy = um(ca + 1, cb + 1) * d.rdy - um(ca + 1, cb) * d.rdy;
        const double vx = vm(ca + 1, cb + 1) * d.rdx - vm(ca, cb + 1) * d.rdx;
        acc += 0.5 * (uy + vx);
      }
      sx[tb] = acc;
    }
    shear = 0.5 * sx[0] + 0.5 * sx[1];
  }
  const double ssr = sqrt(ux * ux + vy * vy + ux * vy + 0.25 * (shear * shear));
  // depth-averaged speed from centred velocities
  const double uc = hm ? (0.5 * u0 + 0.5 * u1) : 0.0;
  const double vc = hm ? (0.5 * v0 + 0.5 * v1) : 0.0;
  const double avs = sqrt(uc * uc + vc * vc);
  const double f2_prev = out.quad_f2[c], beta_prev = out.beta[c];
  const double bs = avs / (1.0 + f2_prev * beta_prev);
  const double ur = in.P->weertman_reg_speed;
  const double beta = in.wc[c] * pow(sqrt(bs * bs + ur * ur), 1.0 / in.P->weertman_m - 1.0);
  const double tau = beta * bs;
  out.shelf_strain_rate[c] = ssr;
  out.av_speed[c] = avs;
  out.bed_speed[c] = bs;
  out.beta[c] = beta;
  out.tau_bed[c] = tau;
  double eav = 0.0, f1 = 0.0, f2 = 0.0;
  if (hm) {
    const TR ex = (TR)(1.0 / in.P->glen_n - 1.0);
    const TR er2 = (TR)(in.P->glen_reg_strain_rate * in.P->glen_reg_strain_rate);
    const int n_iter_viscosity = in.P->n_iter_viscosity;
    const TR e2 = (TR)(ssr * ssr);
    const double hh = in.h[c];
    for (int k = 0; k < d.ns; ++k) {
      const size_t q = (size_t)c + (size_t)d.Nh * k;
      TR eta = (TR)out.eta[q];
      const TR B = (TR)in.glen_b[q];
      const TR tz = (TR)(tau * in.zeta[k]);
      for (int it = 0; it < n_iter_viscosity; ++it) {
        const TR t = tz / eta;
        eta = (TR)0.5 * B * powT<TR>(sqrt(e2 + (TR)0.25 * (t * t) + er2), ex);
      }
      const double e = (double)eta;
      out.eta[q] = e;
      eav += in.qw[k] * e;
      f1 += in.qw[k] * hh * in.zeta[k] / e;
      f2 += in.qw[k] * hh * (in.zeta[k] * in.zeta[k]) / e;
    }
  }
  out.eta_av[c] = eav;
  out.quad_f1[c] = f1;
  out.quad_f2[c] = f2;
  out.beta_eff[c] = beta / (1.0 + f2 * beta);
  const double hn = in.h[c] * eav;
  out.hn[c] = hn;
  const double hh_m = hm ? hn : 0.0;
  const double dm = hm ? in.P->c0 * in.dsdh[c] : 0.0;
  out.heta_h64[c] = hh_m;
  out.dimp64[c] = dm;
  if (out.heta_h32) {
    out.heta_h32[c] = (float)hh_m;
    out.dimp32[c] = (float)dm;
  }
}

// βeff on the u and v grids (update_βeff_on_uv_grids!, update_velocities.jl:348-366) and the c-grid
// coefficient hη_c = c_mask * cent_xy(h ηav) (:378).  One thread per point of the (nx+1) x (ny+1) space.
struct RelinUVIn {
  const uint8_t* mask;   // u | v
  const uint8_t* h_mask;
  const uint8_t* c_mask;
  const double* beta_eff;  // h grid
  const double* gf;        // h grid grounded fraction
  const double* gf_uv;     // u | v grounded fraction
  const double* h_uv;      // u | v thickness
  const double* hn;        // h*ηav
};
struct RelinUVOut {
  double* beta_eff_uv;  // gu.βeff | gv.βeff (written at mask points)
  double *beta_m64, *h_m64, *heta_c64;
  float *beta_m32, *h_m32, *heta_c32;
};
static __global__ void k_relin_uv(Dims d, RelinUVIn in, RelinUVOut out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  auto hmk = [&](int a, int b) { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny && in.h_mask[hidx(d, a, b)]) ? 1.0 : 0.0; };
  auto hv = [&](const double* f, int a, int b) {
    return (a >= 0 && a < d.nx && b >= 0 && b < d.ny && in.h_mask[hidx(d, a, b)]) ? f[hidx(d, a, b)] : 0.0;
  };
  auto point = [&](int q, int a0, int b0, int a1, int b1) {
    // neighbours (a0,b0) then (a1,b1) in ascending index order, weights 0.5 each
    double bm = 0.0, hm = 0.0;
    if (in.mask[q]) {
      const double num = 0.5 * hv(in.beta_eff, a0, b0) + 0.5 * hv(in.beta_eff, a1, b1);
      const double den = 0.5 * hmk(a0, b0) + 0.5 * hmk(a1, b1);
      // den is 0, 0.5 or 1, so x / den is exactly x * (1 / den) — also 0 * inf = NaN = 0 / 0 and
      // x * inf = ±inf = x / 0 — without an FP64 division (a long sequence on GB300's FP64 pipe)
      const double rden = den == 1.0 ? 1.0 : den == 0.5 ? 2.0 : 1.0 / den;
      double be = num * rden;
      const double ip = (0.5 * hv(in.gf, a0, b0) + 0.5 * hv(in.gf, a1, b1)) * rden;
      if (ip > 0.0) be = be * in.gf_uv[q] / ip;
      out.beta_eff_uv[q] = be;
      bm = be;
      hm = in.h_uv[q];
    }
    out.beta_m64[q] = bm;
    out.h_m64[q] = hm;
    if (out.beta_m32) {
      out.beta_m32[q] = (float)bm;
      out.h_m32[q] = (float)hm;
    }
  };
  if (i <= d.nx && j < d.ny) point(uidx(d, i, j), i - 1, j, i, j);
  if (i < d.nx && j <= d.ny) point(vidx(d, i, j), i, j - 1, i, j);
  if (i < d.nx - 1 && j < d.ny - 1) {
    const int q = cidx(d, i, j);
    double v = 0.0;
    if (in.c_mask[q]) {
      // cent_xy = c(ny-1) ⊗ c(nx-1) evaluated y-first (the lazy Kronecker order when ny <= nx)
      const double a = 0.5 * in.hn[hidx(d, i, j)] + 0.5 * in.hn[hidx(d, i, j + 1)];
      const double b = 0.5 * in.hn[hidx(d, i + 1, j)] + 0.5 * in.hn[hidx(d, i + 1, j + 1)];
      v = 0.5 * a + 0.5 * b;
    }
    out.heta_c64[q] = v;
    if (out.heta_c32) out.heta_c32[q] = (float)v;
  }
}

// ------------------------------------------------------------------------------------------------
// Right-hand side f1 + f2 (get_rhs, update_velocities.jl:106-182) at the interior points, plus x = the
// start guess (get_start_guess :92-97) and the Dirichlet values u*u_isfixed (:409-413).
// ------------------------------------------------------------------------------------------------
struct RhsIn {
  const uint8_t* h_mask;
  const uint8_t* inner;   // u | v
  const uint8_t* fixed;   // u | v
  const double* s;
  const double* dsdh;
  const double* acc;
  const double* melt;
  const double* h_uv;
  const double* s_uv;
  const double* uv;
  double rho_i, rho_w, g, sea_level, theta_dt;
};
static __global__ void k_rhs(Dims d, RhsIn in, double* __restrict__ b, double* __restrict__ x, double* __restrict__ xfixed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  auto sadj = [&](int a, int c) -> double {
    if (a < 0 || a >= d.nx || c < 0 || c >= d.ny) return 0.0;
    const int q = hidx(d, a, c);
    if (!in.h_mask[q]) return 0.0;
    return in.s[q] + in.theta_dt * in.dsdh[q] * (in.acc[q] - in.melt[q]);
  };
  auto hmk = [&](int a, int c) -> double {
    return (a >= 0 && a < d.nx && c >= 0 && c < d.ny && in.h_mask[hidx(d, a, c)]) ? 1.0 : 0.0;
  };
  auto point = [&](int q, int a0, int b0, int a1, int b1, double rd) {
    double bv = 0.0;
    if (in.inner[q]) {
      // -(∂ᵀ s_adj) = (s_adj(1) - s_adj(0)) / d ;  -(∂ᵀ h_mask) likewise
      const double ds = sadj(a1, b1) * rd - sadj(a0, b0) * rd;
      const double dm = hmk(a1, b1) * rd - hmk(a0, b0) * rd;
      const double hh = in.h_uv[q], ss = in.s_uv[q];
      const double draft = fmax(hh - (ss - in.sea_level), 0.0);
      const double f1 = (in.rho_i * in.g * hh) * ds;
      const double f2 = dm * in.g * (0.5 * in.rho_i * (hh * hh) - 0.5 * in.rho_w * (draft * draft) - in.rho_i * hh * ss);
      bv = f1 + f2;
    }
    b[q] = bv;
    x[q] = in.inner[q] ? in.uv[q] : 0.0;
    xfixed[q] = in.fixed[q] ? in.uv[q] : 0.0;
  };
  if (i <= d.nx && j < d.ny) point(uidx(d, i, j), i - 1, j, i, j, d.rdx);
  if (i < d.nx && j <= d.ny) point(vidx(d, i, j), i, j - 1, i, j, d.rdy);
}

// ------------------------------------------------------------------------------------------------
// Elementwise and reduction kernels over the N = Nu + Nv solver vectors
// ------------------------------------------------------------------------------------------------
template <typename TA, typename TB>
__global__ void k_convert(int n, const TA* __restrict__ a, TB* __restrict__ b) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) b[k] = (TB)a[k];
}
template <typename T>
__global__ void k_fill(int n, T* __restrict__ a, T v) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) a[k] = v;
}
// out = a - b (elementwise)
template <typename T>
__global__ void k_sub(int n, const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) out[k] = a[k] - b[k];
}
// partial sums of a.b
template <typename TA, typename TB>
__global__ void k_dot(int n, const TA* __restrict__ a, const TB* __restrict__ b, double* __restrict__ partials) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    s += (double)a[k] * (double)b[k];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}
// Jacobi update of one colour (gauss_seidel_smoother!, update_preconditioners.jl:133-150):
// x[c] += ω r[c] / diag[c] for the points of colour `colour` (u: 1 + mod(i-j,2), v: 3 + mod(i-j,2), 1-based).
template <typename T>
__global__ void k_colour_update(Dims d, int colour, T omega, const uint8_t* __restrict__ inner, const T* __restrict__ r,
                                const T* __restrict__ diag, T* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const int par = ((i - j) % 2 + 2) % 2;  // mod(i-j, 2) is the same for 0- and 1-based indices
  if (colour <= 2) {
    if (i <= d.nx && j < d.ny && par == colour - 1) {
      const int q = uidx(d, i, j);
      if (inner[q]) x[q] = x[q] + omega * r[q] / diag[q];
    }
  } else {
    if (i < d.nx && j <= d.ny && par == colour - 3) {
      const int q = vidx(d, i, j);
      if (inner[q]) x[q] = x[q] + omega * r[q] / diag[q];
    }
  }
}
// x64 += corr (at all points; corr is zero off the interior), then write the interior back to uv
template <typename T>
__global__ void k_apply_correction(int n, const uint8_t* __restrict__ inner, const T* __restrict__ corr,
                                   double* __restrict__ x, double* __restrict__ uv) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double v = x[k] + (double)corr[k];
    x[k] = v;
    if (inner[k]) uv[k] = v;
  }
}
// partial sums of |a_new - a_old|^2 and |a_new|^2 over the interior
template <typename T>
__global__ void k_update_norms(int n, const T* __restrict__ corr, const double* __restrict__ x, double* __restrict__ partials) {
  __shared__ double sh[32];
  double s0 = 0.0, s1 = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double c = (double)corr[k];
    s0 += c * c;
    s1 += x[k] * x[k];
  }
  double a = block_sum(s0, sh);
  __syncthreads();
  double b = block_sum(s1, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = a;
    partials[gridDim.x + blockIdx.x] = b;
  }
}

// ------------------------------------------------------------------------------------------------
// Haar wavelet transforms (wavelet_matrix, Wavelets/update_wavelets.jl:38-89), tile-local.
// Lifting pairs (o, o+s/2) with o a multiple of s (0-based) never cross a 2^(L+1)-aligned block, so a
// CTA transforms 16 x 16 blocks (levels = 3; up to 32 x 32 for levels = 4) entirely in shared memory.
// KIND 0: prolong   out = inner ⊙ idwt(in)         (prolong_fun!, utilities.jl:220-237)
// KIND 1: restrict  out = wmask ⊙ idwtᵀ(in)        (restrict_fun!, utilities.jl:175-190)
// KIND 2: forward   out = dwt(mask ⊙ in)           (update_wavelets!, update_wavelets.jl:13-14)
// ACC: out += result instead of out = result.  DOT: partial sums of out . dotv per block.
// ------------------------------------------------------------------------------------------------
constexpr int HAAR_B = 16;

template <typename TI, typename TO, int KIND, bool ACC, bool DOT>
__global__ void __launch_bounds__(HAAR_B* HAAR_B)
    k_haar(Dims d, int levels, const TI* __restrict__ in, TO* __restrict__ out, const uint8_t* __restrict__ outmask,
           const uint8_t* __restrict__ inmask, const TO* __restrict__ dotv, double* __restrict__ partials,
           const int* __restrict__ skip) {
  if (skip && *skip) return;
  // grid.z selects the component: 0 = u grid ((nx+1) x ny), 1 = v grid (nx x (ny+1))
  const int comp = blockIdx.z;
  const int nxg = comp == 0 ? d.nx + 1 : d.nx;
  const int nyg = comp == 0 ? d.ny : d.ny + 1;
  const int off = comp == 0 ? 0 : d.Nu;
  const int B = 1 << (levels + 1);
  const int bx0 = blockIdx.x * B, by0 = blockIdx.y * B;
  __shared__ double tile[32][33];
  __shared__ double sh[32];
  const int tx = threadIdx.x, ty = threadIdx.y;  // blockDim = (B, B)
  double acc_dot = 0.0;
  const bool active_block = bx0 < nxg && by0 < nyg;
  const int gi = bx0 + tx, gj = by0 + ty;
  const bool inside = active_block && gi < nxg && gj < nyg;
  const int q = off + gi + nxg * gj;
  double val = 0.0;
  if (inside) {
    val = (double)in[q];
    if (KIND == 2 && !inmask[q]) val = 0.0;
  }
  tile[ty][tx] = val;
  __syncthreads();
  // along y then along x (the reference's Kronecker order for square factors: y first)
  for (int dir = 0; dir < 2; ++dir) {
    const int n = dir == 0 ? nyg : nxg;
    const int base = dir == 0 ? by0 : bx0;
    const int pos = dir == 0 ? ty : tx;  // position inside the block along dir
    for (int lv = 0; lv <= levels; ++lv) {
      // KIND 0 (idwt = M_2 ... M_B): apply M_B first; KIND 1 (idwtᵀ): M_2ᵀ first; KIND 2 (dwt): F_2 first
      const int s = (KIND == 0) ? (B >> lv) : (2 << lv);
      const int half = s >> 1;
      double a = tile[ty][tx];
      const bool is_o = (pos % s) == 0, is_e = (pos % s) == half;
      double nv = a;
      if (is_o || is_e) {
        const int po = is_o ? pos : pos - half;
        const int pe = po + half;
        if (base + pe < n && inside) {
          const double xo = dir == 0 ? tile[po][tx] : tile[ty][po];
          const double xe = dir == 0 ? tile[pe][tx] : tile[ty][pe];
          if (KIND == 0) nv = is_e ? xe + xo : xo - xe;
          else if (KIND == 1) nv = is_o ? xo + xe : xe - xo;
          else nv = is_e ? 0.5 * (xe - xo) : 0.5 * (xo + xe);
        }
      }
      __syncthreads();
      tile[ty][tx] = nv;
      __syncthreads();
    }
  }
  if (inside) {
    double r = tile[ty][tx];
    if (KIND != 2 && !outmask[q]) r = 0.0;
    TO o = (TO)r;
    if (ACC) o = (TO)((double)out[q] + r);
    out[q] = o;
    if (DOT) acc_dot = (double)o * (double)dotv[q];
  }
  if (DOT) {
    double s = block_sum_2d(acc_dot, sh);
    if (tx == 0 && ty == 0) partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
  }
}

// ------------------------------------------------------------------------------------------------
// Coarse conjugate gradients (IterativeSolvers cg!, called at update_preconditioners.jl:73), with all
// scalars on the device so a batch of iterations needs no host round trip.
//   S[CG_RES] = |r|, S[CG_PREV] = previous |r|, S[CG_TOL] = tolerance, S[CG_ALPHA]
//   I[CG_IT] = iteration, I[CG_DONE] = 1 once it >= maxiter or |r| <= tol
// ------------------------------------------------------------------------------------------------
enum { CG_RES = 0, CG_PREV = 1, CG_TOL = 2, CG_ALPHA = 3, CG_SUM = 4, CG_BNORM = 5, S_RR = 8, S_BB = 9, S_REL = 10,
       S_DU = 11, S_UU = 12, S_COUNT = 16 };
enum { CG_IT = 0, CG_DONE = 1, CG_MAXIT = 2, I_COUNT = 8 };

// u = r + β u with β = |r|^2 / |r_prev|^2
template <typename T>
__global__ void k_cg_dir(int n, const double* __restrict__ S, const int* __restrict__ I, const T* __restrict__ r,
                         T* __restrict__ u) {
  if (I[CG_DONE]) return;
  const double res = S[CG_RES], prev = S[CG_PREV];
  const double beta = (res * res) / (prev * prev);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    u[k] = (T)((double)r[k] + beta * (double)u[k]);
}
// α = |r|^2 / <u, c>  (reduces the partials of <u,c> itself; one block)
static __global__ void k_cg_alpha(const double* __restrict__ partials, int np, double* __restrict__ S, const int* __restrict__ I) {
  if (I[CG_DONE]) return;
  __shared__ double sh[32];
  double s = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) s += partials[k];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) S[CG_ALPHA] = (S[CG_RES] * S[CG_RES]) / s;
}
// x += α u;  r -= α c;  partial |r|^2
template <typename T>
__global__ void k_cg_axpy(int n, const double* __restrict__ S, const int* __restrict__ I, const T* __restrict__ u,
                          const T* __restrict__ c, T* __restrict__ x, T* __restrict__ r, double* __restrict__ partials) {
  if (I[CG_DONE]) return;
  __shared__ double sh[32];
  const double alpha = S[CG_ALPHA];
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    x[k] = (T)((double)x[k] + alpha * (double)u[k]);
    const T rv = (T)((double)r[k] - alpha * (double)c[k]);
    r[k] = rv;
    s += (double)rv * (double)rv;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}
// prev = res; res = |r|; it++; done = it >= maxiter || res <= tol  (one block)
static __global__ void k_cg_res(const double* __restrict__ partials, int np, double* __restrict__ S, int* __restrict__ I) {
  if (I[CG_DONE]) return;
  __shared__ double sh[32];
  double s = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) s += partials[k];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    S[CG_PREV] = S[CG_RES];
    const double res = sqrt(s);
    S[CG_RES] = res;
    const int it = I[CG_IT] + 1;
    I[CG_IT] = it;
    I[CG_DONE] = (it >= I[CG_MAXIT] || res <= S[CG_TOL] || !(res == res)) ? 1 : 0;
  }
}
// out = sqrt(*in)
static __global__ void k_sqrt_slot(const double* __restrict__ in, double* __restrict__ out) { *out = sqrt(*in); }
// CG start: r = b - c (c = A x0), |r|, tol = max(reltol |r0|, abstol), abstol = tol_coarse |b|
template <typename T>
__global__ void k_cg_start_sub(int n, const T* __restrict__ b, const T* __restrict__ c, T* __restrict__ r, T* __restrict__ u,
                               double* __restrict__ partials) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const T rv = b[k] - c[k];
    r[k] = rv;
    u[k] = (T)0;
    s += (double)rv * (double)rv;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}
static __global__ void k_cg_start_scalars(const double* __restrict__ partials, int np, double tol_coarse, int maxiter,
                                   double* __restrict__ S, int* __restrict__ I) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int k = threadIdx.x; k < np; k += blockDim.x) s += partials[k];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    const double res = sqrt(s);
    const double abstol = tol_coarse * S[CG_BNORM];
    const double reltol = 1.4901161193847656e-08;  // sqrt(eps(Float64))
    S[CG_RES] = res;
    S[CG_PREV] = 1.0;
    S[CG_TOL] = fmax(reltol * res, abstol);
    I[CG_IT] = 0;
    I[CG_MAXIT] = maxiter;
    I[CG_DONE] = (0 >= maxiter || res <= S[CG_TOL] || !(res == res)) ? 1 : 0;
  }
}

}  // namespace wavi
