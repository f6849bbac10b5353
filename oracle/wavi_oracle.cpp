// wavi_oracle.cpp — FP64 CPU restatement of WAVI.jl's velocity solve and of the update_state! steps
// around it.  TEST INFRASTRUCTURE ONLY: the oracle that the GPU library is checked against, and the
// timed CPU stand-in for the reference.  Nothing in the product (libwavi_gpu.so, the Python host
// package) links, loads or calls it.
//
// The reference (Julia) cannot run in this build environment, so this file restates it line by line.
// Every function cites the reference lines it follows.  Parity is pinned end-to-end against the
// reference's own golden files (test/version_update_test_verification/*.jld2, 1000 coupled solves).
//
// Fidelity choices:
//  * Every staggered difference, average, Haar transform and sampling step is a lazy Kronecker product
//    in the reference (src/KroneckerProduct.jl:57-73).  `Kron::apply` reproduces its two evaluation
//    orders (x-first or y-first, chosen by the same size test) and, within each 1-D factor, sums the
//    terms in ascending input index starting from zero, which is the summation order of the SparseArrays
//    kernels the reference calls.  1-D factors carry the reference's stored values (±1/dx, 0.5, 1).
//  * The coarse solve restates IterativeSolvers.jl `cg!` (third-party, not vendored by the reference,
//    version unpinned; the `abstol` keyword used at update_preconditioners.jl:73 exists from v0.9):
//    x0 warm start, r = b - A x0, tol = max(reltol*|r0|, abstol) with reltol = sqrt(eps(Float64)),
//    stop when iteration >= maxiter or |r| <= tol; u = r + (|r|^2/|r_prev|^2) u; c = A u;
//    alpha = |r|^2 / <u,c>; x += alpha u; r -= alpha c.
//  * Norms and dot products are plain left-to-right sums (the reference calls BLAS nrm2/dot).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../include/wavi_gpu.h"

namespace {

using Vec = std::vector<double>;
using Mask = std::vector<uint8_t>;

// ---------------------------------------------------------------------------------------------
// 1-D sparse factors (rows with ascending columns).  src/utilities.jl:2-5, Wavelets/update_wavelets.jl:38-89
// ---------------------------------------------------------------------------------------------
struct Op1D {
  int m = 0, n = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
};

Op1D from_triplets(int m, int n, std::vector<std::vector<std::pair<int, double>>> rows) {
  Op1D o;
  o.m = m;
  o.n = n;
  o.rowptr.assign(m + 1, 0);
  for (int r = 0; r < m; ++r) {
    auto& rr = rows[r];
    std::sort(rr.begin(), rr.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (auto& e : rr) {
      o.col.push_back(e.first);
      o.val.push_back(e.second);
    }
    o.rowptr[r + 1] = (int)o.col.size();
  }
  return o;
}

// spI(n) = spdiagm(n,n,0=>ones(n))                                   utilities.jl:2
Op1D spI(int n) {
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  for (int i = 0; i < n; ++i) rows[i].push_back({i, 1.0});
  return from_triplets(n, n, rows);
}
// ∂1d(n,dx) = spdiagm(n,n+1,0=>-ones(n),1=>ones(n))/dx                 utilities.jl:3
Op1D d1d(int n, double dx) {
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  for (int i = 0; i < n; ++i) {
    rows[i].push_back({i, -1.0 / dx});
    rows[i].push_back({i + 1, 1.0 / dx});
  }
  return from_triplets(n, n + 1, rows);
}
// c(n) = spdiagm(n,n+1,0=>ones(n),1=>ones(n))/2                        utilities.jl:4
Op1D cavg(int n) {
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  for (int i = 0; i < n; ++i) {
    rows[i].push_back({i, 0.5});
    rows[i].push_back({i + 1, 0.5});
  }
  return from_triplets(n, n + 1, rows);
}
// χ(n) = spdiagm(n,n+2,1=>ones(n))                                     utilities.jl:5
Op1D chi(int n) {
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  for (int i = 0; i < n; ++i) rows[i].push_back({i + 1, 1.0});
  return from_triplets(n, n + 2, rows);
}
Op1D transpose(const Op1D& a) {
  std::vector<std::vector<std::pair<int, double>>> rows(a.n);
  for (int r = 0; r < a.m; ++r)
    for (int k = a.rowptr[r]; k < a.rowptr[r + 1]; ++k) rows[a.col[k]].push_back({r, a.val[k]});
  return from_triplets(a.n, a.m, rows);
}
// wavelet_matrix(n, levels, direction)                       Wavelets/update_wavelets.jl:38-89
// Reverse: rwav = M_2 * M_4 * ... * M_{2^(levels+1)}, M_s: x[e] <- x[e]+x[o], x[o] <- x[o]-x[e] for the
// pairs (o, e=o+s/2), o = 1:s:(n-s/2).  Forward: fwav = F_{2^(levels+1)} ... F_2 with
// F_s: x[e] <- (x[e]-x[o])/2, x[o] <- (x[o]+x[e])/2.  Columns are built by applying the lifting steps
// to unit vectors (entries are exact: ±1 and powers of 1/2).
Op1D wavelet(int n, int levels, bool forward) {
  std::vector<int> steps;
  int step = 1;
  for (int j = levels; j >= 0; --j) {
    step *= 2;
    steps.push_back(step);
  }
  auto lift = [&](std::vector<double>& x, int s) {
    int half = s / 2;
    for (int o = 0; o + half < n; o += s) {  // 1-based o = 1:s:(n-s/2)  ->  0-based o + half <= n-1
      int e = o + half;
      double xo = x[o], xe = x[e];
      if (forward) {
        x[e] = 0.5 * (xe - xo);
        x[o] = 0.5 * (xo + xe);
      } else {
        x[e] = xe + xo;
        x[o] = xo - xe;
      }
    }
  };
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  std::vector<double> x(n);
  for (int k = 0; k < n; ++k) {
    std::fill(x.begin(), x.end(), 0.0);
    x[k] = 1.0;
    if (forward) {
      for (int s : steps) lift(x, s);  // F_2 applied first
    } else {
      for (int t = (int)steps.size() - 1; t >= 0; --t) lift(x, steps[t]);  // M_{2^(L+1)} first
    }
    for (int r = 0; r < n; ++r)
      if (x[r] != 0.0) rows[r].push_back({k, x[r]});
  }
  return from_triplets(n, n, rows);
}

// ---------------------------------------------------------------------------------------------
// Lazy Kronecker product A ⊗ B: A acts along y (second index), B along x.  KroneckerProduct.jl:57-73
// ---------------------------------------------------------------------------------------------
struct Kron {
  Op1D A, B;
  mutable Vec temp;
  int rows() const { return A.m * B.m; }
  int cols() const { return A.n * B.n; }
  void apply(const double* x, double* y) const {
    const int ma = A.m, na = A.n, mb = B.m, nb = B.n;
    if ((long)nb * ma <= (long)mb * na) {
      // temp = X * transpose(A)  (nb x ma);  Y = B * temp
      temp.assign((size_t)nb * ma, 0.0);
      for (int r = 0; r < ma; ++r)
        for (int k = A.rowptr[r]; k < A.rowptr[r + 1]; ++k) {
          const double a = A.val[k];
          const double* xc = x + (size_t)nb * A.col[k];
          double* tc = temp.data() + (size_t)nb * r;
          for (int i = 0; i < nb; ++i) tc[i] += xc[i] * a;
        }
      for (int r = 0; r < ma; ++r) {
        const double* tc = temp.data() + (size_t)nb * r;
        double* yc = y + (size_t)mb * r;
        for (int o = 0; o < mb; ++o) {
          double s = 0.0;
          for (int k = B.rowptr[o]; k < B.rowptr[o + 1]; ++k) s += B.val[k] * tc[B.col[k]];
          yc[o] = s;
        }
      }
    } else {
      // temp = B * X  (mb x na);  Y = temp * transpose(A)
      temp.assign((size_t)mb * na, 0.0);
      for (int c = 0; c < na; ++c) {
        const double* xc = x + (size_t)nb * c;
        double* tc = temp.data() + (size_t)mb * c;
        for (int o = 0; o < mb; ++o) {
          double s = 0.0;
          for (int k = B.rowptr[o]; k < B.rowptr[o + 1]; ++k) s += B.val[k] * xc[B.col[k]];
          tc[o] = s;
        }
      }
      std::fill(y, y + (size_t)mb * ma, 0.0);
      for (int r = 0; r < ma; ++r)
        for (int k = A.rowptr[r]; k < A.rowptr[r + 1]; ++k) {
          const double a = A.val[k];
          const double* tc = temp.data() + (size_t)mb * A.col[k];
          double* yc = y + (size_t)mb * r;
          for (int o = 0; o < mb; ++o) yc[o] += tc[o] * a;
        }
    }
  }
  Vec operator*(const Vec& x) const {
    Vec y(rows());
    apply(x.data(), y.data());
    return y;
  }
};
Kron kron(const Op1D& a, const Op1D& b) { return Kron{a, b, {}}; }

// Summation order of the coarse CG's norms and dot products.  The reference calls BLAS for both
// (LinearAlgebra `dot` -> BLAS.dot; `norm` -> BLAS.nrm2 for length >= 32), and a coarse CG of hundreds of
// iterations is sensitive to that order at the 1e-5 level, which a 1000-step coupled run carries to its
// end.  Orders 2 and 3 restate the x86-64 OpenBLAS kernels Julia ships: ddot with fused multiply-add
// lanes (order 2: four 4-wide accumulators over blocks of 16, the AVX2 shape; order 3, the default:
// four 8-wide accumulators over blocks of 32, the AVX-512 shape), accumulators combined pairwise, the
// remainder added left to right; dnrm2 accumulated in extended precision.  Order 3 reproduces the
// reference's v1.8.3 golden file within its own tolerance (Julia's isapprox, rtol = sqrt(eps)), so that
// file was made on an AVX-512 machine.  Order 0 is a plain left-to-right sum; order 1 blocked partial
// sums of 64.
int g_sum_order = 3;

double dot_openblas_x86(const double* a, const double* b, size_t n) {
  const size_t n1 = n & ~(size_t)15;
  double lane[16] = {0.0};
  for (size_t i = 0; i < n1; i += 16)
    for (int l = 0; l < 16; ++l) lane[l] = std::fma(a[i + l], b[i + l], lane[l]);
  double acc[4];
  for (int l = 0; l < 4; ++l) acc[l] = (lane[l] + lane[4 + l]) + (lane[8 + l] + lane[12 + l]);
  double dot = n1 ? (acc[0] + acc[2]) + (acc[1] + acc[3]) : 0.0;
  for (size_t i = n1; i < n; ++i) dot += b[i] * a[i];
  return dot;
}

// The AVX-512 shape of the same kernel: four 8-wide accumulators over blocks of 32.
double dot_openblas_x86_avx512(const double* a, const double* b, size_t n) {
  const size_t n1 = n & ~(size_t)31;
  double lane[32] = {0.0};
  for (size_t i = 0; i < n1; i += 32)
    for (int l = 0; l < 32; ++l) lane[l] = std::fma(a[i + l], b[i + l], lane[l]);
  double acc[8];
  for (int l = 0; l < 8; ++l) acc[l] = (lane[l] + lane[8 + l]) + (lane[16 + l] + lane[24 + l]);
  double h4[4], h2[2];
  for (int l = 0; l < 4; ++l) h4[l] = acc[l] + acc[4 + l];
  for (int l = 0; l < 2; ++l) h2[l] = h4[l] + h4[2 + l];
  double dot = n1 ? h2[0] + h2[1] : 0.0;
  for (size_t i = n1; i < n; ++i) dot += b[i] * a[i];
  return dot;
}

double sum_products(const double* a, const double* b, size_t n) {
  if (g_sum_order == 2) return dot_openblas_x86(a, b, n);
  if (g_sum_order == 3) return dot_openblas_x86_avx512(a, b, n);
  if (g_sum_order == 0) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
  }
  double s = 0.0;
  for (size_t k = 0; k < n; k += 64) {
    double p = 0.0;
    for (size_t i = k; i < std::min(n, k + 64); ++i) p += a[i] * b[i];
    s += p;
  }
  return s;
}
double norm2(const Vec& x) {
  if (g_sum_order >= 2 && x.size() >= 32) {
    long double s[4] = {0.0L, 0.0L, 0.0L, 0.0L};
    for (size_t i = 0; i < x.size(); ++i) s[i & 3] += (long double)x[i] * (long double)x[i];
    return (double)std::sqrt((s[0] + s[1]) + (s[2] + s[3]));
  }
  return std::sqrt(sum_products(x.data(), x.data(), x.size()));
}
double dotp(const Vec& a, const Vec& b) { return sum_products(a.data(), b.data(), a.size()); }

// ---------------------------------------------------------------------------------------------
// Model state.  src/Fields/*.jl, src/Models/Model.jl:1-9
// ---------------------------------------------------------------------------------------------
struct Model {
  int nx, ny, ns;
  double dx, dy;
  Vec sigma, zeta, qw;
  wavi_params P;
  wavi_solver_params S;
  double melt_m = 0.0;  // UniformMeltRate(m) (MeltRate/MeltRate.jl:37-54)
  int Nh, Nu, Nv, Nc;
  Mask h_mask, h_isfixed, u_mask, v_mask, c_mask, u_inner, v_inner, u_isfixed, v_isfixed;
  std::vector<int> u_inner_idx, v_inner_idx;  // samp_inner: sampled position -> full index
  int ni_u = 0, ni_v = 0;
  // h grid
  Vec b, h, s, dhdt, accumulation, basal_melt, haf, gf, dsdh, shelf_strain_rate, av_speed, uh, vh, us, vs,
      ub, vb, bed_speed, weertman_c, beta, beta_eff, tau_bed, eta_av, quad_f1, quad_f2;
  Vec weertman_c_param, accumulation_param, glen_a_ref;
  Vec dneg_heta_h, dimplicit, dneg_heta_c;
  // u / v grids
  Vec gu_s, gu_h, gu_gf, gu_beff, gu_dnegbeff, u, gu_resid;
  Vec gv_s, gv_h, gv_gf, gv_beff, gv_dnegbeff, v, gv_resid;
  // sigma grid
  Vec eta, temperature, damage, glen_b;
  // wavelets
  Mask wu_mask, wv_mask;
  Vec wu_corr, wv_corr, wu_wav, wv_wav;
  // operators
  Kron h_cent_xy;
  Kron u_cent, u_centT, u_dx, u_dxT, u_dy, u_dyT, u_dwt, wu_idwt, wu_idwtT;
  Kron v_cent, v_centT, v_dx, v_dxT, v_dy, v_dyT, v_dwt, wv_idwt, wv_idwtT;
  Kron c_cent, c_centT;
  // statistics of the last update_velocities!
  int last_picard = 0;
  double last_rel_resid = 0.0;
  long last_cg_iters = 0;
  long op_applies = 0;
  std::vector<int> cg_iter_history;
  std::vector<double> rel_history, upd_history;  // per Picard iteration: ||b - A u|| / ||b||, ||du|| / ||u||
  Vec cheb_eig;           // coarse variants 4, 5: the power vector (full wavelet layout, u then v), per solve
  Vec last_coarse_b;      // the last V-cycle's coarse right-hand side and starting point (the cached
  Vec last_coarse_x0;     // correction), in the coarse order [u | v], for studies of the coarse solvers
  int cheb_vcycles = 0;   // coarse variants 4, 5: V-cycles so far in this solve
  double picard_rel = 0;  // the current Picard iteration's relative residual (the adaptive coarse tolerance)
  std::string err;
};

inline int hid(const Model& m, int i, int j) { return i + m.nx * j; }

// utilities.jl:475-507
Mask get_u_mask(const Model& m) {
  Mask um((size_t)m.Nu, 0);
  for (int j = 0; j < m.ny; ++j)
    for (int i = 0; i < m.nx; ++i)
      if (m.h_mask[hid(m, i, j)]) {
        um[i + (m.nx + 1) * j] = 1;
        um[i + 1 + (m.nx + 1) * j] = 1;
      }
  return um;
}
Mask get_v_mask(const Model& m) {
  Mask vm((size_t)m.Nv, 0);
  for (int j = 0; j < m.ny; ++j)
    for (int i = 0; i < m.nx; ++i)
      if (m.h_mask[hid(m, i, j)]) {
        vm[i + m.nx * j] = 1;
        vm[i + m.nx * (j + 1)] = 1;
      }
  return vm;
}
Mask get_c_mask(const Model& m) {
  Mask cm((size_t)m.Nc, 0);
  for (int j = 0; j < m.ny - 1; ++j)
    for (int i = 0; i < m.nx - 1; ++i)
      cm[i + (m.nx - 1) * j] = m.h_mask[hid(m, i, j)] && m.h_mask[hid(m, i, j + 1)] &&
                               m.h_mask[hid(m, i + 1, j)] && m.h_mask[hid(m, i + 1, j + 1)];
  return cm;
}

Vec crop(const Mask& mask, const Vec& x) {  // Diagonal(float(mask)) * x
  Vec y(x.size());
  for (size_t i = 0; i < x.size(); ++i) y[i] = (mask[i] ? 1.0 : 0.0) * x[i];
  return y;
}

void build_model(Model& m, const wavi_grid_desc* g, const wavi_params* p, const wavi_solver_params* sp) {
  m.nx = g->nx;
  m.ny = g->ny;
  m.ns = g->nsigma;
  m.dx = g->dx;
  m.dy = g->dy;
  m.P = *p;
  m.S = *sp;
  m.sigma.assign(g->sigma, g->sigma + m.ns);
  m.qw.assign(g->quadrature_weights, g->quadrature_weights + m.ns);
  m.zeta.resize(m.ns);
  for (int k = 0; k < m.ns; ++k) m.zeta[k] = 1.0 - m.sigma[k];  // Grid.jl:170
  m.Nh = m.nx * m.ny;
  m.Nu = (m.nx + 1) * m.ny;
  m.Nv = m.nx * (m.ny + 1);
  m.Nc = (m.nx - 1) * (m.ny - 1);
  auto cp = [](const uint8_t* src, int n) {
    Mask r((size_t)n, 0);
    for (int i = 0; i < n; ++i) r[i] = src ? (src[i] != 0) : 0;
    return r;
  };
  m.h_mask = cp(g->h_mask, m.Nh);
  m.h_isfixed.assign(m.Nh, 0);
  m.u_isfixed = cp(g->u_isfixed, m.Nu);
  m.v_isfixed = cp(g->v_isfixed, m.Nv);
  // Fields.jl:28-35
  m.u_mask = get_u_mask(m);
  m.v_mask = get_v_mask(m);
  m.c_mask = get_c_mask(m);
  Mask uz = cp(g->u_iszero, m.Nu), vz = cp(g->v_iszero, m.Nv);
  for (int i = 0; i < m.Nu; ++i)
    if (uz[i]) m.u_mask[i] = 0;
  for (int i = 0; i < m.Nv; ++i)
    if (vz[i]) m.v_mask[i] = 0;
  // UGrid.jl:76-77, VGrid.jl:77-78
  m.u_inner.resize(m.Nu);
  m.v_inner.resize(m.Nv);
  m.u_inner_idx.clear();
  m.v_inner_idx.clear();
  for (int i = 0; i < m.Nu; ++i) {
    m.u_inner[i] = m.u_mask[i] && !m.u_isfixed[i];
    if (m.u_inner[i]) m.u_inner_idx.push_back(i);
  }
  for (int i = 0; i < m.Nv; ++i) {
    m.v_inner[i] = m.v_mask[i] && !m.v_isfixed[i];
    if (m.v_inner[i]) m.v_inner_idx.push_back(i);
  }
  m.ni_u = (int)m.u_inner_idx.size();
  m.ni_v = (int)m.v_inner_idx.size();

  const int nx = m.nx, ny = m.ny;
  const int L = sp->levels;
  // HGrid.jl:88
  m.h_cent_xy = kron(cavg(ny - 1), cavg(nx - 1));
  // UGrid.jl:83-89 (nxu = nx+1, nyu = ny)
  m.u_cent = kron(spI(ny), cavg(nx));
  m.u_centT = kron(transpose(spI(ny)), transpose(cavg(nx)));
  m.u_dx = kron(spI(ny), d1d(nx, m.dx));
  m.u_dxT = kron(transpose(spI(ny)), transpose(d1d(nx, m.dx)));
  m.u_dy = kron(d1d(ny - 1, m.dy), chi(nx - 1));
  m.u_dyT = kron(transpose(d1d(ny - 1, m.dy)), transpose(chi(nx - 1)));
  m.u_dwt = kron(wavelet(ny, L, true), wavelet(nx + 1, L, true));
  // VGrid.jl:84-90 (nxv = nx, nyv = ny+1)
  m.v_cent = kron(cavg(ny), spI(nx));
  m.v_centT = kron(transpose(cavg(ny)), transpose(spI(nx)));
  m.v_dx = kron(chi(ny - 1), d1d(nx - 1, m.dx));
  m.v_dxT = kron(transpose(chi(ny - 1)), transpose(d1d(nx - 1, m.dx)));
  m.v_dy = kron(d1d(ny, m.dy), spI(nx));
  m.v_dyT = kron(transpose(d1d(ny, m.dy)), transpose(spI(nx)));
  m.v_dwt = kron(wavelet(ny + 1, L, true), wavelet(nx, L, true));
  // CGrid.jl:45-46 (nxc = nx-1, nyc = ny-1)
  m.c_cent = kron(transpose(cavg(ny - 1)), transpose(cavg(nx - 1)));
  m.c_centT = kron(cavg(ny - 1), cavg(nx - 1));
  // UWavelets.jl:48-49, VWavelets.jl:48-49
  m.wu_idwt = kron(wavelet(ny, L, false), wavelet(nx + 1, L, false));
  m.wu_idwtT = kron(transpose(wavelet(ny, L, false)), transpose(wavelet(nx + 1, L, false)));
  m.wv_idwt = kron(wavelet(ny + 1, L, false), wavelet(nx, L, false));
  m.wv_idwtT = kron(transpose(wavelet(ny + 1, L, false)), transpose(wavelet(nx, L, false)));

  auto z = [](int n) { return Vec((size_t)n, 0.0); };
  for (Vec* f : {&m.b, &m.h, &m.s, &m.dhdt, &m.accumulation, &m.basal_melt, &m.haf, &m.gf, &m.dsdh,
                 &m.shelf_strain_rate, &m.av_speed, &m.uh, &m.vh, &m.us, &m.vs, &m.ub, &m.vb, &m.bed_speed,
                 &m.weertman_c, &m.beta, &m.beta_eff, &m.tau_bed, &m.eta_av, &m.quad_f1, &m.quad_f2,
                 &m.weertman_c_param, &m.accumulation_param, &m.glen_a_ref, &m.dneg_heta_h, &m.dimplicit})
    *f = z(m.Nh);
  m.dneg_heta_c = z(m.Nc);
  for (Vec* f : {&m.gu_s, &m.gu_h, &m.gu_gf, &m.gu_beff, &m.gu_dnegbeff, &m.u, &m.gu_resid, &m.wu_wav})
    *f = z(m.Nu);
  for (Vec* f : {&m.gv_s, &m.gv_h, &m.gv_gf, &m.gv_beff, &m.gv_dnegbeff, &m.v, &m.gv_resid, &m.wv_wav})
    *f = z(m.Nv);
  for (Vec* f : {&m.eta, &m.temperature, &m.damage, &m.glen_b}) *f = z(m.Nh * m.ns);
  m.wu_mask.assign(m.Nu, 1);  // UWavelets.jl:38 mask = trues
  m.wv_mask.assign(m.Nv, 1);
  m.wu_corr = z(m.Nu);
  m.wv_corr = z(m.Nv);
}

// Fields.jl:39-113 and HGrid.jl:114 — derived initial state once the caller has filled h, b, the
// initial grounded fraction, u, v, η (initial viscosity), temperature, damage and glen_a_ref.
void init_fields(Model& m) {
  for (int i = 0; i < m.Nh; ++i) m.eta_av[i] = m.eta[i];  // ηav = initial_viscosity[:,:,1]
  for (int i = 0; i < m.Nh; ++i) m.quad_f2[i] = m.h_mask[i] ? m.h[i] / (3 * m.eta_av[i]) : 0.0;
  for (int i = 0; i < m.Nh; ++i) m.dsdh[i] = 1.0;
  for (int i = 0; i < m.Nu; ++i) m.gu_gf[i] = 1.0;
  for (int i = 0; i < m.Nv; ++i) m.gv_gf[i] = 1.0;
  // glen_b (utilities.jl:462-466) per (i,j,k), Fields.jl:88-95
  const wavi_params& P = m.P;
  for (int k = 0; k < m.ns; ++k)
    for (int c = 0; c < m.Nh; ++c) {
      size_t q = (size_t)c + (size_t)m.Nh * k;
      double a0 = m.glen_a_ref[c] * std::exp(+P.glen_a_activation_energy / (P.glen_temperature_ref * P.gas_const));
      m.glen_b[q] = (1 - m.damage[q]) *
                    std::pow(a0 * std::exp(-P.glen_a_activation_energy / (m.temperature[q] * P.gas_const)),
                             -1.0 / P.glen_n);
    }
  m.wu_mask.assign(m.Nu, 1);
  m.wv_mask.assign(m.Nv, 1);
  std::fill(m.wu_corr.begin(), m.wu_corr.end(), 0.0);
  std::fill(m.wv_corr.begin(), m.wv_corr.end(), 0.0);
}

// ---------------------------------------------------------------------------------------------
// The matrix-free momentum operator.  utilities.jl:61-145
// ---------------------------------------------------------------------------------------------
struct OpWork {
  Vec uspread, vspread, dudx, dvdy, rxx_sum, ryy_sum, rxx, ryy, dudy_c, dvdx_c, rxy_sum, rxy_sum_crop, rxy, rxy_crop,
      d_rxx_dx, d_rxy_dy, d_ryy_dy, d_rxy_dx, taubx, tauby, qx, qx_crop, dqxdx, qy, qy_crop, dqydy, divq, extra,
      d_extra_dx, d_extra_dy, h_d_extra_dx, h_d_extra_dy, fx, fy;
};

// in_u (Nu), in_v (Nv): full-rectangle velocities (uspread/vspread); out_u / out_v: fx, fy on the full
// rectangles before sampling.
void op_full(Model& m, OpWork& w, const Vec& us_, const Vec& vs_) {
  ++m.op_applies;
  w.uspread = us_;
  w.vspread = vs_;
  const int Nh = m.Nh, Nc = m.Nc, Nu = m.Nu, Nv = m.Nv;
  // Extensional resistive stresses
  w.dudx = m.u_dx * w.uspread;
  w.dvdy = m.v_dy * w.vspread;
  w.rxx_sum.resize(Nh);
  w.ryy_sum.resize(Nh);
  w.rxx.resize(Nh);
  w.ryy.resize(Nh);
  for (int i = 0; i < Nh; ++i) {
    w.rxx_sum[i] = 2 * w.dudx[i] + w.dvdy[i];
    w.ryy_sum[i] = 2 * w.dvdy[i] + w.dudx[i];
    w.rxx[i] = m.dneg_heta_h[i] * w.rxx_sum[i];
    w.rxx[i] = -2 * w.rxx[i];
    w.ryy[i] = m.dneg_heta_h[i] * w.ryy_sum[i];
    w.ryy[i] = -2 * w.ryy[i];
  }
  // Shearing resistive stresses
  w.dudy_c = m.u_dy * w.uspread;
  w.dvdx_c = m.v_dx * w.vspread;
  w.rxy_sum.resize(Nc);
  w.rxy.resize(Nc);
  for (int i = 0; i < Nc; ++i) w.rxy_sum[i] = w.dudy_c[i] + w.dvdx_c[i];
  w.rxy_sum_crop = crop(m.c_mask, w.rxy_sum);
  for (int i = 0; i < Nc; ++i) {
    w.rxy[i] = m.dneg_heta_c[i] * w.rxy_sum_crop[i];
    w.rxy[i] = -w.rxy[i];
  }
  w.rxy_crop = crop(m.c_mask, w.rxy);
  // Gradients of resistive stresses
  w.d_rxx_dx = m.u_dxT * w.rxx;
  w.d_rxy_dy = m.u_dyT * w.rxy_crop;
  w.d_ryy_dy = m.v_dyT * w.ryy;
  w.d_rxy_dx = m.v_dxT * w.rxy_crop;
  for (auto* f : {&w.d_rxx_dx, &w.d_rxy_dy, &w.d_ryy_dy, &w.d_rxy_dx})
    for (double& x : *f) x = -x;
  // Basal drag
  w.taubx.resize(Nu);
  w.tauby.resize(Nv);
  for (int i = 0; i < Nu; ++i) w.taubx[i] = -(m.gu_dnegbeff[i] * w.uspread[i]);
  for (int i = 0; i < Nv; ++i) w.tauby[i] = -(m.gv_dnegbeff[i] * w.vspread[i]);
  // Schur-complement terms of the semi-implicit system
  w.qx.resize(Nu);
  w.qy.resize(Nv);
  for (int i = 0; i < Nu; ++i) w.qx[i] = m.gu_h[i] * w.uspread[i];
  w.qx_crop = crop(m.u_mask, w.qx);
  w.dqxdx = m.u_dx * w.qx_crop;
  for (int i = 0; i < Nv; ++i) w.qy[i] = m.gv_h[i] * w.vspread[i];
  w.qy_crop = crop(m.v_mask, w.qy);
  w.dqydy = m.v_dy * w.qy_crop;
  w.divq.resize(Nh);
  w.extra.resize(Nh);
  for (int i = 0; i < Nh; ++i) {
    w.divq[i] = w.dqxdx[i] + w.dqydy[i];
    w.extra[i] = m.dimplicit[i] * w.divq[i];
  }
  w.d_extra_dx = m.u_dxT * w.extra;
  w.d_extra_dy = m.v_dyT * w.extra;
  for (double& x : w.d_extra_dx) x = -x;
  for (double& x : w.d_extra_dy) x = -x;
  w.h_d_extra_dx.resize(Nu);
  w.h_d_extra_dy.resize(Nv);
  for (int i = 0; i < Nu; ++i) w.h_d_extra_dx[i] = m.gu_h[i] * w.d_extra_dx[i];
  for (int i = 0; i < Nv; ++i) w.h_d_extra_dy[i] = m.gv_h[i] * w.d_extra_dy[i];
  // Resistive forces
  w.fx.resize(Nu);
  w.fy.resize(Nv);
  for (int i = 0; i < Nu; ++i) w.fx[i] = w.d_rxx_dx[i] + w.d_rxy_dy[i] - w.taubx[i] - w.h_d_extra_dx[i];
  for (int i = 0; i < Nv; ++i) w.fy[i] = w.d_ryy_dy[i] + w.d_rxy_dx[i] - w.tauby[i] - w.h_d_extra_dy[i];
}

// op_fun!(out, x) with vecSampled = true: x and out have length ni_u + ni_v.   utilities.jl:62-71,138-142
void op_sampled(Model& m, OpWork& w, const Vec& x, Vec& out) {
  Vec us((size_t)m.Nu, 0.0), vs((size_t)m.Nv, 0.0);
  for (int k = 0; k < m.ni_u; ++k) us[m.u_inner_idx[k]] = x[k];
  for (int k = 0; k < m.ni_v; ++k) vs[m.v_inner_idx[k]] = x[m.ni_u + k];
  op_full(m, w, us, vs);
  out.resize(m.ni_u + m.ni_v);
  for (int k = 0; k < m.ni_u; ++k) out[k] = w.fx[m.u_inner_idx[k]];
  for (int k = 0; k < m.ni_v; ++k) out[m.ni_u + k] = w.fy[m.v_inner_idx[k]];
}

// get_resid!(resid, x, op, b)                                          utilities.jl:549-552
void resid_sampled(Model& m, OpWork& w, const Vec& x, const Vec& b, Vec& r) {
  op_sampled(m, w, x, r);
  for (size_t i = 0; i < r.size(); ++i) r[i] = b[i] - r[i];
}

// ---------------------------------------------------------------------------------------------
// inner_update!  update_velocities.jl:32-45, :202-383
// ---------------------------------------------------------------------------------------------
void update_shelf_strain_rate(Model& m) {  // :202-209
  Vec ucrop = crop(m.u_mask, m.u), vcrop = crop(m.v_mask, m.v);
  Vec ux = crop(m.h_mask, m.u_dx * ucrop);
  Vec vy = crop(m.h_mask, m.v_dy * vcrop);
  Vec uy = m.u_dy * ucrop, vx = m.v_dx * vcrop;
  Vec sh(m.Nc);
  for (int i = 0; i < m.Nc; ++i) sh[i] = uy[i] + vx[i];
  Vec shc = crop(m.h_mask, m.c_cent * crop(m.c_mask, sh));
  for (int i = 0; i < m.Nh; ++i)
    m.shelf_strain_rate[i] = std::sqrt(ux[i] * ux[i] + vy[i] * vy[i] + ux[i] * vy[i] + 0.25 * (shc[i] * shc[i]));
}
void update_av_speed(Model& m) {  // :216-220
  Vec uc = crop(m.h_mask, m.u_cent * crop(m.u_mask, m.u));
  Vec vc = crop(m.h_mask, m.v_cent * crop(m.v_mask, m.v));
  for (int i = 0; i < m.Nh; ++i) m.av_speed[i] = std::sqrt(uc[i] * uc[i] + vc[i] * vc[i]);
}
void update_bed_speed(Model& m) {  // :227-231
  for (int i = 0; i < m.Nh; ++i) m.bed_speed[i] = m.av_speed[i] / (1.0 + m.quad_f2[i] * m.beta[i]);
}
void update_beta(Model& m) {  // :238-243
  const double ur = m.P.weertman_reg_speed, ex = 1.0 / m.P.weertman_m - 1.0;
  for (int i = 0; i < m.Nh; ++i)
    m.beta[i] = m.weertman_c[i] * std::pow(std::sqrt(m.bed_speed[i] * m.bed_speed[i] + ur * ur), ex);
}
void update_basal_drag(Model& m) {  // :251-255
  for (int i = 0; i < m.Nh; ++i) m.tau_bed[i] = m.beta[i] * m.bed_speed[i];
}
void inner_update_viscosity(Model& m) {  // :264-283
  const double ex = 1.0 / m.P.glen_n - 1.0, er = m.P.glen_reg_strain_rate;
  for (int k = 0; k < m.ns; ++k)
    for (int c = 0; c < m.Nh; ++c) {
      if (!m.h_mask[c]) continue;
      size_t q = (size_t)c + (size_t)m.Nh * k;
      for (int it = 0; it < m.S.n_iter_viscosity; ++it) {
        double t = m.tau_bed[c] * m.zeta[k] / m.eta[q];
        double e = m.shelf_strain_rate[c];
        m.eta[q] = 0.5 * m.glen_b[q] * std::pow(std::sqrt(e * e + 0.25 * (t * t) + er * er), ex);
      }
    }
}
void update_av_viscosity(Model& m) {  // :292-305
  std::fill(m.eta_av.begin(), m.eta_av.end(), 0.0);
  for (int k = 0; k < m.ns; ++k)
    for (int c = 0; c < m.Nh; ++c)
      if (m.h_mask[c]) m.eta_av[c] += m.qw[k] * m.eta[(size_t)c + (size_t)m.Nh * k];
}
void update_quadrature_falpha(Model& m) {  // :313-328
  std::fill(m.quad_f1.begin(), m.quad_f1.end(), 0.0);
  std::fill(m.quad_f2.begin(), m.quad_f2.end(), 0.0);
  for (int k = 0; k < m.ns; ++k)
    for (int c = 0; c < m.Nh; ++c)
      if (m.h_mask[c]) {
        double e = m.eta[(size_t)c + (size_t)m.Nh * k];
        m.quad_f1[c] += m.qw[k] * m.h[c] * m.zeta[k] / e;
        m.quad_f2[c] += m.qw[k] * m.h[c] * (m.zeta[k] * m.zeta[k]) / e;
      }
}
void update_beta_eff(Model& m) {  // :335-339
  for (int i = 0; i < m.Nh; ++i) m.beta_eff[i] = m.beta[i] / (1.0 + m.quad_f2[i] * m.beta[i]);
}
// h -> u/v interpolation of a field with valid-neighbour averaging (update_velocities.jl:353,
// update_state.jl:68): samp*(centᵀ*(crop_h*f)) ./ samp*(centᵀ*(crop_h*ones)) at mask points.
void interp_h_to_uv(const Model& m, const Vec& f, const Kron& centT, const Mask& mask, Vec& out) {
  Vec ones((size_t)m.Nh, 1.0);
  Vec num = centT * crop(m.h_mask, f), den = centT * crop(m.h_mask, ones);
  for (size_t i = 0; i < mask.size(); ++i)
    if (mask[i]) out[i] = num[i] / den[i];
}
void update_beta_eff_on_uv_grids(Model& m) {  // :348-366
  interp_h_to_uv(m, m.beta_eff, m.u_centT, m.u_mask, m.gu_beff);
  Vec ipu((size_t)m.Nu, 0.0);
  interp_h_to_uv(m, m.gf, m.u_centT, m.u_mask, ipu);
  for (int i = 0; i < m.Nu; ++i)
    if (ipu[i] > 0.0) m.gu_beff[i] = m.gu_beff[i] * m.gu_gf[i] / ipu[i];
  interp_h_to_uv(m, m.beta_eff, m.v_centT, m.v_mask, m.gv_beff);
  Vec ipv((size_t)m.Nv, 0.0);
  interp_h_to_uv(m, m.gf, m.v_centT, m.v_mask, ipv);
  for (int i = 0; i < m.Nv; ++i)
    if (ipv[i] > 0.0) m.gv_beff[i] = m.gv_beff[i] * m.gv_gf[i] / ipv[i];
}
void update_rheological_operators(Model& m) {  // :374-383
  Vec hn(m.Nh);
  for (int i = 0; i < m.Nh; ++i) {
    double mk = m.h_mask[i] ? 1.0 : 0.0;
    m.dneg_heta_h[i] = (mk * (-m.h[i] * m.eta_av[i])) * mk;
    hn[i] = m.h[i] * m.eta_av[i];
  }
  Vec hc = m.h_cent_xy * hn;
  for (int i = 0; i < m.Nc; ++i) {
    double mk = m.c_mask[i] ? 1.0 : 0.0;
    m.dneg_heta_c[i] = (mk * (-hc[i])) * mk;
  }
  for (int i = 0; i < m.Nu; ++i) {
    double mk = m.u_mask[i] ? 1.0 : 0.0;
    m.gu_dnegbeff[i] = (mk * (-m.gu_beff[i])) * mk;
  }
  for (int i = 0; i < m.Nv; ++i) {
    double mk = m.v_mask[i] ? 1.0 : 0.0;
    m.gv_dnegbeff[i] = (mk * (-m.gv_beff[i])) * mk;
  }
  const double c0 = -m.P.density_ice * m.P.g * m.S.super_implicitness * m.P.dt;
  for (int i = 0; i < m.Nh; ++i) {
    double mk = m.h_mask[i] ? 1.0 : 0.0;
    m.dimplicit[i] = (mk * (c0 * m.dsdh[i])) * mk;
  }
}
void inner_update(Model& m) {  // :32-45
  update_shelf_strain_rate(m);
  update_av_speed(m);
  update_bed_speed(m);
  update_beta(m);
  update_basal_drag(m);
  inner_update_viscosity(m);
  update_av_viscosity(m);
  update_quadrature_falpha(m);
  update_beta_eff(m);
  update_beta_eff_on_uv_grids(m);
  update_rheological_operators(m);
}

// ---------------------------------------------------------------------------------------------
// Right-hand side.  update_velocities.jl:106-182, :406-421; icedraft utilities.jl:436
// ---------------------------------------------------------------------------------------------
inline double icedraft(double s, double h, double sl) { return std::max(h - (s - sl), 0.0); }

void get_rhs(Model& m, OpWork& w, Vec& rhs) {
  const wavi_params& P = m.P;
  Vec sadj(m.Nh);
  for (int i = 0; i < m.Nh; ++i)
    sadj[i] = m.s[i] + m.S.super_implicitness * P.dt * m.dsdh[i] * (m.accumulation[i] - m.basal_melt[i]);
  sadj = crop(m.h_mask, sadj);
  const int ni = m.ni_u + m.ni_v;
  Vec f1((size_t)ni), f2((size_t)ni), f3((size_t)ni);
  Vec tu = m.u_dxT * sadj, tv = m.v_dyT * sadj;
  for (int k = 0; k < m.ni_u; ++k) {
    int q = m.u_inner_idx[k];
    f1[k] = (P.density_ice * P.g * m.gu_h[q]) * (-tu[q]);
  }
  for (int k = 0; k < m.ni_v; ++k) {
    int q = m.v_inner_idx[k];
    f1[m.ni_u + k] = (P.density_ice * P.g * m.gv_h[q]) * (-tv[q]);
  }
  Vec ones((size_t)m.Nh, 1.0);
  Vec hm = crop(m.h_mask, ones);
  Vec eu = m.u_dxT * hm, ev = m.v_dyT * hm;
  for (int k = 0; k < m.ni_u; ++k) {
    int q = m.u_inner_idx[k];
    double hu = m.gu_h[q], su = m.gu_s[q], du = icedraft(su, hu, P.sea_level_wrt_geoid);
    f2[k] = (-eu[q]) * P.g *
            (0.5 * P.density_ice * (hu * hu) - 0.5 * P.density_ocean * (du * du) - P.density_ice * hu * su);
  }
  for (int k = 0; k < m.ni_v; ++k) {
    int q = m.v_inner_idx[k];
    double hv = m.gv_h[q], sv = m.gv_s[q], dv = icedraft(sv, hv, P.sea_level_wrt_geoid);
    f2[m.ni_u + k] = (-ev[q]) * P.g *
                     (0.5 * P.density_ice * (hv * hv) - 0.5 * P.density_ocean * (dv * dv) - P.density_ice * hv * sv);
  }
  // get_rhs_dirichlet!: - op_fun!([u.*u_isfixed; v.*v_isfixed], vecSampled=false)
  Vec uf((size_t)m.Nu), vf((size_t)m.Nv);
  for (int i = 0; i < m.Nu; ++i) uf[i] = m.u_isfixed[i] ? m.u[i] : 0.0;
  for (int i = 0; i < m.Nv; ++i) vf[i] = m.v_isfixed[i] ? m.v[i] : 0.0;
  op_full(m, w, uf, vf);
  for (int k = 0; k < m.ni_u; ++k) f3[k] = -w.fx[m.u_inner_idx[k]];
  for (int k = 0; k < m.ni_v; ++k) f3[m.ni_u + k] = -w.fy[m.v_inner_idx[k]];
  rhs.resize(ni);
  for (int i = 0; i < ni; ++i) rhs[i] = f1[i] + f2[i] + f3[i];
}

// ---------------------------------------------------------------------------------------------
// Preconditioner.  Wavelets/update_preconditioners.jl
// ---------------------------------------------------------------------------------------------
struct Precond {
  Vec op_diag;
  std::vector<int> sweep;  // colour 1..4 of each sampled unknown
  std::vector<int> wu_idx, wv_idx;  // compact coarse index -> full wavelet-grid index
  Vec corr;  // compact coarse correction (warm start)
  int last_cg = 0;
};

// get_op_diag by coloured probing, stencil_margin colours per direction        :92-109
Vec get_op_diag(Model& m, OpWork& w) {
  const int ni = m.ni_u + m.ni_v, sm = m.S.stencil_margin;
  std::vector<int> sw((size_t)ni);
  for (int k = 0; k < m.ni_u; ++k) {
    int q = m.u_inner_idx[k], i = q % (m.nx + 1), j = q / (m.nx + 1);
    sw[k] = 1 + (i % sm) + sm * (j % sm);
  }
  for (int k = 0; k < m.ni_v; ++k) {
    int q = m.v_inner_idx[k], i = q % m.nx, j = q / m.nx;
    sw[m.ni_u + k] = 1 + sm * sm + (i % sm) + sm * (j % sm);
  }
  std::vector<int> order;
  for (int c : sw)
    if (std::find(order.begin(), order.end(), c) == order.end()) order.push_back(c);
  Vec diag((size_t)ni, 0.0), e((size_t)ni), ope;
  for (int c : order) {
    for (int i = 0; i < ni; ++i) e[i] = (sw[i] == c) ? 1.0 : 0.0;
    op_sampled(m, w, e, ope);
    for (int i = 0; i < ni; ++i)
      if (sw[i] == c) diag[i] = ope[i];
  }
  return diag;
}

// restrict_fun! / prolong_fun!                                  utilities.jl:157-241
void restrict_vec(Model& m, const Precond& p, const Vec& x, Vec& out) {
  Vec sx((size_t)m.Nu, 0.0), sy((size_t)m.Nv, 0.0);
  for (int k = 0; k < m.ni_u; ++k) sx[m.u_inner_idx[k]] = x[k];
  for (int k = 0; k < m.ni_v; ++k) sy[m.v_inner_idx[k]] = x[m.ni_u + k];
  Vec bx = m.wu_idwtT * sx, by = m.wv_idwtT * sy;
  out.resize(p.wu_idx.size() + p.wv_idx.size());
  for (size_t k = 0; k < p.wu_idx.size(); ++k) out[k] = bx[p.wu_idx[k]];
  for (size_t k = 0; k < p.wv_idx.size(); ++k) out[p.wu_idx.size() + k] = by[p.wv_idx[k]];
}
void prolong_vec(Model& m, const Precond& p, const Vec& c, Vec& out) {
  Vec sx((size_t)m.Nu, 0.0), sy((size_t)m.Nv, 0.0);
  for (size_t k = 0; k < p.wu_idx.size(); ++k) sx[p.wu_idx[k]] = c[k];
  for (size_t k = 0; k < p.wv_idx.size(); ++k) sy[p.wv_idx[k]] = c[p.wu_idx.size() + k];
  Vec bx = m.wu_idwt * sx, by = m.wv_idwt * sy;
  out.resize(m.ni_u + m.ni_v);
  for (int k = 0; k < m.ni_u; ++k) out[k] = bx[m.u_inner_idx[k]];
  for (int k = 0; k < m.ni_v; ++k) out[m.ni_u + k] = by[m.v_inner_idx[k]];
}
void op_coarse(Model& m, OpWork& w, const Precond& p, const Vec& c, Vec& out) {  // :176-193
  Vec t1, t2;
  prolong_vec(m, p, c, t1);
  op_sampled(m, w, t1, t2);
  restrict_vec(m, p, t2, out);
}

// IterativeSolvers.cg! restated (see file header).  Returns the iteration count.
int coarse_cg(Model& m, OpWork& w, const Precond& p, Vec& x, const Vec& b, double abstol, int maxiter) {
  const size_t n = b.size();
  Vec u(n, 0.0), r = b, c;
  op_coarse(m, w, p, x, c);
  for (size_t i = 0; i < n; ++i) r[i] -= c[i];
  double residual = norm2(r);
  const double reltol = std::sqrt(2.220446049250313e-16);
  const double tol = std::max(reltol * residual, abstol);
  double prev = 1.0;
  int it = 0;
  while (!(it >= maxiter || residual <= tol)) {
    double beta = residual * residual / (prev * prev);
    for (size_t i = 0; i < n; ++i) u[i] = r[i] + beta * u[i];
    op_coarse(m, w, p, u, c);
    double alpha = residual * residual / dotp(u, c);
    for (size_t i = 0; i < n; ++i) x[i] += alpha * u[i];
    for (size_t i = 0; i < n; ++i) r[i] -= alpha * c[i];
    prev = residual;
    residual = norm2(r);
    ++it;
  }
  return it;
}

// ---------------------------------------------------------------------------------------------
// Coarse-solve variants that the reference does not have.  They restate the GPU library's opt-in coarse
// solvers so that those can be checked step for step; the default (0) is the reference's cg!.
//   0  cg! (coarse_cg above)
//   2  single-reduction CG (Chronopoulos & Gear, "s-step iterative methods for symmetric linear
//      systems", J. Comput. Appl. Math. 25 (1989)): the same Krylov iterates in exact arithmetic, with
//      the two inner products of an iteration computed together after its operator application
//   3  the same, preconditioned by the Jacobi diagonal of R A P
//   4  the same, preconditioned by Chebyshev-accelerated Jacobi steps (coarse_srcg_chebyshev)
//   5  pipelined CG with variant 4's preconditioner, restarted after every hundredfold fall of |r|
//      (coarse_pipelined_chebyshev), the GPU library's opt-in WAVI_COARSE_PIPELINED_CHEBYSHEV
// ---------------------------------------------------------------------------------------------
int g_coarse_variant = 0;

// diag(R A P) by probing: the Haar basis functions of one component, one in-block offset and one parity
// of the block position are far enough apart (two blocks of 2^(levels+1) points) that A, a nearest-
// neighbour operator, couples none of them, so one coarse application yields all their diagonal entries.
Vec coarse_diag(Model& m, OpWork& w, const Precond& p) {
  const int B = 1 << (m.S.levels + 1);
  const size_t nu = p.wu_idx.size(), n = nu + p.wv_idx.size();
  Vec d(n, 0.0), e(n), y;
  for (int comp = 0; comp < 2; ++comp) {
    const int nxg = comp == 0 ? m.nx + 1 : m.nx;
    const size_t k0 = comp == 0 ? 0 : nu, k1 = comp == 0 ? nu : n;
    for (int oy = 0; oy < B; ++oy)
      for (int ox = 0; ox < B; ++ox)
        for (int par = 0; par < 4; ++par) {
          std::fill(e.begin(), e.end(), 0.0);
          bool any = false;
          for (size_t k = k0; k < k1; ++k) {
            const int q = comp == 0 ? p.wu_idx[k] : p.wv_idx[k - nu], i = q % nxg, j = q / nxg;
            if (i % B == ox && j % B == oy && (i / B) % 2 == (par & 1) && (j / B) % 2 == (par >> 1)) {
              e[k] = 1.0;
              any = true;
            }
          }
          if (!any) continue;
          op_coarse(m, w, p, e, y);
          for (size_t k = k0; k < k1; ++k)
            if (e[k] != 0.0) d[k] = y[k];
        }
  }
  return d;
}

// Chronopoulos-Gear CG with cg!'s stopping rule on the unpreconditioned residual.  Per iteration:
//   x += α p;  r -= α s;  z = M⁻¹ r;  w = A z;  γ = (r,z), δ = (w,z), |r|;  stop?
//   β = γ/γ';  α = γ/(δ - β γ/α');  p = z + β p;  s = w + β s
// started from r = b - A x, z = M⁻¹ r, w = A z, α = γ/δ, p = z, s = w.
int coarse_srcg(Model& m, OpWork& w, const Precond& p, Vec& x, const Vec& b, double abstol, int maxiter,
                bool jacobi) {
  const size_t n = b.size();
  Vec minv(n, 1.0);
  if (jacobi) {
    Vec d = coarse_diag(m, w, p);
    for (size_t i = 0; i < n; ++i) minv[i] = d[i] != 0.0 ? 1.0 / d[i] : 0.0;
  }
  Vec c, r = b, z(n), wv;
  op_coarse(m, w, p, x, c);
  for (size_t i = 0; i < n; ++i) r[i] -= c[i];
  for (size_t i = 0; i < n; ++i) z[i] = minv[i] * r[i];
  op_coarse(m, w, p, z, wv);
  double gamma = dotp(r, z), delta = dotp(wv, z), res = norm2(r);
  const double reltol = std::sqrt(2.220446049250313e-16);
  const double tol = std::max(reltol * res, abstol);
  Vec pp = z, s = wv;
  double alpha = gamma / delta;
  int it = 0;
  bool stop = it >= maxiter || res <= tol || !(res == res) || !(alpha == alpha) || std::isinf(alpha);
  while (!stop) {
    for (size_t i = 0; i < n; ++i) x[i] += alpha * pp[i];
    for (size_t i = 0; i < n; ++i) r[i] -= alpha * s[i];
    for (size_t i = 0; i < n; ++i) z[i] = minv[i] * r[i];
    op_coarse(m, w, p, z, wv);
    ++it;
    const double g2 = dotp(r, z), d2 = dotp(wv, z);
    res = norm2(r);
    stop = it >= maxiter || res <= tol || !(res == res);
    if (stop) break;
    const double beta = g2 / gamma;
    alpha = g2 / (d2 - beta * g2 / alpha);
    gamma = g2;
    if (!(alpha == alpha) || std::isinf(alpha)) break;
    for (size_t i = 0; i < n; ++i) pp[i] = z[i] + beta * pp[i];
    for (size_t i = 0; i < n; ++i) s[i] = wv[i] + beta * s[i];
  }
  return it;
}

// Variant 4: coarse_srcg with M⁻¹ r replaced by g_cheb_steps steps of the Chebyshev-accelerated Jacobi
// iteration on D⁻¹ R A P z = D⁻¹ r from z = 0 (D = diag(R A P)), on the interval [b / g_cheb_ratio, b],
// b = 1.15 λmax(D⁻¹ R A P).  λmax by power steps (12 in a solve's first V-cycle, then 4) from the
// previous V-cycle's vector (zero at a solve's start) plus 1e-3 times a fixed hash of the full index.
// The GPU library's WAVI_COARSE_SRCG_CHEBYSHEV with its constants, in the same order of operations.
// The GPU library's defaults (wavi_gpu.cu: kChebSteps, kChebRatio); oracle_set_chebyshev changes them.
static int g_cheb_steps = 3;
static double g_cheb_ratio = 120.0;
static float cheb_start(int q) {  // in [-1, 1)
  const unsigned h = (unsigned)q * 2654435761u;
  return (float)((h >> 8) & 0xffffu) * (1.0f / 32768.0f) - 1.0f;
}
// The preconditioner of variants 4 and 5: D⁻¹ and the Chebyshev interval from the power steps.
struct ChebPrec {
  Vec minv;
  double th = 1.0, de = 1.0, sg = 1.0;
};
ChebPrec cheb_setup(Model& m, OpWork& w, const Precond& p) {
  const size_t n = p.wu_idx.size() + p.wv_idx.size(), nu = p.wu_idx.size();
  ChebPrec c;
  Vec d = coarse_diag(m, w, p);
  c.minv.resize(n);
  for (size_t i = 0; i < n; ++i) c.minv[i] = d[i] != 0.0 ? 1.0 / d[i] : 0.0;
  auto full = [&](size_t k) { return k < nu ? p.wu_idx[k] : m.Nu + p.wv_idx[k - nu]; };
  Vec v(n), t;
  for (size_t k = 0; k < n; ++k)
    v[k] = c.minv[k] != 0.0 ? m.cheb_eig[full(k)] + 1e-3 * (double)cheb_start(full(k)) : 0.0;
  ++m.cheb_vcycles;
  const int npow = m.cheb_vcycles <= 1 ? 12 : 4;
  for (int ps = 0; ps < npow; ++ps) {
    op_coarse(m, w, p, v, t);
    for (size_t k = 0; k < n; ++k) t[k] = c.minv[k] * t[k];
    const double tt = dotp(t, t), vv = dotp(v, v);
    const double lam = (vv > 0.0 && tt > 0.0) ? std::sqrt(tt / vv) : 1.0;
    const double bmax = 1.15 * lam, amin = bmax / g_cheb_ratio;
    c.th = 0.5 * (bmax + amin);
    c.de = 0.5 * (bmax - amin);
    c.sg = (bmax + amin) / (bmax - amin);
    const double nrm = tt > 0.0 ? 1.0 / std::sqrt(tt) : 0.0;
    for (size_t k = 0; k < n; ++k) v[k] = t[k] * nrm;
  }
  for (size_t k = 0; k < n; ++k) m.cheb_eig[full(k)] = v[k];
  return c;
}
// z = g_cheb_steps Chebyshev steps on D⁻¹ R A P z = D⁻¹ r from z = 0
void cheb_apply(Model& m, OpWork& w, const Precond& p, const ChebPrec& c, const Vec& r, Vec& z) {
  const size_t n = r.size();
  z.resize(n);
  Vec dd(n), tt2;
  for (size_t k = 0; k < n; ++k) {
    z[k] = c.minv[k] * r[k];
    z[k] = z[k] / c.th;
    dd[k] = z[k];
  }
  double rho = 1.0 / c.sg;
  for (int st = 1; st < g_cheb_steps; ++st) {
    op_coarse(m, w, p, z, tt2);
    const double rn = 1.0 / (2.0 * c.sg - rho), c1 = rn * rho, c2 = 2.0 * rn / c.de;
    for (size_t k = 0; k < n; ++k) {
      dd[k] = c1 * dd[k] + c2 * (c.minv[k] * (r[k] - tt2[k]));
      z[k] = z[k] + dd[k];
    }
    rho = rn;
  }
}

int coarse_srcg_chebyshev(Model& m, OpWork& w, const Precond& p, Vec& x, const Vec& b, double abstol, int maxiter) {
  const size_t n = b.size();
  const ChebPrec cp = cheb_setup(m, w, p);
  Vec c, r = b, z, wv;
  op_coarse(m, w, p, x, c);
  for (size_t i = 0; i < n; ++i) r[i] -= c[i];
  cheb_apply(m, w, p, cp, r, z);
  op_coarse(m, w, p, z, wv);
  double gamma = dotp(r, z), delta = dotp(wv, z), res = norm2(r);
  const double reltol = std::sqrt(2.220446049250313e-16);
  const double tol = std::max(reltol * res, abstol);
  Vec pp = z, s = wv;
  double alpha = gamma / delta;
  int it = 0;
  bool stop = it >= maxiter || res <= tol || !(res == res) || !(alpha == alpha) || std::isinf(alpha);
  while (!stop) {
    for (size_t i = 0; i < n; ++i) x[i] += alpha * pp[i];
    for (size_t i = 0; i < n; ++i) r[i] -= alpha * s[i];
    cheb_apply(m, w, p, cp, r, z);
    op_coarse(m, w, p, z, wv);
    ++it;
    const double g2 = dotp(r, z), d2 = dotp(wv, z);
    res = norm2(r);
    stop = it >= maxiter || res <= tol || !(res == res);
    if (stop) break;
    const double beta = g2 / gamma;
    alpha = g2 / (d2 - beta * g2 / alpha);
    gamma = g2;
    if (!(alpha == alpha) || std::isinf(alpha)) break;
    for (size_t i = 0; i < n; ++i) pp[i] = z[i] + beta * pp[i];
    for (size_t i = 0; i < n; ++i) s[i] = wv[i] + beta * s[i];
  }
  return it;
}

// Variant 5: pipelined CG (Ghysels & Vanroose, "Hiding global synchronization latency in the
// preconditioned Conjugate Gradient algorithm", Parallel Computing 40 (2014) 224-238) with variant 4's
// preconditioner and cg!'s stopping rule.  The same iterates as variant 4 in exact arithmetic; each
// iteration's one reduction depends on nothing that iteration's preconditioner and operator produce, so a
// GPU kernel can run them while the reduction completes.  Per iteration:
//   γ = (r,u), δ = (w,u), |r|;  m = M⁻¹ w;  n = A m;  stop?
//   β = γ/γ', α = γ/(δ − β γ/α')   (β = 0, α = γ/δ in the first iteration)
//   z = n + β z;  q = m + β q;  s = w + β s;  p = u + β p
//   x += α p;  r −= α s;  u −= α q;  w −= α z
// started from r = b − A x, u = M⁻¹ r, w = A u.  The last iteration's m and n are computed and unused,
// as they are on the GPU, where they run before the reduction that stops the loop is known.  In FP32 the
// recursively updated residual drifts from b − A x (by ~1e-4 of ‖b‖ on the coarse systems here), so the
// iteration restarts from x (r, u, w recomputed, β = 0 for that iteration) once |r| has fallen below
// PCG_RESTART_FACTOR times its value at the start or the last restart, decided from the previous
// iteration's reduction, as the GPU library's k_pcg_persistent does.
constexpr double PCG_RESTART_FACTOR = 1e-2;
int coarse_pipelined_chebyshev(Model& m, OpWork& w, const Precond& p, Vec& x, const Vec& b, double abstol,
                               int maxiter) {
  const size_t n = b.size();
  const ChebPrec cp = cheb_setup(m, w, p);
  Vec c, r = b, u, wv, mm, nn;
  op_coarse(m, w, p, x, c);
  for (size_t i = 0; i < n; ++i) r[i] -= c[i];
  cheb_apply(m, w, p, cp, r, u);
  op_coarse(m, w, p, u, wv);
  Vec z(n, 0.0), q(n, 0.0), s(n, 0.0), pp(n, 0.0);
  const double reltol = std::sqrt(2.220446049250313e-16);
  double tol = 0.0, gamma_prev = 0.0, alpha = 0.0, rr_ref = 0.0;
  bool restart_next = false;
  int it = 0;
  for (;;) {
    const bool restart = it > 0 && restart_next;
    if (restart) {
      op_coarse(m, w, p, x, c);
      for (size_t i = 0; i < n; ++i) r[i] = b[i] - c[i];
      cheb_apply(m, w, p, cp, r, u);
      op_coarse(m, w, p, u, wv);
    }
    const double gamma = dotp(r, u), delta = dotp(wv, u), res = norm2(r);
    if (it == 0) tol = std::max(reltol * res, abstol);
    cheb_apply(m, w, p, cp, wv, mm);
    op_coarse(m, w, p, mm, nn);
    if (it >= maxiter || res <= tol || !(res == res)) break;
    double beta = 0.0;
    if (it == 0 || restart) {
      alpha = gamma / delta;
      rr_ref = res * res;
    } else {
      beta = gamma / gamma_prev;
      alpha = gamma / (delta - beta * gamma / alpha);
    }
    if (!(alpha == alpha) || std::isinf(alpha)) break;
    restart_next = res * res < PCG_RESTART_FACTOR * PCG_RESTART_FACTOR * rr_ref;
    gamma_prev = gamma;
    for (size_t i = 0; i < n; ++i) {
      z[i] = nn[i] + beta * z[i];
      q[i] = mm[i] + beta * q[i];
      s[i] = wv[i] + beta * s[i];
      pp[i] = u[i] + beta * pp[i];
    }
    for (size_t i = 0; i < n; ++i) {
      x[i] += alpha * pp[i];
      r[i] -= alpha * s[i];
      u[i] -= alpha * q[i];
      wv[i] -= alpha * z[i];
    }
    ++it;
  }
  return it;
}

// gauss_seidel_smoother! (4-colour Jacobi with a full residual after each colour)   :133-150
void smoother(Model& m, OpWork& w, const Precond& p, Vec& x, const Vec& b, const int* order) {
  Vec r;
  resid_sampled(m, w, x, b, r);
  const double om = m.S.smoother_omega;
  for (int it = 0; it < m.S.nsmooth; ++it)
    for (int oc = 0; oc < 4; ++oc) {
      int col = order[oc];
      for (size_t i = 0; i < x.size(); ++i)
        if (p.sweep[i] == col) x[i] = x[i] + om * r[i] / p.op_diag[i];
      resid_sampled(m, w, x, b, r);
    }
}

// Relative tolerance of the coarse CG.  The reference's: tol_coarse.  With g_coarse_forcing (not in the
// reference; the GPU library's opt-in wavi_options.coarse_forcing = WAVI_FORCING_ADAPTIVE, restated):
// max(tol_coarse, min(0.1, 0.1 x the Picard iteration's relative residual)) — inexact Newton's forcing
// terms (Eisenstat & Walker, SIAM J. Sci. Comput. 17, 1996); only in solves of more than one Picard
// iteration.
int g_coarse_forcing = 0;
double coarse_reltol(const Model& m) {
  return g_coarse_forcing && m.S.maxiter_picard > 1 ? std::max(m.S.tol_coarse, std::min(0.1, 0.1 * m.picard_rel))
                                                    : m.S.tol_coarse;
}

// precondition!(x, p, b) — one V-cycle                                   :54-83
void vcycle(Model& m, OpWork& w, Precond& p, Vec& x, const Vec& b) {
  static const int fwd[4] = {1, 3, 2, 4}, bwd[4] = {4, 2, 3, 1};
  smoother(m, w, p, x, b, fwd);
  Vec r;
  resid_sampled(m, w, x, b, r);
  Vec bc;
  restrict_vec(m, p, r, bc);
  double abstol = coarse_reltol(m) * norm2(bc);
  m.last_coarse_b = bc;
  m.last_coarse_x0 = p.corr;
  p.last_cg = g_coarse_variant == 0   ? coarse_cg(m, w, p, p.corr, bc, abstol, m.S.maxiter_coarse)
              : g_coarse_variant == 4 ? coarse_srcg_chebyshev(m, w, p, p.corr, bc, abstol, m.S.maxiter_coarse)
              : g_coarse_variant == 5 ? coarse_pipelined_chebyshev(m, w, p, p.corr, bc, abstol, m.S.maxiter_coarse)
                                      : coarse_srcg(m, w, p, p.corr, bc, abstol, m.S.maxiter_coarse, g_coarse_variant == 3);
  Vec pc;
  prolong_vec(m, p, p.corr, pc);
  for (size_t i = 0; i < x.size(); ++i) x[i] = x[i] + pc[i];
  smoother(m, w, p, x, b, bwd);
}

// ---------------------------------------------------------------------------------------------
// Anderson acceleration of the Picard loop (not in the reference; the GPU library's opt-in
// wavi_options.picard_accel = WAVI_PICARD_ANDERSON, restated step for step).  Walker & Ni, "Anderson
// acceleration for fixed-point iterations", SIAM J. Numer. Anal. 49 (2011), with the Picard iteration
// x -> g(x) = x + V(x)(b(x) - A(x) x) (relinearisation, one V-cycle) as the fixed-point map.  The
// acceleration starts at the first Picard iteration whose relative residual is below start_rel (the
// iterations before it, from u = 0 and the default viscosity, are far from the asymptotic regime);
// from then on each iteration keeps f = g(x) - x and g = g(x), stores the differences of consecutive
// f and g in a ring of `depth` columns, and moves to x = g - dG gamma with gamma the least-squares
// solution of min |f - dF gamma|: the normal equations with the columns newest first, by Cholesky;
// at the first pivot that falls below 1e-10 of its diagonal entry (a column numerically in the span
// of the newer ones) that column and every older one are left out.
// ---------------------------------------------------------------------------------------------
int g_aa_depth = 0;           // 0: the reference's plain Picard iteration
double g_aa_start_rel = 0.3;  // first relative residual at which the acceleration acts
constexpr int kAAMax = 5;
constexpr double kAAPivot = 1e-10;

struct Anderson {
  bool started = false, have_prev = false;
  int cols = 0, head = 0;  // columns held, next ring slot
  Vec dF[kAAMax], dG[kAAMax], fprev, gprev;
};

// The accelerated iterate from x (before the V-cycle) and the V-cycle's correction f (g = x + f);
// returns the columns used.
int anderson_step(Anderson& a, const Vec& x, const Vec& f, Vec& out) {
  const size_t n = x.size();
  const int depth = std::min(g_aa_depth, kAAMax);
  Vec g(n);
  for (size_t i = 0; i < n; ++i) g[i] = x[i] + f[i];
  if (a.have_prev) {
    Vec& cf = a.dF[a.head];
    Vec& cg = a.dG[a.head];
    cf.resize(n);
    cg.resize(n);
    for (size_t i = 0; i < n; ++i) {
      cf[i] = f[i] - a.fprev[i];
      cg[i] = g[i] - a.gprev[i];
    }
    a.head = (a.head + 1) % depth;
    a.cols = std::min(a.cols + 1, depth);
  }
  a.fprev = f;
  a.gprev = g;
  a.have_prev = true;
  out = g;
  if (a.cols == 0) return 0;
  int slot[kAAMax];  // newest first
  for (int k = 0; k < a.cols; ++k) slot[k] = ((a.head - 1 - k) % depth + depth) % depth;
  double G[kAAMax][kAAMax], rhs[kAAMax], L[kAAMax][kAAMax] = {};
  for (int p = 0; p < a.cols; ++p) {
    for (int q = 0; q <= p; ++q) G[p][q] = G[q][p] = dotp(a.dF[slot[p]], a.dF[slot[q]]);
    rhs[p] = dotp(a.dF[slot[p]], f);
  }
  int used = 0;
  for (int p = 0; p < a.cols; ++p) {
    for (int q = 0; q < p; ++q) {
      double s = G[p][q];
      for (int k = 0; k < q; ++k) s -= L[p][k] * L[q][k];
      L[p][q] = s / L[q][q];
    }
    double s = G[p][p];
    for (int k = 0; k < p; ++k) s -= L[p][k] * L[p][k];
    if (!(s > kAAPivot * G[p][p])) break;
    L[p][p] = std::sqrt(s);
    used = p + 1;
  }
  double y[kAAMax], gam[kAAMax];
  for (int p = 0; p < used; ++p) {
    double s = rhs[p];
    for (int k = 0; k < p; ++k) s -= L[p][k] * y[k];
    y[p] = s / L[p][p];
  }
  for (int p = used - 1; p >= 0; --p) {
    double s = y[p];
    for (int k = p + 1; k < used; ++k) s -= L[k][p] * gam[k];
    gam[p] = s / L[p][p];
  }
  for (int p = 0; p < used; ++p) {
    const Vec& c = a.dG[slot[p]];
    for (size_t i = 0; i < n; ++i) out[i] -= gam[p] * c[i];
  }
  return used;
}

// precondition!(model, ::BasicParallelSpec)                              update_velocities.jl:50-83
bool precondition_model(Model& m, OpWork& w, double& rel, Anderson* aa = nullptr) {
  const int ni = m.ni_u + m.ni_v;
  Vec x((size_t)ni);  // get_start_guess :92-97
  for (int k = 0; k < m.ni_u; ++k) x[k] = m.u[m.u_inner_idx[k]];
  for (int k = 0; k < m.ni_v; ++k) x[m.ni_u + k] = m.v[m.v_inner_idx[k]];
  Vec b;
  get_rhs(m, w, b);
  Vec r;
  resid_sampled(m, w, x, b, r);
  for (int k = 0; k < m.ni_u; ++k) m.gu_resid[m.u_inner_idx[k]] = r[k];  // set_residual! :428-433
  for (int k = 0; k < m.ni_v; ++k) m.gv_resid[m.v_inner_idx[k]] = r[m.ni_u + k];
  rel = norm2(r) / norm2(b);
  bool converged = rel < m.S.tol_picard;
  m.picard_rel = rel;
  Vec corr((size_t)ni, 0.0);
  if (!converged) {
    Precond p;  // get_preconditioner :7-43
    for (int i = 0; i < m.Nu; ++i)
      if (m.wu_mask[i]) p.wu_idx.push_back(i);
    for (int i = 0; i < m.Nv; ++i)
      if (m.wv_mask[i]) p.wv_idx.push_back(i);
    p.corr.resize(p.wu_idx.size() + p.wv_idx.size());  // get_correction_coarse(model) :195-205
    for (size_t k = 0; k < p.wu_idx.size(); ++k) p.corr[k] = m.wu_corr[p.wu_idx[k]];
    for (size_t k = 0; k < p.wv_idx.size(); ++k) p.corr[p.wu_idx.size() + k] = m.wv_corr[p.wv_idx[k]];
    p.op_diag = get_op_diag(m, w);
    p.sweep.resize(ni);
    for (int k = 0; k < m.ni_u; ++k) {
      int q = m.u_inner_idx[k], i = q % (m.nx + 1) + 1, j = q / (m.nx + 1) + 1;  // 1-based
      p.sweep[k] = 1 + (((i - j) % 2) + 2) % 2;
    }
    for (int k = 0; k < m.ni_v; ++k) {
      int q = m.v_inner_idx[k], i = q % m.nx + 1, j = q / m.nx + 1;
      p.sweep[m.ni_u + k] = 3 + (((i - j) % 2) + 2) % 2;
    }
    vcycle(m, w, p, corr, r);
    m.last_cg_iters += p.last_cg;
    m.cg_iter_history.push_back(p.last_cg);
    for (size_t k = 0; k < p.wu_idx.size(); ++k) m.wu_corr[p.wu_idx[k]] = p.corr[k];  // set_correction_coarse!
    for (size_t k = 0; k < p.wv_idx.size(); ++k) m.wv_corr[p.wv_idx[k]] = p.corr[p.wu_idx.size() + k];
  }
  if (aa && !converged && !aa->started && rel < g_aa_start_rel) aa->started = true;
  if (aa && !converged && aa->started) {
    Vec xa;
    anderson_step(*aa, x, corr, xa);
    for (int i = 0; i < ni; ++i) {
      corr[i] = xa[i] - x[i];  // the iteration's whole update
      x[i] = xa[i];
    }
  } else {
    for (int i = 0; i < ni; ++i) x[i] = x[i] + corr[i];
  }
  m.rel_history.push_back(rel);
  m.upd_history.push_back(converged ? 0.0 : norm2(corr) / norm2(x));
  for (int k = 0; k < m.ni_u; ++k) m.u[m.u_inner_idx[k]] = x[k];  // set_velocities! :190-195
  for (int k = 0; k < m.ni_v; ++k) m.v[m.v_inner_idx[k]] = x[m.ni_u + k];
  return converged;
}

// update_velocities!                                                     update_velocities.jl:11-29
void update_velocities(Model& m) {
  OpWork w;
  bool converged = false;
  int it = 0;
  double rel = INFINITY;
  m.last_cg_iters = 0;
  m.cg_iter_history.clear();
  m.rel_history.clear();
  m.upd_history.clear();
  m.cheb_eig.assign((size_t)(m.Nu + m.Nv), 0.0);
  m.cheb_vcycles = 0;
  Anderson aa;
  while (!converged && it < m.S.maxiter_picard) {
    ++it;
    inner_update(m);
    converged = precondition_model(m, w, rel, g_aa_depth > 0 ? &aa : nullptr);
  }
  m.last_picard = it;
  m.last_rel_resid = rel;
}

// ---------------------------------------------------------------------------------------------
// update_state! neighbours.  Models/update_state.jl, utilities.jl:255-396
// ---------------------------------------------------------------------------------------------
void update_surface_elevation(Model& m) {  // :51-57
  const wavi_params& P = m.P;
  for (int i = 0; i < m.Nh; ++i)
    if (m.h_mask[i])
      m.s[i] = std::max(m.b[i] + m.h[i], P.sea_level_wrt_geoid + m.h[i] * (1 - P.density_ice / P.density_ocean));
}
void update_geometry_on_uv_grids(Model& m) {  // :65-73
  interp_h_to_uv(m, m.h, m.u_centT, m.u_mask, m.gu_h);
  interp_h_to_uv(m, m.s, m.u_centT, m.u_mask, m.gu_s);
  interp_h_to_uv(m, m.h, m.v_centT, m.v_mask, m.gv_h);
  interp_h_to_uv(m, m.s, m.v_centT, m.v_mask, m.gv_s);
}
void update_haf(Model& m) {  // :80-85, utilities.jl:445
  const wavi_params& P = m.P;
  for (int i = 0; i < m.Nh; ++i)
    m.haf[i] = m.h[i] - (P.density_ocean / P.density_ice) * (P.sea_level_wrt_geoid - m.b[i]);
}

// pos_fraction(z1; mask)                                               utilities.jl:255-396
void pos_fraction(const Model& m, const Vec& z1, const Mask& mask, Vec& af, Vec& afu, Vec& afv) {
  const int M = m.nx, N = m.ny;
  af.assign((size_t)M * N, 0.0);
  afu.assign((size_t)(M + 1) * N, 0.0);
  afv.assign((size_t)M * (N + 1), 0.0);
  auto at = [&](int i, int j) { return i + M * j; };
  auto sgn = [](double x) { return (double)((x > 0) - (x < 0)); };
  for (int q = 1; q <= 4; ++q) {
    Vec afq((size_t)M * N, 0.0);
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < M; ++i) {
        int i2, j2, i3, j3;  // neighbour positions for z2 and z3
        int ip = std::min(i + 1, M - 1), im = std::max(i - 1, 0), jp = std::min(j + 1, N - 1), jm = std::max(j - 1, 0);
        if (q == 1) { i2 = ip; j2 = j; i3 = i; j3 = jp; }
        else if (q == 2) { i2 = i; j2 = jp; i3 = im; j3 = j; }
        else if (q == 3) { i2 = im; j2 = j; i3 = i; j3 = jm; }
        else { i2 = i; j2 = jm; i3 = ip; j3 = j; }
        double a1z = z1[at(i, j)];
        double z2 = mask[at(i2, j2)] ? z1[at(i2, j2)] : a1z;
        double z3 = mask[at(i3, j3)] ? z1[at(i3, j3)] : a1z;
        double z = a1z, val = 0.0;
        bool sc = !((sgn(z) == sgn(z2)) && (sgn(z) == sgn(z3)));
        if (sc) {
          bool flip = std::fabs(z3 - z) < std::fabs(z2 - z);
          double a, bb;
          if (!flip) {
            a = -(z2 - z) / (z3 - z);
            bb = -2 * z / (z3 - z);
          } else {
            a = -(z3 - z) / (z2 - z);
            bb = -2 * z / (z2 - z);
          }
          double A1 = 0.5 * (bb * bb) / a;
          double A2 = 0.5 * ((1.0 - bb) * (1.0 - bb)) / a;
          double A3 = 0.5 * a + bb;
          int t1 = (bb > 0.0) + (bb > 1.0);
          int t2 = ((a + bb) > 0.0) + ((a + bb) > 1.0);
          int ix = 1 + t1 + 3 * t2;
          double ar = 0.0;
          switch (ix) {
            case 1: ar = 0.0; break;
            case 2: ar = -A1; break;
            case 3: ar = A2 - A1; break;
            case 4: ar = A1 + A3; break;
            case 5: ar = A3; break;
            case 6: ar = A2 + A3; break;
            case 7: ar = 1.0 - A2 + A1; break;
            case 8: ar = 1.0 - A2; break;
            default: ar = 1.0; break;
          }
          if (bb < 0.0) ar = 1.0 - ar;
          if (z < 0.0) ar = 1.0 - ar;
          val = ar;
        }
        if (z > 0.0 && z2 > 0.0 && z3 > 0.0) val = 1.0;
        if (z <= 0.0 && z2 <= 0.0 && z3 <= 0.0) val = 0.0;
        if (!mask[at(i, j)]) val = 0.0;
        afq[at(i, j)] = val;
      }
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < M; ++i) {
        double a = afq[at(i, j)];
        af[at(i, j)] = af[at(i, j)] + 0.25 * a;
        int iu = (q == 1 || q == 4) ? i + 1 : i;  // [zeros(1,n); afq] for q = 1, 4
        afu[iu + (M + 1) * j] = afu[iu + (M + 1) * j] + 0.25 * a;
        int jv = (q == 1 || q == 2) ? j + 1 : j;  // [zeros(m,1) afq] for q = 1, 2
        afv[i + M * jv] = afv[i + M * jv] + 0.25 * a;
      }
  }
}
void update_grounded_fraction(Model& m) {  // :92-99
  pos_fraction(m, m.haf, m.h_mask, m.gf, m.gu_gf, m.gv_gf);
}
void update_accumulation_rate(Model& m) { m.accumulation = m.accumulation_param; }  // :106-111
void update_basal_melt(Model& m) { std::fill(m.basal_melt.begin(), m.basal_melt.end(), m.melt_m); }
void update_weertman_c(Model& m) {  // :129-134
  for (int i = 0; i < m.Nh; ++i) m.weertman_c[i] = m.weertman_c_param[i] * m.gf[i];
}
void update_dsdh(Model& m) {  // :141-147
  const double r = m.P.density_ice / m.P.density_ocean;
  for (int i = 0; i < m.Nh; ++i) m.dsdh[i] = (1.0 - r) + r * m.gf[i];
}
void update_velocities_on_h_grid(Model& m) {  // :164-178
  m.uh = m.u_cent * m.u;
  m.vh = m.v_cent * m.v;
  for (int i = 0; i < m.Nh; ++i) {
    m.ub[i] = m.uh[i] / (1 + (m.beta[i] * m.quad_f2[i]));
    m.vb[i] = m.vh[i] / (1 + (m.beta[i] * m.quad_f2[i]));
    m.us[i] = m.ub[i] * (1 + (m.beta[i] * m.quad_f1[i]));
    m.vs[i] = m.vb[i] * (1 + (m.beta[i] * m.quad_f1[i]));
  }
}
void update_dhdt(Model& m) {  // :184-189
  Vec qx((size_t)m.Nu), qy((size_t)m.Nv);
  for (int i = 0; i < m.Nu; ++i) qx[i] = m.gu_h[i] * m.u[i];
  for (int i = 0; i < m.Nv; ++i) qy[i] = m.gv_h[i] * m.v[i];
  Vec a = m.u_dx * crop(m.u_mask, qx), c = m.v_dy * crop(m.v_mask, qy);
  for (int i = 0; i < m.Nh; ++i)
    if (m.h_mask[i]) m.dhdt[i] = m.accumulation[i] - m.basal_melt[i] - (a[i] + c[i]);
}
void update_wavelets(Model& m) {  // Wavelets/update_wavelets.jl:6-32
  m.wu_wav = m.u_dwt * crop(m.u_mask, m.u);
  m.wv_wav = m.v_dwt * crop(m.v_mask, m.v);
  for (int i = 0; i < m.Nu; ++i) m.wu_mask[i] = std::fabs(m.wu_wav[i]) >= m.S.wavelet_threshold;
  for (int i = 0; i < m.Nv; ++i) m.wv_mask[i] = std::fabs(m.wv_wav[i]) >= m.S.wavelet_threshold;
  std::fill(m.wu_corr.begin(), m.wu_corr.end(), 0.0);
  std::fill(m.wv_corr.begin(), m.wv_corr.end(), 0.0);
}
// update_state! steps before the velocity solve (update_state.jl:8-15)
void pre_solve(Model& m) {
  update_surface_elevation(m);
  update_geometry_on_uv_grids(m);
  update_haf(m);
  update_grounded_fraction(m);
  update_accumulation_rate(m);
  update_basal_melt(m);
  update_weertman_c(m);
  update_dsdh(m);
}
void post_solve(Model& m) {  // update_state.jl:17-19
  update_velocities_on_h_grid(m);
  update_dhdt(m);
  update_wavelets(m);
}
void update_state(Model& m) {  // update_state.jl:7-21
  pre_solve(m);
  update_velocities(m);
  post_solve(m);
}
// update_thickness!                                                  Simulations/run_simulation.jl:24-42
void update_thickness(Model& m, double dt) {
  Vec hup((size_t)m.Nh, 0.0);
  for (int i = 0; i < m.Nh; ++i)
    if (m.h_mask[i]) hup[i] = std::max(m.P.minimum_thickness - m.h[i], dt * m.dhdt[i]);
  // the evolveShelves == false branch (ImageFiltering imfilter) is not restated; callers must keep it true
  for (int i = 0; i < m.Nh; ++i)
    if (m.h_isfixed[i]) hup[i] = 0;
  for (int i = 0; i < m.Nh; ++i)
    if (m.h_mask[i]) m.h[i] = m.h[i] + hup[i];
}

Vec* field_by_name(Model& m, const std::string& n) {
#define F(name, member) \
  if (n == name) return &m.member;
  F("b", b) F("h", h) F("s", s) F("dhdt", dhdt) F("accumulation", accumulation) F("basal_melt", basal_melt)
  F("haf", haf) F("grounded_fraction", gf) F("dsdh", dsdh) F("shelf_strain_rate", shelf_strain_rate)
  F("av_speed", av_speed) F("uh", uh) F("vh", vh) F("us", us) F("vs", vs) F("ub", ub) F("vb", vb)
  F("bed_speed", bed_speed) F("weertman_c", weertman_c) F("beta", beta) F("beta_eff", beta_eff)
  F("tau_bed", tau_bed) F("eta_av", eta_av) F("quad_f1", quad_f1) F("quad_f2", quad_f2)
  F("weertman_c_param", weertman_c_param) F("accumulation_param", accumulation_param) F("glen_a_ref", glen_a_ref)
  F("dneg_heta_h", dneg_heta_h) F("dimplicit", dimplicit) F("dneg_heta_c", dneg_heta_c)
  F("gu_s", gu_s) F("gu_h", gu_h) F("gu_grounded_fraction", gu_gf) F("gu_beta_eff", gu_beff)
  F("gu_dnegbeff", gu_dnegbeff) F("u", u) F("gu_residual", gu_resid)
  F("gv_s", gv_s) F("gv_h", gv_h) F("gv_grounded_fraction", gv_gf) F("gv_beta_eff", gv_beff)
  F("gv_dnegbeff", gv_dnegbeff) F("v", v) F("gv_residual", gv_resid)
  F("eta", eta) F("temperature", temperature) F("damage", damage) F("glen_b", glen_b)
  F("wu_correction_full", wu_corr) F("wv_correction_full", wv_corr) F("wu_wavelets", wu_wav) F("wv_wavelets", wv_wav)
  F("coarse_b", last_coarse_b) F("coarse_x0", last_coarse_x0)
#undef F
  return nullptr;
}
Mask* mask_by_name(Model& m, const std::string& n) {
#define F(name, member) \
  if (n == name) return &m.member;
  F("h_mask", h_mask) F("h_isfixed", h_isfixed) F("u_mask", u_mask) F("v_mask", v_mask) F("c_mask", c_mask)
  F("u_inner", u_inner) F("v_inner", v_inner) F("u_isfixed", u_isfixed) F("v_isfixed", v_isfixed)
  F("wu_mask", wu_mask) F("wv_mask", wv_mask)
#undef F
  return nullptr;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// C ABI (ctypes).  Test infrastructure only.
// ---------------------------------------------------------------------------------------------
extern "C" {

void* oracle_create(const wavi_grid_desc* g, const wavi_params* p, const wavi_solver_params* sp) {
  if (!g || !p || !sp || g->nx < 2 || g->ny < 2 || g->nsigma < 2) return nullptr;
  Model* m = new Model();
  build_model(*m, g, p, sp);
  return m;
}
void oracle_destroy(void* h) { delete static_cast<Model*>(h); }
void oracle_set_sum_order(int order) { g_sum_order = order; }

// Pointer to a float64 field (length written to *len), or null for an unknown name.
double* oracle_field(void* h, const char* name, int64_t* len) {
  Vec* f = field_by_name(*static_cast<Model*>(h), name);
  if (!f) return nullptr;
  if (len) *len = (int64_t)f->size();
  return f->data();
}
uint8_t* oracle_mask(void* h, const char* name, int64_t* len) {
  Mask* f = mask_by_name(*static_cast<Model*>(h), name);
  if (!f) return nullptr;
  if (len) *len = (int64_t)f->size();
  return f->data();
}
void oracle_set_params(void* h, const wavi_params* p, const wavi_solver_params* sp, double melt_m) {
  Model& m = *static_cast<Model*>(h);
  if (p) m.P = *p;
  if (sp) m.S = *sp;
  m.melt_m = melt_m;
}
void oracle_init_fields(void* h) { init_fields(*static_cast<Model*>(h)); }
void oracle_pre_solve(void* h) { pre_solve(*static_cast<Model*>(h)); }
void oracle_update_velocities(void* h) { update_velocities(*static_cast<Model*>(h)); }
void oracle_post_solve(void* h) { post_solve(*static_cast<Model*>(h)); }
void oracle_update_state(void* h) { update_state(*static_cast<Model*>(h)); }
void oracle_update_thickness(void* h, double dt) { update_thickness(*static_cast<Model*>(h), dt); }
void oracle_update_wavelets(void* h) { update_wavelets(*static_cast<Model*>(h)); }
void oracle_inner_update(void* h) { inner_update(*static_cast<Model*>(h)); }
// n timesteps of run_simulation! (timestep!: update_state!, update_thickness!), run_simulation.jl:6-17,61-100
void oracle_run(void* h, int nsteps, double dt) {
  Model& m = *static_cast<Model*>(h);
  m.P.dt = dt;  // set_dt_in_model! (Simulation.jl:56-59)
  for (int i = 0; i < nsteps; ++i) {
    update_state(m);
    update_thickness(m, dt);
  }
}
// op_fun!(out, [u; v], vecSampled=false) on full rectangles; outputs sampled at the interior (zero elsewhere)
void oracle_apply_operator(void* h, const double* u, const double* v, double* fu, double* fv) {
  Model& m = *static_cast<Model*>(h);
  OpWork w;
  op_full(m, w, Vec(u, u + m.Nu), Vec(v, v + m.Nv));
  for (int i = 0; i < m.Nu; ++i) fu[i] = m.u_inner[i] ? w.fx[i] : 0.0;
  for (int i = 0; i < m.Nv; ++i) fv[i] = m.v_inner[i] ? w.fy[i] : 0.0;
}
// get_rhs on full rectangles (zero off the interior)
void oracle_rhs(void* h, double* bu, double* bv) {
  Model& m = *static_cast<Model*>(h);
  OpWork w;
  Vec b;
  get_rhs(m, w, b);
  std::fill(bu, bu + m.Nu, 0.0);
  std::fill(bv, bv + m.Nv, 0.0);
  for (int k = 0; k < m.ni_u; ++k) bu[m.u_inner_idx[k]] = b[k];
  for (int k = 0; k < m.ni_v; ++k) bv[m.v_inner_idx[k]] = b[m.ni_u + k];
}
// probed operator diagonal on full rectangles
void oracle_op_diag(void* h, double* du, double* dv) {
  Model& m = *static_cast<Model*>(h);
  OpWork w;
  Vec d = get_op_diag(m, w);
  std::fill(du, du + m.Nu, 0.0);
  std::fill(dv, dv + m.Nv, 0.0);
  for (int k = 0; k < m.ni_u; ++k) du[m.u_inner_idx[k]] = d[k];
  for (int k = 0; k < m.ni_v; ++k) dv[m.v_inner_idx[k]] = d[m.ni_u + k];
}
// Haar transforms on full rectangles: which = 0 idwt (reverse), 1 idwtᵀ, 2 dwt (forward); grid 0 = u, 1 = v
void oracle_haar(void* h, int grid, int which, const double* x, double* y) {
  Model& m = *static_cast<Model*>(h);
  const Kron* k = grid == 0 ? (which == 0 ? &m.wu_idwt : which == 1 ? &m.wu_idwtT : &m.u_dwt)
                            : (which == 0 ? &m.wv_idwt : which == 1 ? &m.wv_idwtT : &m.v_dwt);
  k->apply(x, y);
}
// One V-cycle precondition!(corr, p, resid) with the model's current coarse space and correction cache,
// on full rectangles (interior points only).  Returns the coarse CG iteration count.
int oracle_vcycle(void* h, const double* ru, const double* rv, double* cu, double* cv) {
  Model& m = *static_cast<Model*>(h);
  OpWork w;
  const int ni = m.ni_u + m.ni_v;
  Vec r((size_t)ni), x((size_t)ni, 0.0);
  for (int k = 0; k < m.ni_u; ++k) r[k] = ru[m.u_inner_idx[k]];
  for (int k = 0; k < m.ni_v; ++k) r[m.ni_u + k] = rv[m.v_inner_idx[k]];
  Precond p;
  for (int i = 0; i < m.Nu; ++i)
    if (m.wu_mask[i]) p.wu_idx.push_back(i);
  for (int i = 0; i < m.Nv; ++i)
    if (m.wv_mask[i]) p.wv_idx.push_back(i);
  p.corr.resize(p.wu_idx.size() + p.wv_idx.size());
  for (size_t k = 0; k < p.wu_idx.size(); ++k) p.corr[k] = m.wu_corr[p.wu_idx[k]];
  for (size_t k = 0; k < p.wv_idx.size(); ++k) p.corr[p.wu_idx.size() + k] = m.wv_corr[p.wv_idx[k]];
  p.op_diag = get_op_diag(m, w);
  p.sweep.resize(ni);
  for (int k = 0; k < m.ni_u; ++k) {
    int q = m.u_inner_idx[k], i = q % (m.nx + 1) + 1, j = q / (m.nx + 1) + 1;
    p.sweep[k] = 1 + (((i - j) % 2) + 2) % 2;
  }
  for (int k = 0; k < m.ni_v; ++k) {
    int q = m.v_inner_idx[k], i = q % m.nx + 1, j = q / m.nx + 1;
    p.sweep[m.ni_u + k] = 3 + (((i - j) % 2) + 2) % 2;
  }
  vcycle(m, w, p, x, r);
  std::fill(cu, cu + m.Nu, 0.0);
  std::fill(cv, cv + m.Nv, 0.0);
  for (int k = 0; k < m.ni_u; ++k) cu[m.u_inner_idx[k]] = x[k];
  for (int k = 0; k < m.ni_v; ++k) cv[m.v_inner_idx[k]] = x[m.ni_u + k];
  for (size_t k = 0; k < p.wu_idx.size(); ++k) m.wu_corr[p.wu_idx[k]] = p.corr[k];
  for (size_t k = 0; k < p.wv_idx.size(); ++k) m.wv_corr[p.wv_idx[k]] = p.corr[p.wu_idx.size() + k];
  return p.last_cg;
}
void oracle_set_coarse_variant(int variant) { g_coarse_variant = variant; }
// The adaptive coarse tolerance in later V-cycles (1) or the reference's tol_coarse (0).
void oracle_set_coarse_forcing(int on) { g_coarse_forcing = on ? 1 : 0; }
// Anderson acceleration of later solves: depth 0 (the reference's Picard loop) or 1..5 columns, from the
// first Picard iteration whose relative residual is below start_rel.
void oracle_set_anderson(int depth, double start_rel) {
  g_aa_depth = std::max(0, std::min(depth, kAAMax));
  g_aa_start_rel = start_rel;
}
// The Chebyshev preconditioner of variants 4 and 5: steps per application (odd, >= 1) and the interval's
// ratio b / a.
void oracle_set_chebyshev(int steps, double ratio) {
  g_cheb_steps = steps;
  g_cheb_ratio = ratio;
}
// diag(R A P) of the model's current linearisation and coarse space, scattered to the full wavelet
// grids (zero off the coarse space).
void oracle_coarse_diag(void* h, double* du, double* dv) {
  Model& m = *static_cast<Model*>(h);
  OpWork w;
  Precond p;
  for (int i = 0; i < m.Nu; ++i)
    if (m.wu_mask[i]) p.wu_idx.push_back(i);
  for (int i = 0; i < m.Nv; ++i)
    if (m.wv_mask[i]) p.wv_idx.push_back(i);
  Vec d = coarse_diag(m, w, p);
  std::fill(du, du + m.Nu, 0.0);
  std::fill(dv, dv + m.Nv, 0.0);
  for (size_t k = 0; k < p.wu_idx.size(); ++k) du[p.wu_idx[k]] = d[k];
  for (size_t k = 0; k < p.wv_idx.size(); ++k) dv[p.wv_idx[k]] = d[p.wu_idx.size() + k];
}
// statistics of the last update_velocities!
void oracle_stats(void* h, int* picard, double* rel_resid, int64_t* cg_iters, int64_t* op_applies) {
  Model& m = *static_cast<Model*>(h);
  if (picard) *picard = m.last_picard;
  if (rel_resid) *rel_resid = m.last_rel_resid;
  if (cg_iters) *cg_iters = m.last_cg_iters;
  if (op_applies) *op_applies = m.op_applies;
}
int oracle_cg_history(void* h, int* out, int cap) {
  Model& m = *static_cast<Model*>(h);
  int n = (int)m.cg_iter_history.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = m.cg_iter_history[i];
  return n;
}
// the last solve's per-Picard-iteration relative residual (before the correction) and relative update
int oracle_picard_history(void* h, double* rel, double* upd, int cap) {
  Model& m = *static_cast<Model*>(h);
  int n = (int)m.rel_history.size();
  for (int i = 0; i < n && i < cap; ++i) {
    if (rel) rel[i] = m.rel_history[i];
    if (upd) upd[i] = m.upd_history[i];
  }
  return n;
}
// pos_fraction on an arbitrary m x n array (KAT hook, utilities.jl:255-396)
void oracle_pos_fraction(int M, int N, const double* z, const uint8_t* mask, double* af, double* afu, double* afv) {
  Model m;
  m.nx = M;
  m.ny = N;
  Vec zz(z, z + (size_t)M * N), a, au, av;
  Mask mk(mask, mask + (size_t)M * N);
  pos_fraction(m, zz, mk, a, au, av);
  std::copy(a.begin(), a.end(), af);
  std::copy(au.begin(), au.end(), afu);
  std::copy(av.begin(), av.end(), afv);
}
// Kronecker-product KAT hook (test_kronecker.jl semantics): A (ma x na) and B (mb x nb) dense column-major
// matrices, x of length na*nb; y = (A ⊗ B) x through the lazy evaluation.
void oracle_kron_apply(int ma, int na, const double* A, int mb, int nb, const double* B, const double* x, double* y) {
  auto dense_to_op = [](int m_, int n_, const double* D) {
    std::vector<std::vector<std::pair<int, double>>> rows(m_);
    for (int c = 0; c < n_; ++c)
      for (int r = 0; r < m_; ++r)
        if (D[r + (size_t)m_ * c] != 0.0) rows[r].push_back({c, D[r + (size_t)m_ * c]});
    return from_triplets(m_, n_, rows);
  };
  Kron k = kron(dense_to_op(ma, na, A), dense_to_op(mb, nb, B));
  k.apply(x, y);
}

}  // extern "C"
