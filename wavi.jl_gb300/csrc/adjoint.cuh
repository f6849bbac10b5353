// adjoint.cuh — tangent-linear and adjoint of the Picard-converged velocity solve (FP64).
//
// At convergence the solve's state satisfies, besides A(coef) x = b (update_velocities.jl:11-29), the
// per-cell fixed points the Picard loop iterates to (update_velocities.jl:227-339):
//   F2 = Σ_k w_k h ζ_k² / η_k,   u_b = S / (1 + F2 β),
//   g_β = β − Cg (u_b² + u_r²)^((1/m − 1)/2) = 0,
//   g_k = η_k − ½ B_k (ε² + ¼ (β u_b ζ_k / η_k)² + ε_r²)^((1/n − 1)/2) = 0,     k = 1..nσ,
// with ε² the shelf strain rate squared and S the depth-averaged speed (both functions of the velocity),
// Cg = C·grounded fraction (update_state.jl:129-134) and B_k ∝ A^(−1/n) (utilities.jl:462-466).  The
// operator's coefficients are ηav = Σ w_k η_k (→ hη_h, hη_c) and βeff = β / (1 + F2 β) (→ β on the u, v
// grids).  Differentiating these equations exactly gives, per cell, the 2 x 4 sensitivity L of
// (ηav, βeff) to (ε², S, log C, log A) (k_adj_local).  With F(x; θ) = A(coef(x, θ)) x − b:
//   J_F v  = A v + A(δcoef(v)) x                      (k_tlm_cell, k_tlm_uv, then the operator)
//   J_Fᵀ w = A w + (∂coef/∂x)ᵀ G(w, x)                (k_adj_cell, k_adj_uv)
// where G(w, x) = ∂(wᵀ A(coef) x)/∂coef:  −2[(2u_x + v_y) w_x + (2v_y + u_x) w_y] per h cell for hη_h,
// −(u_y + v_x)(w_y + w_x) per c point for hη_c, −x w per u/v point for β (summation by parts of
// op_fun!, utilities.jl:61-145; the dimp term does not depend on x or θ).  The gradient of J with
// respect to θ = (log C, log A) is −λᵀ A(∂coef/∂θ) x with J_Fᵀ λ = ∂J/∂x.
#pragma once
#include "fused.cuh"

namespace wavi {

constexpr int ADJ_NSMAX = 16;  // σ levels the local solve supports

// Per-cell state of the converged solution the adjoint linearises about (struct of arrays, Nh each).
struct AdjCell {
  double *ux, *vy, *sh, *uc, *vc, *S;  // strain components, shear (c -> h average), centred velocities, speed
  double* L;                           // 8 per cell: d(ηav, βeff)/d(ε², S, log C, log A), row-major
};

struct AdjIn {
  const double* uv;        // converged velocities (full layout)
  const uint8_t* mask;     // u | v masks
  const uint8_t* h_mask;
  const uint8_t* c_mask;
  const double* eta;       // Nh x nσ
  const double* beta;
  const double* quad_f2;
  const double* wc;        // C · grounded fraction
  const double* glen_b;    // Nh x nσ
  const double* h;
  const double* zeta;
  const double* qw;
  const DevParams* P;
};

// Per cell: the state's strain components and speed, and L (Gaussian elimination with partial pivoting
// on the (nσ+1) x (nσ+1) Jacobian of (g_1..g_nσ, g_β) in (η, β), four right-hand sides).
static __global__ void k_adj_local(Dims d, AdjIn in, AdjCell out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const int i = c % d.nx, j = c / d.nx;
  const bool hm = in.h_mask[c];
  auto um = [&](int a, int b) { const int q = uidx(d, a, b); return in.mask[q] ? in.uv[q] : 0.0; };
  auto vm = [&](int a, int b) { const int q = vidx(d, a, b); return in.mask[q] ? in.uv[q] : 0.0; };
  const double u0 = um(i, j), u1 = um(i + 1, j), v0 = vm(i, j), v1 = vm(i, j + 1);
  const double ux = hm ? (u1 * d.rdx - u0 * d.rdx) : 0.0;
  const double vy = hm ? (v1 * d.rdy - v0 * d.rdy) : 0.0;
  double sh = 0.0;
  if (hm) {
    for (int tb = 0; tb < 2; ++tb)
      for (int ta = 0; ta < 2; ++ta) {
        const int ca = i - 1 + ta, cb = j - 1 + tb;
        if (ca < 0 || ca >= d.nx - 1 || cb < 0 || cb >= d.ny - 1 || !in.c_mask[cidx(d, ca, cb)]) continue;
        sh += 0.25 * ((um(ca + 1, cb + 1) - um(ca + 1, cb)) * d.rdy + (vm(ca + 1, cb + 1) - vm(ca, cb + 1)) * d.rdx);
      }
  }
  const double uc = hm ? 0.5 * (u0 + u1) : 0.0, vc = hm ? 0.5 * (v0 + v1) : 0.0;
  const double S = sqrt(uc * uc + vc * vc);
  out.ux[c] = ux;
  out.vy[c] = vy;
  out.sh[c] = sh;
  out.uc[c] = uc;
  out.vc[c] = vc;
  out.S[c] = S;
  double* L = out.L + 8 * (size_t)c;
  for (int k = 0; k < 8; ++k) L[k] = 0.0;
  const int ns = d.ns;
  if (!hm || ns > ADJ_NSMAX) return;
  const double e2 = ux * ux + vy * vy + ux * vy + 0.25 * (sh * sh);
  const double p = 1.0 / in.P->weertman_m - 1.0, q = 1.0 / in.P->glen_n - 1.0, n = in.P->glen_n;
  const double ur = in.P->weertman_reg_speed, er = in.P->glen_reg_strain_rate;
  const double beta = in.beta[c], F2 = in.quad_f2[c], Cg = in.wc[c], hh = in.h[c];
  const double D = 1.0 + F2 * beta, ub = S / D, Pb = ub * ub + ur * ur, tau = beta * ub;
  const int nb = ns + 1, ib = ns;
  double M[ADJ_NSMAX + 1][ADJ_NSMAX + 1], N[ADJ_NSMAX + 1][4];
  for (int r = 0; r < nb; ++r) {
    for (int s = 0; s < nb; ++s) M[r][s] = 0.0;
    for (int s = 0; s < 4; ++s) N[r][s] = 0.0;
  }
  double dF2[ADJ_NSMAX], dub[ADJ_NSMAX];
  for (int k = 0; k < ns; ++k) {
    const double e = in.eta[c + (size_t)d.Nh * k];
    dF2[k] = -in.qw[k] * hh * in.zeta[k] * in.zeta[k] / (e * e);
    dub[k] = -S * beta * dF2[k] / (D * D);
  }
  const double dub_db = -S * F2 / (D * D), dub_dS = 1.0 / D;
  // g_β
  const double cp = Cg * p * pow(Pb, 0.5 * p - 1.0) * ub;
  M[ib][ib] = 1.0 - cp * dub_db;
  for (int k = 0; k < ns; ++k) M[ib][k] = -cp * dub[k];
  N[ib][1] = -cp * dub_dS;
  N[ib][2] = -Cg * pow(Pb, 0.5 * p);
  // g_k
  const double dt_db = ub + beta * dub_db, dt_dS = beta * dub_dS;
  for (int k = 0; k < ns; ++k) {
    const size_t qk = c + (size_t)d.Nh * k;
    const double e = in.eta[qk], B = in.glen_b[qk], z = in.zeta[k];
    const double Q = e2 + 0.25 * (tau * z / e) * (tau * z / e) + er * er;
    const double H = 0.5 * B * pow(Q, 0.5 * q);
    const double hq = 0.5 * B * (0.5 * q) * pow(Q, 0.5 * q - 1.0);
    const double dQ_dt = 0.5 * tau * z * z / (e * e), dQ_de = -0.5 * tau * tau * z * z / (e * e * e);
    for (int jj = 0; jj < ns; ++jj) M[k][jj] = (jj == k ? 1.0 : 0.0) - hq * (dQ_dt * beta * dub[jj] + (jj == k ? dQ_de : 0.0));
    M[k][ib] = -hq * dQ_dt * dt_db;
    N[k][0] = -hq;
    N[k][1] = -hq * dQ_dt * dt_dS;
    N[k][3] = H / n;
  }
  // solve M Y = -N
  for (int col = 0; col < nb; ++col) {
    int piv = col;
    for (int r = col + 1; r < nb; ++r)
      if (fabs(M[r][col]) > fabs(M[piv][col])) piv = r;
    if (piv != col) {
      for (int s = 0; s < nb; ++s) {
        const double t = M[col][s];
        M[col][s] = M[piv][s];
        M[piv][s] = t;
      }
      for (int s = 0; s < 4; ++s) {
        const double t = N[col][s];
        N[col][s] = N[piv][s];
        N[piv][s] = t;
      }
    }
    const double dg = M[col][col];
    if (dg == 0.0) return;  // singular local system: no sensitivity
    for (int r = col + 1; r < nb; ++r) {
      const double f = M[r][col] / dg;
      if (f == 0.0) continue;
      for (int s = col; s < nb; ++s) M[r][s] -= f * M[col][s];
      for (int s = 0; s < 4; ++s) N[r][s] -= f * N[col][s];
    }
  }
  double Y[ADJ_NSMAX + 1][4];
  for (int r = nb - 1; r >= 0; --r)
    for (int s = 0; s < 4; ++s) {
      double v = -N[r][s];
      for (int t = r + 1; t < nb; ++t) v -= M[r][t] * Y[t][s];
      Y[r][s] = v / M[r][r];
    }
  // (ηav, βeff) rows
  for (int s = 0; s < 4; ++s) {
    double de = 0.0, db = Y[ib][s] / (D * D);
    for (int k = 0; k < ns; ++k) {
      de += in.qw[k] * Y[k][s];
      db += -beta * beta * dF2[k] / (D * D) * Y[k][s];
    }
    L[s] = de;
    L[4 + s] = db;
  }
}

// Weights of β on the u/v grid: beta_m(q) = Σ_n ω_n βeff(n) over the two h neighbours of q
// (k_relin_uv: valid-neighbour average, grounded-fraction rescaling).
struct BetaWeights {
  double w0, w1;
};
__device__ __forceinline__ BetaWeights beta_weights(const Dims& d, const uint8_t* mask, const uint8_t* h_mask,
                                                    const double* gf, const double* gf_uv, int q, int a0, int b0,
                                                    int a1, int b1) {
  BetaWeights r{0.0, 0.0};
  if (!mask[q]) return r;
  auto hmk = [&](int a, int b) { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny && h_mask[hidx(d, a, b)]) ? 1.0 : 0.0; };
  auto hv = [&](const double* f, int a, int b) {
    return (a >= 0 && a < d.nx && b >= 0 && b < d.ny && h_mask[hidx(d, a, b)]) ? f[hidx(d, a, b)] : 0.0;
  };
  const double den = 0.5 * hmk(a0, b0) + 0.5 * hmk(a1, b1);
  if (den == 0.0) return r;
  double s = 1.0;
  const double ip = (0.5 * hv(gf, a0, b0) + 0.5 * hv(gf, a1, b1)) / den;
  if (ip > 0.0) s = gf_uv[q] / ip;
  r.w0 = 0.5 * hmk(a0, b0) / den * s;
  r.w1 = 0.5 * hmk(a1, b1) / den * s;
  return r;
}

struct AdjUV {
  const uint8_t* mask;    // u | v
  const uint8_t* h_mask;
  const uint8_t* c_mask;
  const double* gf;
  const double* gf_uv;
  const double* h;
};

// Tangent linear, per cell: δ(ηav, βeff) from an interior velocity perturbation dx (zero off the
// interior) and optional parameter perturbations dlogC, dlogA; writes δhη_h and the per-cell
// δ(h ηav), δβeff for k_tlm_uv.
static __global__ void k_tlm_cell(Dims d, AdjCell st, AdjUV m, const double* __restrict__ dx,
                                  const double* __restrict__ dlogC, const double* __restrict__ dlogA,
                                  double* __restrict__ dheta_h, double* __restrict__ dhn, double* __restrict__ dbeff) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const int i = c % d.nx, j = c / d.nx;
  const bool hm = m.h_mask[c];
  double de = 0.0, db = 0.0;
  if (hm) {
    double e2 = 0.0, dS = 0.0;
    if (dx) {
      auto du = [&](int a, int b) { return dx[uidx(d, a, b)]; };
      auto dv = [&](int a, int b) { return dx[vidx(d, a, b)]; };
      const double dux = (du(i + 1, j) - du(i, j)) * d.rdx, dvy = (dv(i, j + 1) - dv(i, j)) * d.rdy;
      double dsh = 0.0;
      for (int tb = 0; tb < 2; ++tb)
        for (int ta = 0; ta < 2; ++ta) {
          const int ca = i - 1 + ta, cb = j - 1 + tb;
          if (ca < 0 || ca >= d.nx - 1 || cb < 0 || cb >= d.ny - 1 || !m.c_mask[cidx(d, ca, cb)]) continue;
          dsh += 0.25 * ((du(ca + 1, cb + 1) - du(ca + 1, cb)) * d.rdy + (dv(ca + 1, cb + 1) - dv(ca, cb + 1)) * d.rdx);
        }
      const double ux = st.ux[c], vy = st.vy[c], sh = st.sh[c], S = st.S[c];
      e2 = (2.0 * ux + vy) * dux + (2.0 * vy + ux) * dvy + 0.5 * sh * dsh;
      if (S > 0.0)
        dS = (st.uc[c] * 0.5 * (du(i, j) + du(i + 1, j)) + st.vc[c] * 0.5 * (dv(i, j) + dv(i, j + 1))) / S;
    }
    const double* L = st.L + 8 * (size_t)c;
    const double gc = dlogC ? dlogC[c] : 0.0, ga = dlogA ? dlogA[c] : 0.0;
    de = L[0] * e2 + L[1] * dS + L[2] * gc + L[3] * ga;
    db = L[4] * e2 + L[5] * dS + L[6] * gc + L[7] * ga;
  }
  dheta_h[c] = hm ? m.h[c] * de : 0.0;
  dhn[c] = m.h[c] * de;
  dbeff[c] = db;
}

// Tangent linear on the u/v/c grids: δβ_m and δhη_c from the per-cell perturbations.
static __global__ void k_tlm_uv(Dims d, AdjUV m, const double* __restrict__ dhn, const double* __restrict__ dbeff,
                                double* __restrict__ dbeta_m, double* __restrict__ dheta_c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  auto bv = [&](int a, int b) { return (a >= 0 && a < d.nx && b >= 0 && b < d.ny) ? dbeff[hidx(d, a, b)] : 0.0; };
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    const BetaWeights w = beta_weights(d, m.mask, m.h_mask, m.gf, m.gf_uv, q, i - 1, j, i, j);
    dbeta_m[q] = w.w0 * bv(i - 1, j) + w.w1 * bv(i, j);
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    const BetaWeights w = beta_weights(d, m.mask, m.h_mask, m.gf, m.gf_uv, q, i, j - 1, i, j);
    dbeta_m[q] = w.w0 * bv(i, j - 1) + w.w1 * bv(i, j);
  }
  if (i < d.nx - 1 && j < d.ny - 1) {
    const int q = cidx(d, i, j);
    double v = 0.0;
    if (m.c_mask[q]) {
      const double a = 0.5 * dhn[hidx(d, i, j)] + 0.5 * dhn[hidx(d, i, j + 1)];
      const double b = 0.5 * dhn[hidx(d, i + 1, j)] + 0.5 * dhn[hidx(d, i + 1, j + 1)];
      v = 0.5 * a + 0.5 * b;
    }
    dheta_c[q] = v;
  }
}

// Adjoint, per cell: G(w, x) gathered onto (ηav, βeff), then through Lᵀ: the cell's adjoint strain
// source ē² and speed source S̄ (for k_adj_uv) and, when grad_c/grad_a are given, the parameter
// gradients −(ḡ_ηav, ḡ_βeff)·L[:, log C | log A].
static __global__ void k_adj_cell(Dims d, AdjCell st, AdjUV m, const uint8_t* __restrict__ inner,
                                  const double* __restrict__ x, const double* __restrict__ w, double* __restrict__ ebar,
                                  double* __restrict__ sbar, double* __restrict__ grad_c, double* __restrict__ grad_a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const int i = c % d.nx, j = c / d.nx;
  double ge = 0.0, gb = 0.0;
  // G(w, x) for hη_h (this cell) and hη_c (its up-to-four corners), with the operator's differences
  auto xu = [&](const double* f, int a, int b) { return f[uidx(d, a, b)]; };
  auto xv = [&](const double* f, int a, int b) { return f[vidx(d, a, b)]; };
  {
    const double ux = (xu(x, i + 1, j) - xu(x, i, j)) * d.rdx, vy = (xv(x, i, j + 1) - xv(x, i, j)) * d.rdy;
    const double wx = (xu(w, i + 1, j) - xu(w, i, j)) * d.rdx, wy = (xv(w, i, j + 1) - xv(w, i, j)) * d.rdy;
    const double ghh = -2.0 * ((2.0 * ux + vy) * wx + (2.0 * vy + ux) * wy);
    if (m.h_mask[c]) ge += m.h[c] * ghh;
    double gc = 0.0;
    for (int tb = 0; tb < 2; ++tb)
      for (int ta = 0; ta < 2; ++ta) {
        const int ca = i - 1 + ta, cb = j - 1 + tb;
        if (ca < 0 || ca >= d.nx - 1 || cb < 0 || cb >= d.ny - 1 || !m.c_mask[cidx(d, ca, cb)]) continue;
        const double sx = (xu(x, ca + 1, cb + 1) - xu(x, ca + 1, cb)) * d.rdy + (xv(x, ca + 1, cb + 1) - xv(x, ca, cb + 1)) * d.rdx;
        const double sw = (xu(w, ca + 1, cb + 1) - xu(w, ca + 1, cb)) * d.rdy + (xv(w, ca + 1, cb + 1) - xv(w, ca, cb + 1)) * d.rdx;
        gc += 0.25 * (-sx * sw);
      }
    ge += m.h[c] * gc;
  }
  // G for β at the four u/v points this cell feeds (−x w, interior points only)
  {
    auto gbq = [&](int q) { return inner[q] ? -x[q] * w[q] : 0.0; };
    int q = uidx(d, i, j);  // cell is the high neighbour of u(i, j)
    gb += beta_weights(d, m.mask, m.h_mask, m.gf, m.gf_uv, q, i - 1, j, i, j).w1 * gbq(q);
    q = uidx(d, i + 1, j);  // ... and the low neighbour of u(i+1, j)
    gb += beta_weights(d, m.mask, m.h_mask, m.gf, m.gf_uv, q, i, j, i + 1, j).w0 * gbq(q);
    q = vidx(d, i, j);
    gb += beta_weights(d, m.mask, m.h_mask, m.gf, m.gf_uv, q, i, j - 1, i, j).w1 * gbq(q);
    q = vidx(d, i, j + 1);
    gb += beta_weights(d, m.mask, m.h_mask, m.gf, m.gf_uv, q, i, j, i, j + 1).w0 * gbq(q);
  }
  const double* L = st.L + 8 * (size_t)c;
  if (ebar) ebar[c] = L[0] * ge + L[4] * gb;
  if (sbar) sbar[c] = L[1] * ge + L[5] * gb;
  if (grad_c) grad_c[c] = -(L[2] * ge + L[6] * gb);
  if (grad_a) grad_a[c] = -(L[3] * ge + L[7] * gb);
}

// Adjoint on the u/v grid: out = (∂(ε², S)/∂x)ᵀ (ē², S̄) at the interior points (zero elsewhere),
// added to `base` (A w) when given.
static __global__ void k_adj_uv(Dims d, AdjCell st, AdjUV m, const uint8_t* __restrict__ inner,
                                const double* __restrict__ ebar, const double* __restrict__ sbar,
                                const double* __restrict__ base, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  auto cellok = [&](int a, int b) { return a >= 0 && a < d.nx && b >= 0 && b < d.ny && m.h_mask[hidx(d, a, b)]; };
  // shear source at c point (ca, cb): c_mask · ¼ Σ over its cells of ½ sh ē²
  auto cbar = [&](int ca, int cb) -> double {
    if (ca < 0 || ca >= d.nx - 1 || cb < 0 || cb >= d.ny - 1 || !m.c_mask[cidx(d, ca, cb)]) return 0.0;
    double s = 0.0;
    for (int tb = 0; tb < 2; ++tb)
      for (int ta = 0; ta < 2; ++ta) {
        const int a = ca + ta, b = cb + tb;
        if (cellok(a, b)) {
          const int h = hidx(d, a, b);
          s += 0.25 * 0.5 * st.sh[h] * ebar[h];
        }
      }
    return s;
  };
  auto speed_term = [&](int a, int b, bool isu) -> double {
    if (!cellok(a, b)) return 0.0;
    const int h = hidx(d, a, b);
    const double S = st.S[h];
    if (!(S > 0.0)) return 0.0;
    return 0.5 * (isu ? st.uc[h] : st.vc[h]) / S * sbar[h];
  };
  if (i <= d.nx && j < d.ny) {
    const int q = uidx(d, i, j);
    double g = 0.0;
    if (inner[q]) {
      // ux of cell (i-1, j) (+1/dx) and of cell (i, j) (-1/dx)
      if (cellok(i - 1, j)) {
        const int h = hidx(d, i - 1, j);
        g += (2.0 * st.ux[h] + st.vy[h]) * ebar[h] * d.rdx;
      }
      if (cellok(i, j)) {
        const int h = hidx(d, i, j);
        g -= (2.0 * st.ux[h] + st.vy[h]) * ebar[h] * d.rdx;
      }
      // u_y at c(i-1, j-1) (+1/dy) and c(i-1, j) (-1/dy)
      g += (cbar(i - 1, j - 1) - cbar(i - 1, j)) * d.rdy;
      g += speed_term(i - 1, j, true) + speed_term(i, j, true);
      if (base) g += base[q];
    }
    out[q] = g;
  }
  if (i < d.nx && j <= d.ny) {
    const int q = vidx(d, i, j);
    double g = 0.0;
    if (inner[q]) {
      if (cellok(i, j - 1)) {
        const int h = hidx(d, i, j - 1);
        g += (2.0 * st.vy[h] + st.ux[h]) * ebar[h] * d.rdy;
      }
      if (cellok(i, j)) {
        const int h = hidx(d, i, j);
        g -= (2.0 * st.vy[h] + st.ux[h]) * ebar[h] * d.rdy;
      }
      // v_x at c(i-1, j-1) (+1/dx) and c(i, j-1) (-1/dx)
      g += (cbar(i - 1, j - 1) - cbar(i, j - 1)) * d.rdx;
      g += speed_term(i, j - 1, false) + speed_term(i, j, false);
      if (base) g += base[q];
    }
    out[q] = g;
  }
}

// y = inner ⊙ (a + b) (the two halves of J_F v).
static __global__ void k_add_inner(int n, const uint8_t* __restrict__ inner, const double* __restrict__ a,
                                   const double* __restrict__ b, double* __restrict__ y) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    y[k] = inner[k] ? a[k] + b[k] : 0.0;
}

// y = inner ⊙ y
static __global__ void k_mask_inner(int n, const uint8_t* __restrict__ inner, double* __restrict__ y) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    if (!inner[k]) y[k] = 0.0;
}

// Deterministic dot product: per-block partials, the last block adds them in block order.
static __global__ void k_dot(int n, const double* __restrict__ a, const double* __restrict__ b,
                             double* __restrict__ partials, unsigned* counter, double* __restrict__ out) {
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) s += a[k] * b[k];
  double tot[2];
  if (last_block_sum2(s, 0.0, partials, counter, tot))
    if (flat_tid() == 0) *out = tot[0];
}

// y = a·x + b·y for a list of scalars read from device memory: y += Σ_k coef[k] x_k (FGMRES updates).
static __global__ void k_axpy(int n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) y[k] += alpha * x[k];
}
static __global__ void k_scale(int n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) y[k] = alpha * x[k];
}

// Batched Gram-Schmidt pieces of FGMRES (classical Gram-Schmidt twice: two passes h = Vᵀw, w -= V h, the
// Hessenberg column the sum of both), so that an Arnoldi step needs one host round trip instead of one per
// basis vector.  Dot products: grid (blocks, m), block (bx, j) sums V[j]·w over its chunk into
// partials[j * gridDim.x + bx]; k_sum_rows then adds each row in block order (deterministic).
static __global__ void __launch_bounds__(256) k_multi_dot(int n, const double* const* __restrict__ V,
                                                          const double* __restrict__ w, double* __restrict__ partials) {
  __shared__ double sh[32];
  const int j = blockIdx.y;
  const double* __restrict__ v = V[j];
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) s += v[k] * w[k];
  s = block_sum_any(s, sh);
  if (threadIdx.x == 0) partials[(size_t)j * gridDim.x + blockIdx.x] = s;
}
// out[j] (+)= Σ_b partials[j * nb + b] for j < m, one warp per row; accumulate: add to out (the second pass)
static __global__ void k_sum_rows(const double* __restrict__ partials, int nb, int m, double* __restrict__ out,
                                  int accumulate) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = wid; j < m; j += nw) {
    double s = 0.0;
    for (int b = lane; b < nb; b += 32) s += partials[(size_t)j * nb + b];
    s = warp_sum(s);
    if (lane == 0) out[j] = accumulate ? out[j] + s : s;
  }
}
// w -= Σ_{j<m} h[j] V[j], h read from device memory
static __global__ void __launch_bounds__(256) k_multi_axpy(int n, const double* const* __restrict__ V, int m,
                                                           const double* __restrict__ h, double* __restrict__ w) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double s = w[k];
    for (int j = 0; j < m; ++j) s -= h[j] * V[j][k];
    w[k] = s;
  }
}

}  // namespace wavi
