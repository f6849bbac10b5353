// timestep.cuh — the update_state! steps around the velocity solve and update_thickness!, on the device,
// so that a time-stepping run keeps the model in HBM between steps (update_state.jl:7-193,
// run_simulation.jl:6-42).  Every kernel reads and writes the context's own solve buffers.
#pragma once
#include "fused.cuh"

namespace wavi {

struct StepBuf {
  const double* b;          // bed elevation (Nh)
  const double* c_param;    // Weertman C before the grounded-fraction factor (Nh)
  const double* acc_param;  // accumulation rate (Nh)
  const uint8_t* h_isfixed; // (Nh)
  double melt_rate;         // uniform basal melt rate (UniformMeltRate)
  double* haf;              // height above floatation (Nh)
  double* afq;              // 4 x Nh quarter-cell grounded fractions of pos_fraction
  double* dhdt;             // (Nh)
  double *uh, *vh, *ub, *vb, *us, *vs;  // velocities on the h grid (Nh each)
};

struct StepState {
  const uint8_t* h_mask;
  const uint8_t* mask;      // u | v
  double* h;
  double* s;
  double* dsdh;
  double* gf;
  double* wc;
  double* acc;
  double* melt;
  double* h_uv;             // u | v
  double* s_uv;             // u | v
  double* gf_uv;            // u | v
  const DevParams* P;
};

// update_surface_elevation! (:51-57), update_height_above_floatation! (:80-85, utilities.jl:445),
// update_accumulation_rate! (:106-111), update_basal_melt! (UniformMeltRate, MeltRate.jl:37-54).
static __global__ void k_step_pre_h(Dims d, StepState s, StepBuf b) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const double ri = s.P->rho_i, rw = s.P->rho_w, sl = s.P->sea_level;
  const double h = s.h[c], bed = b.b[c];
  if (s.h_mask[c]) s.s[c] = fmax(bed + h, sl + h * (1 - ri / rw));
  b.haf[c] = h - (rw / ri) * (sl - bed);
  s.acc[c] = b.acc_param[c];
  s.melt[c] = b.melt_rate;
}

// Thickness and surface on the u/v grids at the mask points (update_geometry_on_uv_grids!, :65-73):
// the valid-neighbour average of the two adjacent h cells; other points keep their previous values.
static __global__ void k_step_geom_uv(Dims d, StepState s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  auto hv = [&](const double* f, int a, int bb) {
    return (a >= 0 && a < d.nx && bb >= 0 && bb < d.ny && s.h_mask[hidx(d, a, bb)]) ? f[hidx(d, a, bb)] : 0.0;
  };
  auto hm = [&](int a, int bb) { return (a >= 0 && a < d.nx && bb >= 0 && bb < d.ny && s.h_mask[hidx(d, a, bb)]) ? 1.0 : 0.0; };
  auto point = [&](int q, int a0, int b0, int a1, int b1) {
    if (!s.mask[q]) return;
    const double den = 0.5 * hm(a0, b0) + 0.5 * hm(a1, b1);
    s.h_uv[q] = (0.5 * hv(s.h, a0, b0) + 0.5 * hv(s.h, a1, b1)) / den;
    s.s_uv[q] = (0.5 * hv(s.s, a0, b0) + 0.5 * hv(s.s, a1, b1)) / den;
  };
  if (i <= d.nx && j < d.ny) point(uidx(d, i, j), i - 1, j, i, j);
  if (i < d.nx && j <= d.ny) point(vidx(d, i, j), i, j - 1, i, j);
}

// pos_fraction (utilities.jl:255-396), first half: the grounded fraction of each quarter q = 1..4 of
// every h cell from the height above floatation at the cell and two neighbours (sub-grid linear
// interpolation of the zero contour), written to afq[q-1][cell].
static __global__ void k_step_pos_quarters(Dims d, const uint8_t* __restrict__ mask, const double* __restrict__ z1,
                                           double* __restrict__ afq) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const int M = d.nx, N = d.ny, i = c % M, j = c / M;
  auto at = [&](int a, int bb) { return a + M * bb; };
  auto sgn = [](double x) { return (double)((x > 0) - (x < 0)); };
  const int ip = min(i + 1, M - 1), im = max(i - 1, 0), jp = min(j + 1, N - 1), jm = max(j - 1, 0);
  for (int q = 1; q <= 4; ++q) {
    int i2, j2, i3, j3;
    if (q == 1) { i2 = ip; j2 = j; i3 = i; j3 = jp; }
    else if (q == 2) { i2 = i; j2 = jp; i3 = im; j3 = j; }
    else if (q == 3) { i2 = im; j2 = j; i3 = i; j3 = jm; }
    else { i2 = i; j2 = jm; i3 = ip; j3 = j; }
    const double z = z1[c];
    const double z2 = mask[at(i2, j2)] ? z1[at(i2, j2)] : z;
    const double z3 = mask[at(i3, j3)] ? z1[at(i3, j3)] : z;
    double val = 0.0;
    if (!((sgn(z) == sgn(z2)) && (sgn(z) == sgn(z3)))) {
      const bool flip = fabs(z3 - z) < fabs(z2 - z);
      double a, bb;
      if (!flip) {
        a = -(z2 - z) / (z3 - z);
        bb = -2 * z / (z3 - z);
      } else {
        a = -(z3 - z) / (z2 - z);
        bb = -2 * z / (z2 - z);
      }
      const double A1 = 0.5 * (bb * bb) / a, A2 = 0.5 * ((1.0 - bb) * (1.0 - bb)) / a, A3 = 0.5 * a + bb;
      const int t1 = (bb > 0.0) + (bb > 1.0), t2 = ((a + bb) > 0.0) + ((a + bb) > 1.0);
      double ar;
      switch (1 + t1 + 3 * t2) {
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
    if (!mask[c]) val = 0.0;
    afq[(size_t)(q - 1) * d.Nh + c] = val;
  }
}

// pos_fraction, second half, gathered (summation in the order q = 1..4, as the reference accumulates):
// the cell fraction is the mean of its quarters; a u (v) point takes the quarters of the two adjacent
// cells that touch it.  Then update_grounded_fraction_on_huv_grids! (:92-99), update_weertman_c!
// (:129-134) and update_dsdh! (:141-147).
static __global__ void k_step_pos_gather(Dims d, StepState s, const double* __restrict__ afq,
                                         const double* __restrict__ c_param) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  const int M = d.nx, N = d.ny;
  auto A = [&](int q, int a, int bb) -> double {
    return (a >= 0 && a < M && bb >= 0 && bb < N) ? afq[(size_t)(q - 1) * d.Nh + a + M * bb] : 0.0;
  };
  if (i < M && j < N) {
    const int c = hidx(d, i, j);
    double af = 0.0;
    af = af + 0.25 * A(1, i, j);
    af = af + 0.25 * A(2, i, j);
    af = af + 0.25 * A(3, i, j);
    af = af + 0.25 * A(4, i, j);
    s.gf[c] = af;
    s.wc[c] = c_param[c] * af;
    const double r = s.P->rho_i / s.P->rho_w;
    s.dsdh[c] = (1.0 - r) + r * af;
  }
  if (i <= M && j < N) {  // u point (i, j): quarters 1, 4 of cell (i-1, j), quarters 2, 3 of cell (i, j)
    double a = 0.0;
    a = a + 0.25 * A(1, i - 1, j);
    a = a + 0.25 * A(2, i, j);
    a = a + 0.25 * A(3, i, j);
    a = a + 0.25 * A(4, i - 1, j);
    s.gf_uv[uidx(d, i, j)] = a;
  }
  if (i < M && j <= N) {  // v point (i, j): quarters 1, 2 of cell (i, j-1), quarters 3, 4 of cell (i, j)
    double a = 0.0;
    a = a + 0.25 * A(1, i, j - 1);
    a = a + 0.25 * A(2, i, j - 1);
    a = a + 0.25 * A(3, i, j);
    a = a + 0.25 * A(4, i, j);
    s.gf_uv[vidx(d, i, j)] = a;
  }
}

// update_velocities_on_h_grid! (:164-178) and update_dhdt! (:184-189).
static __global__ void k_step_post_h(Dims d, StepState s, StepBuf b, const double* __restrict__ uv,
                                     const double* __restrict__ beta, const double* __restrict__ f1,
                                     const double* __restrict__ f2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  const int i = c % d.nx, j = c / d.nx;
  const double uh = 0.5 * uv[uidx(d, i, j)] + 0.5 * uv[uidx(d, i + 1, j)];
  const double vh = 0.5 * uv[vidx(d, i, j)] + 0.5 * uv[vidx(d, i, j + 1)];
  const double ub = uh / (1 + (beta[c] * f2[c])), vb = vh / (1 + (beta[c] * f2[c]));
  b.uh[c] = uh;
  b.vh[c] = vh;
  b.ub[c] = ub;
  b.vb[c] = vb;
  b.us[c] = ub * (1 + (beta[c] * f1[c]));
  b.vs[c] = vb * (1 + (beta[c] * f1[c]));
  if (s.h_mask[c]) {
    auto qx = [&](int a) { const int q = uidx(d, a, j); return s.mask[q] ? s.h_uv[q] * uv[q] : 0.0; };
    auto qy = [&](int bb) { const int q = vidx(d, i, bb); return s.mask[q] ? s.h_uv[q] * uv[q] : 0.0; };
    const double dq = (qx(i + 1) * d.rdx - qx(i) * d.rdx) + (qy(j + 1) * d.rdy - qy(j) * d.rdy);
    b.dhdt[c] = s.acc[c] - s.melt[c] - dq;
  }
}

// update_wavelets! (Wavelets/update_wavelets.jl:6-32) after the forward transform: the coarse space is
// where |wavelet coefficient| >= threshold, and the coarse-correction cache starts again from zero.
static __global__ void k_step_wavelet_mask(int n, const double* __restrict__ wav, double thr, uint8_t* __restrict__ wmask,
                                           double* __restrict__ xc_full) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    wmask[k] = fabs(wav[k]) >= thr ? 1 : 0;
    xc_full[k] = 0.0;
  }
}

// update_thickness! with evolve_shelves (run_simulation.jl:24-42): h += max(h_min - h, dt dh/dt) on the
// ice mask, except at h_isfixed cells.
static __global__ void k_step_thickness(Dims d, StepState s, StepBuf b, double dt, double h_min) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Nh) return;
  if (!s.h_mask[c]) return;
  double hup = fmax(h_min - s.h[c], dt * b.dhdt[c]);
  if (b.h_isfixed[c]) hup = 0.0;
  s.h[c] = s.h[c] + hup;
}

}  // namespace wavi
