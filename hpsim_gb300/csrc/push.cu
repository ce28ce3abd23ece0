// push.cu -- element transfer maps on FP64 particle state.
//
// Each kernel restates one kernel of src/simulation/inc/simulation_kernel.cu
// with the same arithmetic in the same order, so that FP64 beams follow the
// reference to rounding.  Launches use a grid-stride loop sized from the
// particle count (not the reference's NextPow2 geometry); where the
// reference's geometry changes what is computed, the host reproduces it
// (invalid zero-thread launches are not issued).
#include "internal.h"
#include "reduce.cuh"

namespace hps {

void load_gap_args(const double *p, GapArgs *g) {
  g->length = p[HPS_P_LENGTH];
  g->frequency = p[HPS_P_RF_FREQ];
  g->clbl = p[HPS_P_RF_CLBL];
  g->amplitude = p[HPS_P_RF_AMP];
  g->phase_ref = p[HPS_P_RF_PHASE_REF];
  g->phase_shift = p[HPS_P_RF_PHASE_SHIFT];
  g->energy_out = p[HPS_P_RF_ENERGY_OUT];
  g->beta_center = p[HPS_P_RF_BETA_CENTER];
  g->dg = p[HPS_P_RF_DG];
  g->t = p[HPS_P_RF_T];
  g->tp = p[HPS_P_RF_TP];
  g->sp = p[HPS_P_RF_SP];
  g->fbc = p[HPS_P_RF_FIT_BETA_CENTER];
  g->fbm = p[HPS_P_RF_FIT_BETA_MIN];
  for (int k = 0; k < 6; ++k) g->ta[k] = p[HPS_P_RF_FIT_T0 + k];
  for (int k = 0; k < 5; ++k) g->sa[k] = p[HPS_P_RF_FIT_S1 + k];
}

namespace {

#define PARTICLES(b) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (b).n; i += gridDim.x * blockDim.x)

// SimulatePartialDriftKernel, simulation_kernel.cu:86-118
__global__ void k_partial_drift(DevBeam b, double wl, double hf, double aper, uint32_t eid) {
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double aper2 = aper * aper;
    double x = b.x[i], y = b.y[i];
    x += b.xp[i] * hf;
    y += b.yp[i] * hf;
    if (aper2 != 0.0 && x * x + y * y > aper2) b.loss[i] = eid;
    else {
      b.x[i] = x;
      b.y[i] = y;
      double gm1 = b.w[i] / b.mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b.phi[i] += TWOPI * hf / (wl * bt);
    }
  }
}

// SimulateSteererKernel, simulation_kernel.cu:120-140
__global__ void k_steerer(DevBeam b, double blh, double blv) {
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double gm1 = b.w[i] / b.mass;
    double btgm = sqrt(gm1 * (gm1 + 2.0));
    double p = btgm * b.mass / CLIGHT;
    if (blh > 1e-10) b.xp[i] += blh * b.charge / p;
    if (blv > 1e-10) b.yp[i] += blv * b.charge / p;
  }
}

// SimulateHalfQuadKernel, simulation_kernel.cu:142-218
__global__ void k_half_quad(DevBeam b, double wl, double len, double aper, double grad, uint32_t eid) {
  double aper2 = aper * aper;
  double qg = grad * b.charge;
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double x = b.x[i], y = b.y[i], xp = b.xp[i], yp = b.yp[i], w = b.w[i];
    if (qg == 0) {
      b.x[i] = x + xp * len * 0.5;
      b.y[i] = y + yp * len * 0.5;
    } else {
      double gamma1 = w / b.mass;
      double bg = sqrt(gamma1 * (gamma1 + 2.0) * (1.0 + xp * xp + yp * yp));
      double absqg = qg > 0.0 ? qg : -qg;
      double k = sqrt(absqg / (bg * b.mass) * CLIGHT);
      double inv_k = 1.0 / k;
      double kds = len * 0.25 * k;
      double s, c, sh = sinh(kds), ch = cosh(kds);
      sincos(kds, &s, &c);
      double xx, yy, sovk = s * inv_k, shovk = sh * inv_k, sk = s * k, shk = sh * k;
#pragma unroll
      for (int rep = 0; rep < 2; ++rep) {
        if (qg > 0.0) {
          xx = c * x + sovk * xp; xp = -sk * x + c * xp; x = xx;
          yy = ch * y + shovk * yp; yp = shk * y + ch * yp; y = yy;
        } else {
          xx = ch * x + shovk * xp; xp = shk * x + ch * xp; x = xx;
          yy = c * y + sovk * yp; yp = -sk * y + c * yp; y = yy;
        }
      }
      b.x[i] = x; b.y[i] = y; b.xp[i] = xp; b.yp[i] = yp;
    }
    if (aper2 != 0 && x * x + y * y > aper2) b.loss[i] = eid;
    else {
      double gm1 = w / b.mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b.phi[i] += TWOPI * len * 0.5 / (wl * bt);
    }
  }
}

// SimulateRFGapFirstHalfKernel, simulation_kernel.cu:226-288
__global__ void k_gap_first(DevBeam b, GapArgs g) {
  double wave_len = CLIGHT / g.frequency;
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double x = b.x[i], y = b.y[i], xp = b.xp[i], yp = b.yp[i], phi = b.phi[i], w = b.w[i];
    double cell_len = g.length + g.q1 * 0.5 + g.q2 * 0.5;
    double dd1 = 0.5 * cell_len - g.dg - 0.5 * g.q1;
    b.x[i] = x + dd1 * xp;
    b.y[i] = y + dd1 * yp;
    if (g.amplitude == 0.0) {
      double gm1 = w / b.mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b.phi[i] += TWOPI * dd1 / (wave_len * bt);
    } else {
      double gam = g.design_w_in / b.mass;
      double beta_in = sqrt((gam + 2.0) * gam) / (gam + 1.0);
      gam = w / b.mass;
      double beta = sqrt((gam + 2.0) * gam) / (gam + 1.0);
      if (!g.ccl) {
        double dps = g.phase_ref - g.phi_in;
        double d_cell_len = cell_len - g.beta_center * wave_len;
        double dphi_qlen1 = TWOPI * 0.5 * g.q1 / (beta * wave_len);
        double dphi_clen = 0.0;
        if (d_cell_len > 1e-15 || d_cell_len < -1e-15) dphi_clen = PI * d_cell_len / (beta * wave_len);
        b.phi[i] = phi + (1.0 - (beta - beta_in) / beta) * (PI * g.clbl + dps) + dphi_clen - dphi_qlen1;
      } else {
        double dps = g.phase_ref - g.phi_in;
        double betag = cell_len / (g.clbl * wave_len);
        b.phi[i] = phi + (1.0 - (beta - beta_in) * betag / (beta * beta_in)) * (PI * g.clbl + dps);
      }
    }
  }
}

// Bessi0c / Bessi1c / Bessi1p, simulation_kernel.cu:15-73
__device__ inline double bessi0c(double r_x) {
  double ans, cy, ax = fabs(r_x);
  if (ax < 3.75) {
    cy = r_x / 3.75;
    cy = cy * cy;
    ans = 1.0 + cy * (3.5156229 + cy * (3.0899424 + cy * (1.2067492 + cy * (0.2659732 +
          cy * (0.360768e-1 + cy * 0.45813e-2)))));
  } else {
    cy = 3.75 / ax;
    ans = (exp(ax) * rsqrt(ax)) * (0.39894228 + cy * (0.1328592e-1 + cy * (0.225319e-2 +
          cy * (-0.157565e-2 + cy * (0.916281e-2 + cy * (-0.2057706e-1 + cy * (0.2635537e-1 +
          cy * (-0.1647633e-1 + cy * 0.392377e-2))))))));
  }
  return ans;
}
__device__ inline double bessi1c(double r_x) {
  double cy, ans, ax = fabs(r_x);
  if (ax < 3.75) {
    cy = r_x / 3.75;
    cy = cy * cy;
    ans = ax * (0.5 + cy * (0.87890594 + cy * (0.51498869 + cy * (0.15084934 + cy * (0.2658733e-1 +
          cy * (0.301532e-2 + cy * 0.32411e-3))))));
  } else {
    cy = 3.75 / ax;
    ans = 0.2282967e-1 + cy * (-0.2895312e-1 + cy * (0.1787654e-1 - cy * 0.420059e-2));
    ans = 0.39894228 + cy * (-0.3988024e-1 + cy * (-0.362018e-2 + cy * (0.163801e-2 + cy *
          (-0.1031555e-1 + cy * ans))));
    ans = ans * (exp(ax) * rsqrt(ax));
  }
  return r_x < 0.0 ? -ans : ans;
}
__device__ inline double bessi1p(double r_x) {
  if (r_x != 0.0) return bessi0c(r_x) - bessi1c(r_x) / r_x;
  return 0.5;
}

// GetTransitTimeFactors, simulation_kernel.cu:290-308
__device__ inline void ttf(const GapArgs &g, double r_beta, double *t, double *tp, double *sp) {
  double beta = r_beta;
  if (r_beta > 1.1 * g.fbc) beta = g.fbc;
  else if (r_beta < g.fbm) beta = g.fbm;
  const double *ta = g.ta, *sa = g.sa;
  *t = ta[0] + beta * (ta[1] + beta * (ta[2] + beta * (ta[3] + beta * (ta[4] + beta * ta[5]))));
  double coef = beta * beta / (TWOPI * g.fbc);
  *tp = coef * (ta[1] + beta * (2 * ta[2] + beta * (3 * ta[3] + beta * (4 * ta[4] + 5 * beta * ta[5]))));
  *sp = -coef * (sa[0] + beta * (2 * sa[1] + beta * (3 * sa[2] + beta * (4 * sa[3] + 5 * beta * sa[4]))));
}

// SimulateRFGapSecondHalfKernel, simulation_kernel.cu:310-497
__global__ void k_gap_second(DevBeam b, GapArgs g) {
  const double mass = b.mass;
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double cell_len = g.length + g.q1 * 0.5 + g.q2 * 0.5;
    double dd2 = 0.5 * cell_len + g.dg - g.q2 * 0.5;
    double x = b.x[i], y = b.y[i], xp = b.xp[i], yp = b.yp[i];
    double inv_mass = 1.0 / mass;
    double phi = b.phi[i], w = b.w[i];
    double gm_in = g.design_w_in * inv_mass + 1.0;
    double beta_in = sqrt(1.0 - 1.0 / (gm_in * gm_in));
    double gam = w * inv_mass;
    double bg1 = sqrt(gam * (gam + 2.0));
    double beta = bg1 / (gam + 1.0);
    double t_fac, tp_fac, sp_fac;
    ttf(g, beta, &t_fac, &tp_fac, &sp_fac);
    if (g.amplitude == 0.0 || (g.ccl && beta < g.fbm)) {
      b.x[i] = x + dd2 * xp;
      b.y[i] = y + dd2 * yp;
      double gm1 = w / mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b.phi[i] += TWOPI * dd2 / (g.wl * bt);
      continue;
    }
    double wave_len = CLIGHT / g.frequency;
    double cl = cell_len / g.clbl;
    double betag_ccl = cl / wave_len;
    double betag = g.ccl ? g.beta_center : betag_ccl;
    double betag2 = betag * betag;
    double gmg = 1.0 / sqrt(1.0 - betag2);
    double inv_gmg2 = 1.0 / (gmg * gmg);
    double q = b.charge;
    q = q > 0.0 ? q : -q;
    double gm_out = g.energy_out * inv_mass + 1.0;
    double beta_out = sqrt(1.0 - 1.0 / (gm_out * gm_out));
    double efl = g.amplitude * cell_len;
    double concomm = q * efl / (mass * betag2);
    double concomm1 = concomm * inv_gmg2 / gmg;
    double con1 = PI * concomm1;
    double con2nex = concomm * inv_gmg2;
    double con5nex, tw, inv_fkis, inv_gmgcl;
    if (g.ccl) {
      inv_gmgcl = 1.0 / (gmg * betag * wave_len);
      inv_fkis = betag * wave_len / TWOPI;
      con5nex = concomm * (t_fac * inv_fkis - betag_ccl * wave_len * tp_fac * inv_gmg2);
      tw = t_fac - TWOPI * tp_fac * (beta_in / beta - 1.0) * betag_ccl / beta_in;
    } else {
      inv_gmgcl = 1.0 / (gmg * cl);
      inv_fkis = cl / TWOPI;
      con5nex = concomm * (t_fac * inv_fkis - beta_in * wave_len * tp_fac * inv_gmg2);
      tw = t_fac;
    }
    double con5nex1 = concomm1 * t_fac;
    double con5nex2 = -con2nex * t_fac * inv_fkis;
    double fkr = TWOPI * inv_gmgcl;
    double sinps, cosps;
    sincos(g.phase_ref, &sinps, &cosps);
    double phi1, sinp1, cosp1;
    if (g.ccl) phi1 = phi + g.phase_shift - TWOPI * g.dg / (beta * wave_len) + g.ccl_cell_num * PI;
    else phi1 = phi + g.phase_shift;
    sincos(phi1, &sinp1, &cosp1);
    double prome1 = -con1 * (tp_fac * (sinp1 - sinps) + sp_fac * (cosp1 - cosps));
    sincos(phi1 + prome1, &sinp1, &cosp1);
    double rs_p = x * x + y * y;
    double rrp = x * xp + y * yp;
    double rpris = 0.0, bes1covr;
    double ris = sqrt(rs_p);
    double fkrris = fkr * ris;
    double b0c = bessi0c(fkrris);
    double b1c = bessi1c(fkrris);
    double b1p = bessi1p(fkrris);
    if (ris != 0.0) bes1covr = b1c / ris;
    else bes1covr = fkr * 0.5;
    double delte = q * efl * (tw * b0c * cosp1 + ((tw - TWOPI * tp_fac) / gmg * bes1covr +
                   tw / gmg * fkr * b1p - tw * gmg * bes1covr) * rrp * sinp1);
    w += delte;
    gam = w * inv_mass;
    double bg = sqrt(gam * (gam + 2.0));
    beta = bg / (gam + 1.0);
    double bgr = bg1 / bg;
    double onema = 1.0 - (con5nex * bes1covr + con5nex1 * b1p + con5nex2 * bes1covr) * cosp1;
    double dovbl = con2nex * bes1covr * tw * sinp1;
    double bgrovonema = bgr / onema;
    xp = -dovbl * x + bgrovonema * xp;
    x = x * onema + dd2 * xp;
    yp = -dovbl * y + bgrovonema * yp;
    y = y * onema + dd2 * yp;
    if (rs_p > 0.0) rpris = rrp / ris;
    double prome = 2.0 * con1 * (-tp_fac * b0c + ris * tw * b1c * inv_gmgcl) * (sinp1 - sinps) -
                   efl * inv_mass * tw * b1c * rpris * (cosp1 - cosps);
    double phi_new;
    if (g.ccl) {
      double dps = g.phi_in - g.phase_ref;
      phi_new = phi + (1.0 - (beta - beta_out) * betag_ccl / (beta * beta_out)) * (PI * g.clbl + dps) + prome;
    } else {
      double d_cell_len = cell_len - g.beta_center * wave_len;
      double dphi_qlen2 = TWOPI * 0.5 * g.q2 / (beta * wave_len);
      double dphi_clen = 0.0;
      if (d_cell_len > 1e-15 || d_cell_len < -1e-15) dphi_clen = PI * d_cell_len / (beta * wave_len);
      double dps = g.phase_ref - g.phi_in;
      phi_new = phi + (1.0 - (beta - beta_out) / beta) * (PI * g.clbl + dps) + prome + dphi_clen - dphi_qlen2;
    }
    if (w <= 0.0 || x != x || y != y || xp != xp || yp != yp || w != w || phi_new != phi_new) {
      b.loss[i] = 33333333u;
    } else {
      b.x[i] = x; b.y[i] = y; b.xp[i] = xp; b.yp[i] = yp; b.w[i] = w; b.phi[i] = phi_new;
    }
  }
}

// SimulateBuncherKernel, simulation_kernel.cu:807-871
__global__ void k_buncher(DevBeam b, double wl, double w_ref, double freq, double voltage, double phase,
                          double aper, double freq_ratio, uint32_t eid) {
  const double mass = b.mass;
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double x = b.x[i], y = b.y[i], xp = b.xp[i], yp = b.yp[i];
    double phi = b.phi[i] * freq_ratio;
    double w = b.w[i];
    double r2 = x * x + y * y;
    double aper2 = aper * aper;
    if (aper2 != 0.0 && r2 > aper2) { b.loss[i] = eid; continue; }
    double h = freq * wl / CLIGHT;
    double gm1 = w_ref / mass;
    double gm = gm1 + 1.0;
    double btgm = sqrt(gm1 * (gm1 + 2.0));
    double beta = btgm / gm;
    double k = h * TWOPI / (btgm * wl);
    double k2 = k * k;
    double q = b.charge;
    q = q > 0.0 ? q : -q;
    double con1 = TWOPI * h * voltage * q / (beta * wl * mass);
    double arg = k2 * r2 * 0.25;
    double ph = h * phi + phase;
    double dw = q * voltage * cos(ph) * (1.0 + arg * (1.0 + arg * (0.25 + arg / 36.0)));
    double wb_par = w + 0.5 * dw;
    double wf = w + dw;
    if (wb_par <= 0.0 || wf <= 0.0) { b.loss[i] = eid; continue; }
    double gmtmp = wb_par / mass;
    double bav = sqrt(gmtmp * (gmtmp + 2.0)) / (gmtmp + 1.0);
    gmtmp = w / mass;
    double bg = sqrt(gmtmp * (gmtmp + 2.0));
    gmtmp = wf / mass;
    double rbgf = rsqrt(gmtmp * (gmtmp + 2.0));
    double del = -con1 * sin(ph) * (1.0 - bav * beta) * (0.5 + arg * (0.25 + arg / 24.0)) / bav;
    b.xp[i] = (xp * bg + del * x) * rbgf;
    b.yp[i] = (yp * bg + del * y) * rbgf;
    b.w[i] = wf;
  }
}

// SimulateRotationKernel, simulation_kernel.cu:511-529
__global__ void k_rotation(DevBeam b, double cosa, double sina) {
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double x = b.x[i], y = b.y[i], xp = b.xp[i], yp = b.yp[i];
    b.x[i] = x * cosa + y * sina;
    b.y[i] = y * cosa - x * sina;
    b.xp[i] = xp * cosa + yp * sina;
    b.yp[i] = yp * cosa - xp * sina;
  }
}

// Simulate{Circular,Rectangular}ApertureKernel, simulation_kernel.cu:543-575;
// the centroid is the x_avg / y_avg left by UpdateAvgXY (index 0 skipped)
__global__ void k_aperture(DevBeam b, int rect, double aper, double xl, double xr, double yt, double yb,
                           uint32_t eid) {
  double cx = b.st->st[X_AVG], cy = b.st->st[Y_AVG];
  PARTICLES(b) {
    if (i == 0 || b.loss[i] != 0u) continue;
    if (!rect) {
      double aper2 = aper * aper;
      double x = b.x[i] - cx, y = b.y[i] - cy;
      if (x * x + y * y > aper2) b.loss[i] = eid;
    } else {
      double xmin = cx - xl, xmax = cx + xr, ymin = cy - yb, ymax = cy + yt;
      double x = b.x[i], y = b.y[i];
      if (x < xmin || x > xmax || y < ymin || y > ymax) b.loss[i] = eid;
    }
  }
}

// Simulate{First,Second}HalfDipoleKernel, simulation_kernel.cu:603-805
struct DipoleMap {
  double r11, r12, r16, r21, r22, r26, r33, r34, r43, r44, r51, r52, r56, beta, dl, design_w, gamma,
      e21, e43;
};

__global__ void k_dipole(DevBeam b, DipoleMap d, double wl, int second) {
  PARTICLES(b) {
    if (b.loss[i] != 0u) continue;
    double x = b.x[i], xp = b.xp[i], y = b.y[i], yp = b.yp[i];
    double dpop = d.gamma / (d.design_w * (d.gamma + 1.0)) * (b.w[i] - d.design_w);
    if (!second) {
      xp += d.e21 * x;
      yp -= d.e43 * y;
      b.x[i] = d.r11 * x + d.r12 * xp + d.r16 * dpop;
      b.xp[i] = d.r21 * x + d.r22 * xp + d.r26 * dpop;
      b.y[i] = d.r33 * y + d.r34 * yp;
      b.yp[i] = d.r43 * y + d.r44 * yp;
      b.phi[i] += TWOPI * (-(d.r51 * x + d.r52 * xp + d.r56 * dpop) + d.dl) / (d.beta * wl);
    } else {
      b.phi[i] += TWOPI * (-(d.r51 * x + d.r52 * xp + d.r56 * dpop) + d.dl) / (d.beta * wl);
      double x_new = d.r11 * x + d.r12 * xp + d.r16 * dpop;
      xp = d.r21 * x + d.r22 * xp + d.r26 * dpop;
      double y_new = d.r33 * y + d.r34 * yp;
      yp = d.r43 * y + d.r44 * yp;
      b.x[i] = x_new;
      b.y[i] = y_new;
      b.xp[i] = xp + d.e21 * x_new;
      b.yp[i] = yp - d.e43 * y_new;
    }
  }
}

// The particle-independent part of the dipole kernels, evaluated once on the
// host with the same operations (simulation_kernel.cu:620-693, 722-783).
DipoleMap dipole_map(const double *p, double mass, int second) {
  DipoleMap m;
  double h = 1.0 / p[HPS_P_DIP_RADIUS];
  double findx = p[HPS_P_DIP_FIELD_INDEX];
  m.design_w = p[HPS_P_DIP_KINETIC_ENERGY];
  double h2 = h * h;
  m.dl = 0.5 * p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE];
  double yk2 = findx * h2;
  double yk = sqrt(fabs(yk2));
  double inv_yk = 1.0 / yk;
  double ykl = yk * m.dl;
  double xk2 = h2 - yk2;
  double inv_xk2 = 1.0 / xk2;
  double xk = sqrt(fabs(xk2));
  double inv_xk = 1.0 / xk;
  double xkl = xk * m.dl;
  double cxkl = 1.0, sxokx = m.dl;
  if (xk2 > 0.0) { cxkl = cos(xkl); sxokx = sin(xkl) * inv_xk; }
  else if (xk2 < 0.0) { cxkl = cosh(xkl); sxokx = sinh(xkl) * inv_xk; }
  double cykl = 1.0, syoky = m.dl;
  if (yk2 > 0.0) { cykl = cos(ykl); syoky = sin(ykl) * inv_yk; }
  else if (yk2 < 0.0) { cykl = cosh(ykl); syoky = sinh(ykl) * inv_yk; }
  m.r11 = cxkl; m.r12 = sxokx; m.r21 = -xk2 * sxokx; m.r22 = cxkl;
  m.r33 = cykl; m.r34 = syoky; m.r43 = -yk2 * syoky; m.r44 = cykl;
  m.r26 = h * sxokx;
  m.r16 = h * (1.0 - cxkl) * inv_xk2;
  m.r51 = -m.r26;
  m.r52 = -m.r16;
  m.gamma = m.design_w / mass + 1.0;
  double beta2 = 1.0 - 1.0 / (m.gamma * m.gamma);
  m.beta = sqrt(beta2);
  m.r56 = -h2 * (m.dl * beta2 - sxokx) * inv_xk2 + m.dl * (1.0 - h2 * inv_xk2) / (m.gamma * m.gamma);
  double bedge = second ? p[HPS_P_DIP_EDGE_OUT] : p[HPS_P_DIP_EDGE_IN];
  double c1 = 2.0 * p[HPS_P_DIP_HALF_GAP] * p[HPS_P_DIP_K1] * h;
  double sinb = sin(bedge), inv_cosb = 1.0 / cos(bedge);
  double psi = c1 * (1.0 + sinb * sinb) * inv_cosb * (1.0 - c1 * p[HPS_P_DIP_K2] * sinb * inv_cosb);
  m.e21 = tan(bedge) * h;
  m.e43 = tan(bedge - psi) * h;
  return m;
}

}  // namespace

void push_partial_drift(const DevBeam &b, double wl, double hf, double aper, uint32_t eid, cudaStream_t st) {
  k_partial_drift<<<grid_for(b.n), kBlock, 0, st>>>(b, wl, hf, aper, eid); note_launch();
}
void push_half_quad(const DevBeam &b, double wl, double len, double aper, double grad, uint32_t eid,
                    cudaStream_t st) {
  k_half_quad<<<grid_for(b.n), kBlock, 0, st>>>(b, wl, len, aper, grad, eid); note_launch();
}
void push_steerer(const DevBeam &b, double blh, double blv, cudaStream_t st) {
  k_steerer<<<grid_for(b.n), kBlock, 0, st>>>(b, blh, blv); note_launch();
}
void push_gap_first(const DevBeam &b, const GapArgs &g, cudaStream_t st) {
  k_gap_first<<<grid_for(b.n), kBlock, 0, st>>>(b, g); note_launch();
}
void push_gap_second(const DevBeam &b, const GapArgs &g, cudaStream_t st) {
  k_gap_second<<<grid_for(b.n), kBlock, 0, st>>>(b, g); note_launch();
}
void push_buncher(const DevBeam &b, double wl, double w_ref, double freq, double voltage, double phase,
                  double aper, double freq_ratio, uint32_t eid, cudaStream_t st) {
  k_buncher<<<grid_for(b.n), kBlock, 0, st>>>(b, wl, w_ref, freq, voltage, phase, aper, freq_ratio, eid);
  note_launch();
}
void push_rotation(const DevBeam &b, double angle, cudaStream_t st) {
  k_rotation<<<grid_for(b.n), kBlock, 0, st>>>(b, cos(angle), sin(angle)); note_launch();
}
void push_aperture(const DevBeam &b, int rect, const double *p, uint32_t eid, cudaStream_t st) {
  k_aperture<<<grid_for(b.n), kBlock, 0, st>>>(b, rect, p[HPS_P_APERTURE], p[HPS_P_APT_XL], p[HPS_P_APT_XR],
                                                p[HPS_P_APT_YT], p[HPS_P_APT_YB], eid);
  note_launch();
}
void push_dipole(const DevBeam &b, const double *p, double wl, int second, cudaStream_t st) {
  k_dipole<<<grid_for(b.n), kBlock, 0, st>>>(b, dipole_map(p, b.mass, second), wl, second); note_launch();
}

}  // namespace hps
