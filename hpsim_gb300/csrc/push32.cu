// push32.cu -- element transfer maps on FP32 particle state.
//
// FP32 beams store x, x', y, y' as FP32 and the phase and kinetic energy as
// FP32 offsets from a synchronous particle: dphi = phi - phi_ref,
// dw = w - w_ref.  The synchronous particle (on axis, never kicked by space
// charge) is advanced on the host in FP64 through the same formulas the FP64
// kernels apply (simulation_kernel.cu), so absolute phases (hundreds of
// radians after a DTL) and energies never pass through FP32.  Each kernel
// moves a particle's offsets from the reference before the element to the
// reference after it; every phase and energy increment is written as a
// difference from the reference's increment in a form that keeps FP32
// relative precision (1/beta_i - 1/beta_ref from dinvb, cos(p + e) - cos(p)
// from half-angle products, transit-time factors re-expanded about the
// reference's beta).
#include <cmath>

#include "internal.h"
#include "reduce.cuh"

namespace hps {

namespace {

constexpr float F_TWOPI = 6.28318530717958647692f;

#define PARTICLES(b) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (b).n; i += gridDim.x * blockDim.x)

double beta_of(double w, double mass) {
  double gm1 = w / mass;
  return sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
}

// ---- drift (SimulatePartialDriftKernel, simulation_kernel.cu:86-118) ----
__global__ void k32_drift(DevBeam b, RefK r, float hf, float aper2, float c, uint32_t eid) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    const float x0 = b.fx[i], y0 = b.fy[i], xp = b.fxp[i], yp = b.fyp[i], dw = b.fw[i], ph = b.fphi[i];
    if (lo != 0u) continue;
    float x = fmaf(xp, hf, x0);
    float y = fmaf(yp, hf, y0);
    if (aper2 != 0.0f && x * x + y * y > aper2) { b.loss[i] = eid; continue; }
    b.fx[i] = x;
    b.fy[i] = y;
    float g, beta;
    float D = dinvb(dw, r, g, beta);
    b.fphi[i] = fmaf(c, D, ph);
  }
}

// ---- half quad (SimulateHalfQuadKernel, simulation_kernel.cu:142-218) ----
__global__ void k32_half_quad(DevBeam b, RefK r, float len, float aper2, float qg, float kcoef, float c,
                              uint32_t eid) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    float x = b.fx[i], y = b.fy[i], xp = b.fxp[i], yp = b.fyp[i];
    const float dw = b.fw[i], ph = b.fphi[i];
    if (lo != 0u) continue;
    if (qg == 0.0f) {
      x = x + xp * len * 0.5f;
      y = y + yp * len * 0.5f;
      b.fx[i] = x;
      b.fy[i] = y;
    } else {
      float g = fmaf(dw, r.minv, r.g);
      float bg = sqrtf(g * (g + 2.0f) * (1.0f + xp * xp + yp * yp));
      float k = sqrtf(kcoef / bg);  // kcoef = |qG| c / m
      float inv_k = 1.0f / k;
      float kds = len * 0.25f * k;
      float s, cc;
      sincosf(kds, &s, &cc);
      float sh = sinhf(kds), ch = coshf(kds);
      float sovk = s * inv_k, shovk = sh * inv_k, sk = s * k, shk = sh * k, xx, yy;
#pragma unroll
      for (int rep = 0; rep < 2; ++rep) {
        if (qg > 0.0f) {
          xx = cc * x + sovk * xp; xp = -sk * x + cc * xp; x = xx;
          yy = ch * y + shovk * yp; yp = shk * y + ch * yp; y = yy;
        } else {
          xx = ch * x + shovk * xp; xp = shk * x + ch * xp; x = xx;
          yy = cc * y + sovk * yp; yp = -sk * y + cc * yp; y = yy;
        }
      }
      b.fx[i] = x; b.fy[i] = y; b.fxp[i] = xp; b.fyp[i] = yp;
    }
    if (aper2 != 0.0f && x * x + y * y > aper2) { b.loss[i] = eid; continue; }
    float g, beta;
    float D = dinvb(dw, r, g, beta);
    b.fphi[i] = fmaf(c, D, ph);
  }
}

// ---- steerer (SimulateSteererKernel, simulation_kernel.cu:120-140) ----
__global__ void k32_steerer(DevBeam b, RefK r, float kh, float kv) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    const float dw = b.fw[i], xp = b.fxp[i], yp = b.fyp[i];
    if (lo != 0u) continue;
    float g = fmaf(dw, r.minv, r.g);
    float btgm = sqrtf(g * (g + 2.0f));
    if (kh != 0.0f) b.fxp[i] = xp + kh / btgm;  // kh = BL_h q c / m
    if (kv != 0.0f) b.fyp[i] = yp + kv / btgm;
  }
}

// ---- RF gap first half (simulation_kernel.cu:226-288) ----
// every branch advances phi by K / beta: DTL K = beta_in (pi clbl + dps) +
// pi dcell/lambda - pi q1/lambda, CCL K = betag (pi clbl + dps) (+ const),
// zero amplitude K = 2 pi dd1 / lambda.
__global__ void k32_gap_first(DevBeam b, RefK r, float dd1, float K) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    const float x = b.fx[i], y = b.fy[i], xp = b.fxp[i], yp = b.fyp[i], dw = b.fw[i], ph = b.fphi[i];
    if (lo != 0u) continue;
    b.fx[i] = fmaf(dd1, xp, x);
    b.fy[i] = fmaf(dd1, yp, y);
    float g, beta;
    float D = dinvb(dw, r, g, beta);
    b.fphi[i] = fmaf(K, D, ph);
  }
}

// ---- RF gap second half (simulation_kernel.cu:310-497) ----
struct Gap32 {
  RefK rin, rh;          // reference before the gap, reference after its (hypothetical) kick
  float dd2, drift_c;    // drift branch: phi += drift_c / beta
  float fbc, fbm, b0, tc[6], sc[6], inv2pifbc;  // T(beta), S(beta) as Taylor series about b0
  float beta_in, betag_ccl, gmg, q, efl, efl_m, concomm, concomm1, con1, con2nex, inv_gmg2, inv_gmgcl,
      inv_fkis, fkr, sinps, cosps, X, ccl_dg;
  float sinF, cosF, prome1_r, sinP, cosP, tw_r, prome_r, K2;
  float dphi_ref, dw_ref;  // actual reference change
  float corr_phi, corr_w;  // hypothetical minus actual reference after the gap
  int ccl, amp0, ref_drift;
};

__device__ inline float fbessi0c(float x, float *m1) {
  float ax = fabsf(x);
  if (ax < 3.75f) {
    float cy = x / 3.75f;
    cy = cy * cy;
    float s = cy * (3.5156229f + cy * (3.0899424f + cy * (1.2067492f + cy * (0.2659732f +
              cy * (0.360768e-1f + cy * 0.45813e-2f)))));
    *m1 = s;
    return 1.0f + s;
  }
  float cy = 3.75f / ax;
  float ans = (expf(ax) * rsqrtf(ax)) * (0.39894228f + cy * (0.1328592e-1f + cy * (0.225319e-2f +
              cy * (-0.157565e-2f + cy * (0.916281e-2f + cy * (-0.2057706e-1f + cy * (0.2635537e-1f +
              cy * (-0.1647633e-1f + cy * 0.392377e-2f))))))));
  *m1 = ans - 1.0f;
  return ans;
}
__device__ inline float fbessi1c(float x) {
  float ax = fabsf(x), ans;
  if (ax < 3.75f) {
    float cy = x / 3.75f;
    cy = cy * cy;
    ans = ax * (0.5f + cy * (0.87890594f + cy * (0.51498869f + cy * (0.15084934f + cy * (0.2658733e-1f +
          cy * (0.301532e-2f + cy * 0.32411e-3f))))));
  } else {
    float cy = 3.75f / ax;
    ans = 0.2282967e-1f + cy * (-0.2895312e-1f + cy * (0.1787654e-1f - cy * 0.420059e-2f));
    ans = 0.39894228f + cy * (-0.3988024e-1f + cy * (-0.362018e-2f + cy * (0.163801e-2f + cy *
          (-0.1031555e-1f + cy * ans))));
    ans = ans * (expf(ax) * rsqrtf(ax));
  }
  return x < 0.0f ? -ans : ans;
}

__global__ void __launch_bounds__(kBlock) k32_gap_second(DevBeam b, Gap32 G) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    float x = b.fx[i], y = b.fy[i], xp = b.fxp[i], yp = b.fyp[i], dphi = b.fphi[i], dw = b.fw[i];
    if (lo != 0u) continue;
    float g, beta;
    float D = dinvb(dw, G.rin, g, beta);
    float bg1 = sqrtf(g * (g + 2.0f));
    // GetTransitTimeFactors (simulation_kernel.cu:290-308) about the reference's beta
    float bcl = beta;
    if (beta > 1.1f * G.fbc) bcl = G.fbc;
    else if (beta < G.fbm) bcl = G.fbm;
    float u = bcl - G.b0;
    const float *tc = G.tc, *sc = G.sc;
    float dT = u * (tc[1] + u * (tc[2] + u * (tc[3] + u * (tc[4] + u * tc[5]))));
    float t = tc[0] + dT;
    float dTd = tc[1] + u * (2.0f * tc[2] + u * (3.0f * tc[3] + u * (4.0f * tc[4] + 5.0f * u * tc[5])));
    float dSd = sc[1] + u * (2.0f * sc[2] + u * (3.0f * sc[3] + u * (4.0f * sc[4] + 5.0f * u * sc[5])));
    float coef = bcl * bcl * G.inv2pifbc;
    float tp = coef * dTd, sp = -coef * dSd;
    if (G.amp0 || (G.ccl && beta < G.fbm)) {
      b.fx[i] = fmaf(G.dd2, xp, x);
      b.fy[i] = fmaf(G.dd2, yp, y);
      if (G.ref_drift) b.fphi[i] = fmaf(G.drift_c, D, dphi);
      else {
        b.fphi[i] = dphi + G.drift_c / beta - G.dphi_ref;
        b.fw[i] = dw - G.dw_ref;
      }
      continue;
    }
    float tw, dtw;
    if (G.ccl) {
      tw = t - F_TWOPI * tp * (G.beta_in / beta - 1.0f) * G.betag_ccl / G.beta_in;
      dtw = tw - G.tw_r;
    } else {
      tw = t;
      dtw = dT;
    }
    float con5nex = G.concomm * (t * G.inv_fkis - G.X * tp * G.inv_gmg2);
    float con5nex1 = G.concomm1 * t;
    float con5nex2 = -G.con2nex * t * G.inv_fkis;
    float delta = G.ccl ? dphi - G.ccl_dg * D : dphi;
    float sd, cd;
    sincosf(delta, &sd, &cd);
    float sinp1 = G.sinF * cd + G.cosF * sd, cosp1 = G.cosF * cd - G.sinF * sd;
    float prome1 = -G.con1 * (tp * (sinp1 - G.sinps) + sp * (cosp1 - G.cosps));
    float eps = delta + (prome1 - G.prome1_r);
    float se, ce;
    sincosf(eps, &se, &ce);
    float sinp = G.sinP * ce + G.cosP * se, cosp = G.cosP * ce - G.sinP * se;
    float sh = sinf(0.5f * eps);
    float dcos = -G.cosP * 2.0f * sh * sh - G.sinP * se;
    float rs_p = x * x + y * y, rrp = x * xp + y * yp;
    float ris = sqrtf(rs_p), fkrris = G.fkr * ris;
    float b0m1;
    float b0c = fbessi0c(fkrris, &b0m1);
    float b1c = fbessi1c(fkrris);
    float b1p = fkrris != 0.0f ? b0c - b1c / fkrris : 0.5f;
    float bes1covr = ris != 0.0f ? b1c / ris : G.fkr * 0.5f;
    float rest = ((tw - F_TWOPI * tp) / G.gmg * bes1covr + tw / G.gmg * G.fkr * b1p - tw * G.gmg * bes1covr) * rrp * sinp;
    float ddelte = G.q * G.efl * (tw * b0c * dcos + (dtw * b0c + G.tw_r * b0m1) * G.cosP + rest);
    float dwh = dw + ddelte;
    float gh, betah;
    float Dh = dinvb(dwh, G.rh, gh, betah);
    float bg = sqrtf(gh * (gh + 2.0f));
    float bgr = bg1 / bg;
    float onema = 1.0f - (con5nex * bes1covr + con5nex1 * b1p + con5nex2 * bes1covr) * cosp;
    float dovbl = G.con2nex * bes1covr * tw * sinp;
    float bgrovonema = bgr / onema;
    xp = -dovbl * x + bgrovonema * xp;
    x = x * onema + G.dd2 * xp;
    yp = -dovbl * y + bgrovonema * yp;
    y = y * onema + G.dd2 * yp;
    float rpris = rs_p > 0.0f ? rrp / ris : 0.0f;
    float prome = 2.0f * G.con1 * (-tp * b0c + ris * tw * b1c * G.inv_gmgcl) * (sinp - G.sinps) -
                  G.efl_m * tw * b1c * rpris * (cosp - G.cosps);
    float dphih = dphi + G.K2 * Dh + (prome - G.prome_r);
    float wabs = G.rh.w + dwh;
    if (wabs <= 0.0f || x != x || y != y || xp != xp || yp != yp || dwh != dwh || dphih != dphih) {
      b.loss[i] = 33333333u;
    } else {
      b.fx[i] = x; b.fy[i] = y; b.fxp[i] = xp; b.fyp[i] = yp;
      b.fphi[i] = dphih + G.corr_phi;
      b.fw[i] = dwh + G.corr_w;
    }
  }
}

// ---- buncher (SimulateBuncherKernel, simulation_kernel.cu:807-871) ----
struct Bun32 {
  RefK r;
  float hr, sinB, cosB, k2q, qV, con1, beta_w, aper2;
  uint32_t eid;
};
__global__ void k32_buncher(DevBeam b, Bun32 B) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    const float x = b.fx[i], y = b.fy[i], xp = b.fxp[i], yp = b.fyp[i], dw = b.fw[i], ph = b.fphi[i];
    if (lo != 0u) continue;
    float r2 = x * x + y * y;
    if (B.aper2 != 0.0f && r2 > B.aper2) { b.loss[i] = B.eid; continue; }
    float delta = B.hr * ph;
    float sd, cd;
    sincosf(delta, &sd, &cd);
    float cosph = B.cosB * cd - B.sinB * sd, sinph = B.sinB * cd + B.cosB * sd;
    float sh = sinf(0.5f * delta);
    float dcos = -B.cosB * 2.0f * sh * sh - B.sinB * sd;
    float arg = B.k2q * r2;
    float poly = arg * (1.0f + arg * (0.25f + arg / 36.0f));
    float dwi = B.qV * cosph * (1.0f + poly);
    float ddw = B.qV * (dcos + cosph * poly);
    float w = B.r.w + dw;
    float wb_par = w + 0.5f * dwi, wf = w + dwi;
    if (wb_par <= 0.0f || wf <= 0.0f) { b.loss[i] = B.eid; continue; }
    float gt = wb_par * B.r.minv;
    float bav = sqrtf(gt * (gt + 2.0f)) / (gt + 1.0f);
    gt = fmaf(dw, B.r.minv, B.r.g);
    float bg = sqrtf(gt * (gt + 2.0f));
    gt = wf * B.r.minv;
    float rbgf = rsqrtf(gt * (gt + 2.0f));
    float del = -B.con1 * sinph * (1.0f - bav * B.beta_w) * (0.5f + arg * (0.25f + arg / 24.0f)) / bav;
    b.fxp[i] = (xp * bg + del * x) * rbgf;
    b.fyp[i] = (yp * bg + del * y) * rbgf;
    b.fw[i] = dw + ddw;
  }
}

// ---- rotation, apertures (simulation_kernel.cu:511-575) ----
__global__ void k32_rotation(DevBeam b, float cosa, float sina) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    const float x = b.fx[i], y = b.fy[i], xp = b.fxp[i], yp = b.fyp[i];
    if (lo != 0u) continue;
    b.fx[i] = x * cosa + y * sina;
    b.fy[i] = y * cosa - x * sina;
    b.fxp[i] = xp * cosa + yp * sina;
    b.fyp[i] = yp * cosa - xp * sina;
  }
}
__global__ void k32_aperture(DevBeam b, int rect, float aper, float xl, float xr, float yt, float yb, uint32_t eid) {
  float cx = (float)b.st->st[X_AVG], cy = (float)b.st->st[Y_AVG];
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    const float x = b.fx[i], y = b.fy[i];
    if (i == 0 || lo != 0u) continue;
    if (!rect) {
      float dx = x - cx, dy = y - cy;
      if (dx * dx + dy * dy > aper * aper) b.loss[i] = eid;
    } else if (x < cx - xl || x > cx + xr || y < cy - yb || y > cy + yt) {
      b.loss[i] = eid;
    }
  }
}

// ---- dipole halves (simulation_kernel.cu:603-805) ----
struct Dip32 {
  float r11, r12, r16, r21, r22, r26, r33, r34, r43, r44, r51, r52, r56, e21, e43;
  float cdp, dpop_ref, cph;  // dpop_i = dpop_ref + cdp * dw; phase offset = cph * (...)
};
__global__ void k32_dipole(DevBeam b, Dip32 d, int second) {
  PARTICLES(b) {
    const uint32_t lo = b.loss[i];
    float x = b.fx[i], xp = b.fxp[i], y = b.fy[i], yp = b.fyp[i];
    const float dw = b.fw[i], ph = b.fphi[i];
    if (lo != 0u) continue;
    float ddp = d.cdp * dw;
    float dpop = d.dpop_ref + ddp;
    if (!second) {
      xp += d.e21 * x;
      yp -= d.e43 * y;
      b.fx[i] = d.r11 * x + d.r12 * xp + d.r16 * dpop;
      b.fxp[i] = d.r21 * x + d.r22 * xp + d.r26 * dpop;
      b.fy[i] = d.r33 * y + d.r34 * yp;
      b.fyp[i] = d.r43 * y + d.r44 * yp;
      b.fphi[i] = ph - d.cph * (d.r51 * x + d.r52 * xp + d.r56 * ddp);
    } else {
      b.fphi[i] = ph - d.cph * (d.r51 * x + d.r52 * xp + d.r56 * ddp);
      float xn = d.r11 * x + d.r12 * xp + d.r16 * dpop;
      xp = d.r21 * x + d.r22 * xp + d.r26 * dpop;
      float yn = d.r33 * y + d.r34 * yp;
      yp = d.r43 * y + d.r44 * yp;
      b.fx[i] = xn;
      b.fy[i] = yn;
      b.fxp[i] = xp + d.e21 * xn;
      b.fyp[i] = yp - d.e43 * yn;
    }
  }
}

// T(beta) = sum_k a_k beta^k re-expanded as sum_j c_j (beta - b0)^j
void taylor(const double *a, int na, double b0, double *c) {
  for (int j = 0; j < 6; ++j) {
    double s = 0.0, binom = 1.0;
    for (int k = j; k < na; ++k) {
      if (k > j) binom = binom * k / (k - j);
      s += binom * a[k] * pow(b0, k - j);
    }
    c[j] = s;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers: FP64 reference update on the host, FP32 kernel for the particles
// ---------------------------------------------------------------------------
void push32_partial_drift(DevBeam &b, double wl, double hf, double aper, uint32_t eid, cudaStream_t st) {
  RefK r = make_refk(b.w_ref, b.mass);
  k32_drift<<<grid_for(b.n), kBlock, 0, st>>>(b, r, (float)hf, (float)(aper * aper), (float)(TWOPI * hf / wl), eid);
  note_launch();
  b.phi_ref += TWOPI * hf / (wl * beta_of(b.w_ref, b.mass));
}

void push32_half_quad(DevBeam &b, double wl, double len, double aper, double grad, uint32_t eid, cudaStream_t st) {
  RefK r = make_refk(b.w_ref, b.mass);
  double qg = grad * b.charge;
  k32_half_quad<<<grid_for(b.n), kBlock, 0, st>>>(b, r, (float)len, (float)(aper * aper), (float)qg,
                                                  (float)(fabs(qg) * CLIGHT / b.mass), (float)(TWOPI * len * 0.5 / wl),
                                                  eid);
  note_launch();
  b.phi_ref += TWOPI * len * 0.5 / (wl * beta_of(b.w_ref, b.mass));
}

void push32_steerer(DevBeam &b, double blh, double blv, cudaStream_t st) {
  RefK r = make_refk(b.w_ref, b.mass);
  float kh = blh > 1e-10 ? (float)(blh * b.charge * CLIGHT / b.mass) : 0.0f;
  float kv = blv > 1e-10 ? (float)(blv * b.charge * CLIGHT / b.mass) : 0.0f;
  k32_steerer<<<grid_for(b.n), kBlock, 0, st>>>(b, r, kh, kv);
  note_launch();
}

void push32_gap_first(DevBeam &b, const GapArgs &g, cudaStream_t st) {
  RefK r = make_refk(b.w_ref, b.mass);
  double mass = b.mass;
  double wave_len = CLIGHT / g.frequency;
  double cell_len = g.length + g.q1 * 0.5 + g.q2 * 0.5;
  double dd1 = 0.5 * cell_len - g.dg - 0.5 * g.q1;
  double K, dphi_ref;
  double bref = beta_of(b.w_ref, mass);
  if (g.amplitude == 0.0) {
    K = TWOPI * dd1 / wave_len;
    dphi_ref = TWOPI * dd1 / (wave_len * bref);
  } else {
    double gam = g.design_w_in / mass;
    double beta_in = sqrt((gam + 2.0) * gam) / (gam + 1.0);
    gam = b.w_ref / mass;
    double beta = sqrt((gam + 2.0) * gam) / (gam + 1.0);
    double dps = g.phase_ref - g.phi_in;
    double A = PI * g.clbl + dps;
    if (!g.ccl) {
      double d_cell_len = cell_len - g.beta_center * wave_len;
      double dphi_qlen1 = TWOPI * 0.5 * g.q1 / (beta * wave_len);
      double dphi_clen = 0.0;
      bool dc = d_cell_len > 1e-15 || d_cell_len < -1e-15;
      if (dc) dphi_clen = PI * d_cell_len / (beta * wave_len);
      dphi_ref = (1.0 - (beta - beta_in) / beta) * A + dphi_clen - dphi_qlen1;
      K = beta_in * A + (dc ? PI * d_cell_len / wave_len : 0.0) - PI * g.q1 / wave_len;
    } else {
      double betag = cell_len / (g.clbl * wave_len);
      dphi_ref = (1.0 - (beta - beta_in) * betag / (beta * beta_in)) * A;
      K = betag * A;
    }
  }
  k32_gap_first<<<grid_for(b.n), kBlock, 0, st>>>(b, r, (float)dd1, (float)K);
  note_launch();
  b.phi_ref += dphi_ref;
}

void push32_gap_second(DevBeam &b, const GapArgs &g, cudaStream_t st) {
  const double mass = b.mass;
  Gap32 G{};
  G.rin = make_refk(b.w_ref, mass);
  double cell_len = g.length + g.q1 * 0.5 + g.q2 * 0.5;
  double dd2 = 0.5 * cell_len + g.dg - g.q2 * 0.5;
  G.dd2 = (float)dd2;
  G.drift_c = (float)(TWOPI * dd2 / g.wl);
  double inv_mass = 1.0 / mass;
  double gm_in = g.design_w_in * inv_mass + 1.0;
  double beta_in = sqrt(1.0 - 1.0 / (gm_in * gm_in));
  double gam = b.w_ref * inv_mass;
  double bg1 = sqrt(gam * (gam + 2.0));
  double beta = bg1 / (gam + 1.0);
  // transit-time factors of the reference, as in the FP64 kernel
  double bcl = beta;
  if (beta > 1.1 * g.fbc) bcl = g.fbc;
  else if (beta < g.fbm) bcl = g.fbm;
  const double *ta = g.ta, *sa = g.sa;
  double t_r = ta[0] + bcl * (ta[1] + bcl * (ta[2] + bcl * (ta[3] + bcl * (ta[4] + bcl * ta[5]))));
  double coef = bcl * bcl / (TWOPI * g.fbc);
  double tp_r = coef * (ta[1] + bcl * (2 * ta[2] + bcl * (3 * ta[3] + bcl * (4 * ta[4] + 5 * bcl * ta[5]))));
  double sp_r = -coef * (sa[0] + bcl * (2 * sa[1] + bcl * (3 * sa[2] + bcl * (4 * sa[3] + 5 * bcl * sa[4]))));
  double tcoef[6], scoef[6], sfull[6] = {0.0, sa[0], sa[1], sa[2], sa[3], sa[4]};
  taylor(ta, 6, bcl, tcoef);
  taylor(sfull, 6, bcl, scoef);
  for (int k = 0; k < 6; ++k) { G.tc[k] = (float)tcoef[k]; G.sc[k] = (float)scoef[k]; }
  G.tc[0] = (float)t_r;
  G.fbc = (float)g.fbc;
  G.fbm = (float)g.fbm;
  G.b0 = (float)bcl;
  G.inv2pifbc = (float)(1.0 / (TWOPI * g.fbc));
  G.ccl = g.ccl;
  G.amp0 = g.amplitude == 0.0;
  bool ref_drift = g.amplitude == 0.0 || (g.ccl && beta < g.fbm);
  G.ref_drift = ref_drift;
  double dphi_drift_ref = TWOPI * dd2 / (g.wl * beta);
  double phi_h, w_h;  // reference after a kick (hypothetical if it drifts)
  double wave_len = CLIGHT / g.frequency;
  if (g.amplitude != 0.0) {
    double cl = cell_len / g.clbl;
    double betag_ccl = cl / wave_len;
    double betag = g.ccl ? g.beta_center : betag_ccl;
    double betag2 = betag * betag;
    double gmg = 1.0 / sqrt(1.0 - betag2);
    double inv_gmg2 = 1.0 / (gmg * gmg);
    double q = fabs(b.charge);
    double gm_out = g.energy_out * inv_mass + 1.0;
    double beta_out = sqrt(1.0 - 1.0 / (gm_out * gm_out));
    double efl = g.amplitude * cell_len;
    double concomm = q * efl / (mass * betag2);
    double concomm1 = concomm * inv_gmg2 / gmg;
    double con1 = PI * concomm1;
    double con2nex = concomm * inv_gmg2;
    double tw, inv_fkis, inv_gmgcl, X;
    if (g.ccl) {
      inv_gmgcl = 1.0 / (gmg * betag * wave_len);
      inv_fkis = betag * wave_len / TWOPI;
      X = betag_ccl * wave_len;
      tw = t_r - TWOPI * tp_r * (beta_in / beta - 1.0) * betag_ccl / beta_in;
    } else {
      inv_gmgcl = 1.0 / (gmg * cl);
      inv_fkis = cl / TWOPI;
      X = beta_in * wave_len;
      tw = t_r;
    }
    double fkr = TWOPI * inv_gmgcl;
    double sinps = sin(g.phase_ref), cosps = cos(g.phase_ref);
    double phi1;
    if (g.ccl) phi1 = b.phi_ref + g.phase_shift - TWOPI * g.dg / (beta * wave_len) + g.ccl_cell_num * PI;
    else phi1 = b.phi_ref + g.phase_shift;
    double sinp1 = sin(phi1), cosp1 = cos(phi1);
    double prome1 = -con1 * (tp_r * (sinp1 - sinps) + sp_r * (cosp1 - cosps));
    double P = phi1 + prome1;
    double sinP = sin(P), cosP = cos(P);
    // on axis: b0c = 1, b1c = 0, b1p = 0.5, rrp = 0
    double delte = q * efl * (tw * cosP);
    w_h = b.w_ref + delte;
    double gh = w_h * inv_mass;
    double bgh = sqrt(gh * (gh + 2.0));
    double beta_h = bgh / (gh + 1.0);
    double prome = 2.0 * con1 * (-tp_r) * (sinP - sinps);
    double A = PI * g.clbl + (g.ccl ? (g.phi_in - g.phase_ref) : (g.phase_ref - g.phi_in));
    double K2;
    if (g.ccl) {
      phi_h = b.phi_ref + (1.0 - (beta_h - beta_out) * betag_ccl / (beta_h * beta_out)) * A + prome;
      K2 = betag_ccl * A;
    } else {
      double d_cell_len = cell_len - g.beta_center * wave_len;
      double dphi_qlen2 = TWOPI * 0.5 * g.q2 / (beta_h * wave_len);
      bool dc = d_cell_len > 1e-15 || d_cell_len < -1e-15;
      double dphi_clen = dc ? PI * d_cell_len / (beta_h * wave_len) : 0.0;
      phi_h = b.phi_ref + (1.0 - (beta_h - beta_out) / beta_h) * A + prome + dphi_clen - dphi_qlen2;
      K2 = beta_out * A + (dc ? PI * d_cell_len / wave_len : 0.0) - PI * g.q2 / wave_len;
    }
    G.beta_in = (float)beta_in; G.betag_ccl = (float)betag_ccl; G.gmg = (float)gmg; G.q = (float)q;
    G.efl = (float)efl; G.efl_m = (float)(efl * inv_mass); G.concomm = (float)concomm;
    G.concomm1 = (float)concomm1; G.con1 = (float)con1; G.con2nex = (float)con2nex;
    G.inv_gmg2 = (float)inv_gmg2; G.inv_gmgcl = (float)inv_gmgcl; G.inv_fkis = (float)inv_fkis;
    G.fkr = (float)fkr; G.sinps = (float)sinps; G.cosps = (float)cosps; G.X = (float)X;
    G.ccl_dg = (float)(TWOPI * g.dg / wave_len);
    double F = fmod(phi1, TWOPI), Pm = fmod(P, TWOPI);
    G.sinF = (float)sin(F); G.cosF = (float)cos(F);
    G.prome1_r = (float)prome1;
    G.sinP = (float)sin(Pm); G.cosP = (float)cos(Pm);
    G.tw_r = (float)tw;
    G.prome_r = (float)prome;
    G.K2 = (float)K2;
  } else {
    phi_h = b.phi_ref + dphi_drift_ref;
    w_h = b.w_ref;
  }
  G.rh = make_refk(w_h, mass);
  double phi_new = ref_drift ? b.phi_ref + dphi_drift_ref : phi_h;
  double w_new = ref_drift ? b.w_ref : w_h;
  G.dphi_ref = (float)(phi_new - b.phi_ref);
  G.dw_ref = (float)(w_new - b.w_ref);
  G.corr_phi = (float)(phi_h - phi_new);
  G.corr_w = (float)(w_h - w_new);
  k32_gap_second<<<grid_for(b.n), kBlock, 0, st>>>(b, G);
  note_launch();
  b.phi_ref = phi_new;
  b.w_ref = w_new;
}

void push32_buncher(DevBeam &b, double wl, double w_ref_design, double freq, double voltage, double phase,
                    double aper, double freq_ratio, uint32_t eid, cudaStream_t st) {
  double mass = b.mass;
  Bun32 B{};
  B.r = make_refk(b.w_ref, mass);
  double h = freq * wl / CLIGHT;
  double gm1 = w_ref_design / mass;
  double gm = gm1 + 1.0;
  double btgm = sqrt(gm1 * (gm1 + 2.0));
  double beta = btgm / gm;
  double k = h * TWOPI / (btgm * wl);
  double q = fabs(b.charge);
  double con1 = TWOPI * h * voltage * q / (beta * wl * mass);
  double ph = fmod(h * b.phi_ref * freq_ratio + phase, TWOPI);
  B.hr = (float)(h * freq_ratio);
  B.sinB = (float)sin(ph);
  B.cosB = (float)cos(ph);
  B.k2q = (float)(k * k * 0.25);
  B.qV = (float)(q * voltage);
  B.con1 = (float)con1;
  B.beta_w = (float)beta;
  B.aper2 = (float)(aper * aper);
  B.eid = eid;
  k32_buncher<<<grid_for(b.n), kBlock, 0, st>>>(b, B);
  note_launch();
  b.w_ref += q * voltage * cos(h * b.phi_ref * freq_ratio + phase);
}

void push32_rotation(DevBeam &b, double angle, cudaStream_t st) {
  k32_rotation<<<grid_for(b.n), kBlock, 0, st>>>(b, (float)cos(angle), (float)sin(angle));
  note_launch();
}

void push32_aperture(DevBeam &b, int rect, const double *p, uint32_t eid, cudaStream_t st) {
  k32_aperture<<<grid_for(b.n), kBlock, 0, st>>>(b, rect, (float)p[HPS_P_APERTURE], (float)p[HPS_P_APT_XL],
                                                 (float)p[HPS_P_APT_XR], (float)p[HPS_P_APT_YT], (float)p[HPS_P_APT_YB],
                                                 eid);
  note_launch();
}

void push32_dipole(DevBeam &b, const double *p, double wl, int second, cudaStream_t st) {
  double mass = b.mass;
  double h = 1.0 / p[HPS_P_DIP_RADIUS];
  double findx = p[HPS_P_DIP_FIELD_INDEX];
  double design_w = p[HPS_P_DIP_KINETIC_ENERGY];
  double h2 = h * h;
  double dl = 0.5 * p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE];
  double yk2 = findx * h2, yk = sqrt(fabs(yk2)), inv_yk = 1.0 / yk, ykl = yk * dl;
  double xk2 = h2 - yk2, inv_xk2 = 1.0 / xk2, xk = sqrt(fabs(xk2)), inv_xk = 1.0 / xk, xkl = xk * dl;
  double cxkl = 1.0, sxokx = dl;
  if (xk2 > 0.0) { cxkl = cos(xkl); sxokx = sin(xkl) * inv_xk; }
  else if (xk2 < 0.0) { cxkl = cosh(xkl); sxokx = sinh(xkl) * inv_xk; }
  double cykl = 1.0, syoky = dl;
  if (yk2 > 0.0) { cykl = cos(ykl); syoky = sin(ykl) * inv_yk; }
  else if (yk2 < 0.0) { cykl = cosh(ykl); syoky = sinh(ykl) * inv_yk; }
  double gamma = design_w / mass + 1.0;
  double beta2 = 1.0 - 1.0 / (gamma * gamma);
  double beta = sqrt(beta2);
  double r26 = h * sxokx, r16 = h * (1.0 - cxkl) * inv_xk2;
  double r56 = -h2 * (dl * beta2 - sxokx) * inv_xk2 + dl * (1.0 - h2 * inv_xk2) / (gamma * gamma);
  double bedge = second ? p[HPS_P_DIP_EDGE_OUT] : p[HPS_P_DIP_EDGE_IN];
  double c1 = 2.0 * p[HPS_P_DIP_HALF_GAP] * p[HPS_P_DIP_K1] * h;
  double sinb = sin(bedge), inv_cosb = 1.0 / cos(bedge);
  double psi = c1 * (1.0 + sinb * sinb) * inv_cosb * (1.0 - c1 * p[HPS_P_DIP_K2] * sinb * inv_cosb);
  double cdp = gamma / (design_w * (gamma + 1.0));
  double dpop_ref = cdp * (b.w_ref - design_w);
  Dip32 d;
  d.r11 = (float)cxkl; d.r12 = (float)sxokx; d.r16 = (float)r16; d.r21 = (float)(-xk2 * sxokx); d.r22 = (float)cxkl;
  d.r26 = (float)r26; d.r33 = (float)cykl; d.r34 = (float)syoky; d.r43 = (float)(-yk2 * syoky); d.r44 = (float)cykl;
  d.r51 = (float)(-r26); d.r52 = (float)(-r16); d.r56 = (float)r56;
  d.e21 = (float)(tan(bedge) * h); d.e43 = (float)(tan(bedge - psi) * h);
  d.cdp = (float)cdp; d.dpop_ref = (float)dpop_ref; d.cph = (float)(TWOPI / (beta * wl));
  k32_dipole<<<grid_for(b.n), kBlock, 0, st>>>(b, d, second);
  note_launch();
  b.phi_ref += TWOPI * (-(r56 * dpop_ref) + dl) / (beta * wl);
}

}  // namespace hps
