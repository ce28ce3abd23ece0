// push32_maps.cuh -- element transfer maps on FP32 particle state, as device
// functors.  A map's apply() takes one live particle (in registers) and
// returns the set of fields it changed, so one kernel template serves every
// element and the same map can run alone, followed by a reduction of the
// new state, or after the space-charge kick (push32.cu).
//
// Particle state: x, x', y, y' in FP32; phi and W as FP32 offsets from the
// synchronous particle, which the host advances in FP64.  Every phase and
// energy increment is formed as a difference from the synchronous
// particle's increment: 1/beta_i - 1/beta_ref from dinvb, cos(p + e) - cos(p)
// from half-angle products, transit-time factors re-expanded about the
// reference's beta.
#pragma once

#include "common.cuh"

namespace hps {

struct Part {
  uint32_t lo;                  // loss flag
  float x, xp, y, yp, ph, w;    // ph, w: offsets from the synchronous particle
};

enum : uint32_t { WR_X = 1, WR_XP = 2, WR_Y = 4, WR_YP = 8, WR_PH = 16, WR_W = 32, WR_LOSS = 64 };

__device__ inline Part load_part(const DevBeam &b, uint32_t i) {
  return {b.loss[i], b.fx[i], b.fxp[i], b.fy[i], b.fyp[i], b.fphi[i], b.fw[i]};
}
__device__ inline void store_part(const DevBeam &b, uint32_t i, const Part &p, uint32_t m) {
  if (m & WR_X) b.fx[i] = p.x;
  if (m & WR_XP) b.fxp[i] = p.xp;
  if (m & WR_Y) b.fy[i] = p.y;
  if (m & WR_YP) b.fyp[i] = p.yp;
  if (m & WR_PH) b.fphi[i] = p.ph;
  if (m & WR_W) b.fw[i] = p.w;
  if (m & WR_LOSS) b.loss[i] = p.lo;
}

constexpr float F_TWOPI = 6.28318530717958647692f;

// SimulatePartialDriftKernel, simulation_kernel.cu:86-118
struct DriftMap {
  RefK r;
  float hf, aper2, c;  // c = 2 pi hf / lambda
  uint32_t eid;
  __device__ uint32_t apply(Part &p) const {
    const float x = fmaf(p.xp, hf, p.x), y = fmaf(p.yp, hf, p.y);
    if (aper2 != 0.0f && x * x + y * y > aper2) { p.lo = eid; return WR_LOSS; }
    p.x = x;
    p.y = y;
    float g, beta;
    p.ph = fmaf(c, dinvb(p.w, r, g, beta), p.ph);
    return WR_X | WR_Y | WR_PH;
  }
};

// SimulateHalfQuadKernel, simulation_kernel.cu:142-218 (coordinates are
// written before the aperture test, the phase only for particles kept).
// k = sqrt(|qG| c / (m beta gamma)) differs from the synchronous particle's
// k_r by a small fraction, so sin, cos, sinh, cosh of k ds/4 are Taylor
// steps of order 4 from their FP64 values at k_r ds/4 (truncation below
// e^5/120 for the step e).
struct QuadMap {
  RefK r;
  float len, aper2, qg, c;         // c = 2 pi len / (2 lambda)
  float sk0, isk0;                 // sqrt(|qG| c / m) and its inverse
  float kds_r, s_r, c_r, sh_r, ch_r;
  uint32_t eid;
  __device__ uint32_t apply(Part &p) const {
    float x = p.x, y = p.y, xp = p.xp, yp = p.yp;
    uint32_t m;
    if (qg == 0.0f) {
      // the drifted coordinates are stored, but the aperture test below sees
      // the ones before the half (the reference writes memory and tests its
      // unchanged locals)
      p.x = x + xp * len * 0.5f;
      p.y = y + yp * len * 0.5f;
      m = WR_X | WR_Y;
      if (aper2 != 0.0f && x * x + y * y > aper2) { p.lo = eid; return m | WR_LOSS; }
      float g, beta;
      p.ph = fmaf(c, dinvb(p.w, r, g, beta), p.ph);
      return m | WR_PH;
    } else {
      const float g = fmaf(p.w, r.minv, r.g);
      const float bg = sqrt_fast(g * (g + 2.0f) * (1.0f + xp * xp + yp * yp));
      const float rb = rsqrtf(bg);
      const float k = sk0 * rb;              // sqrt(kcoef / bg)
      const float inv_k = bg * rb * isk0;    // sqrt(bg / kcoef)
      const float e = len * 0.25f * k - kds_r;
      const float e2 = e * e;
      const float t1 = e * (1.0f + e2 * (1.0f / 6.0f)), t0 = e2 * (0.5f + e2 * (1.0f / 24.0f));
      // sin(a + e) = s_r (1 - e^2/2 + e^4/24) + c_r (e - e^3/6); sinh, cosh alike
      const float s = fmaf(c_r, e - e * e2 * (1.0f / 6.0f), s_r * (1.0f - e2 * (0.5f - e2 * (1.0f / 24.0f))));
      const float cc = fmaf(-s_r, e - e * e2 * (1.0f / 6.0f), c_r * (1.0f - e2 * (0.5f - e2 * (1.0f / 24.0f))));
      const float sh = fmaf(ch_r, t1, sh_r * (1.0f + t0));
      const float ch = fmaf(sh_r, t1, ch_r * (1.0f + t0));
      const float sovk = s * inv_k, shovk = sh * inv_k, sk = s * k, shk = sh * k;
      float xx, yy;
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
      m = WR_X | WR_Y | WR_XP | WR_YP;
    }
    p.x = x; p.y = y; p.xp = xp; p.yp = yp;
    if (aper2 != 0.0f && x * x + y * y > aper2) { p.lo = eid; return m | WR_LOSS; }
    float g, beta;
    p.ph = fmaf(c, dinvb(p.w, r, g, beta), p.ph);
    return m | WR_PH;
  }
};

// SimulateSteererKernel, simulation_kernel.cu:120-140
struct SteerMap {
  RefK r;
  float kh, kv;  // B L q c / m of each plane, 0 when off
  __device__ uint32_t apply(Part &p) const {
    const float g = fmaf(p.w, r.minv, r.g);
    const float btgm = sqrtf(g * (g + 2.0f));
    uint32_t m = 0;
    if (kh != 0.0f) { p.xp += kh / btgm; m |= WR_XP; }
    if (kv != 0.0f) { p.yp += kv / btgm; m |= WR_YP; }
    return m;
  }
};

// RF gap first half (simulation_kernel.cu:226-288): every branch advances
// phi by K / beta: DTL K = beta_in (pi clbl + dps) + pi dcell/lambda -
// pi q1/lambda, CCL K = betag (pi clbl + dps) (+ const), zero amplitude
// K = 2 pi dd1 / lambda.
struct Gap1Map {
  RefK r;
  float dd1, K;
  __device__ uint32_t apply(Part &p) const {
    p.x = fmaf(dd1, p.xp, p.x);
    p.y = fmaf(dd1, p.yp, p.y);
    float g, beta;
    p.ph = fmaf(K, dinvb(p.w, r, g, beta), p.ph);
    return WR_X | WR_Y | WR_PH;
  }
};

// sin and cos of a phase: reduced to [-pi, pi] by whole turns, then the
// hardware approximation (absolute error about 2^-21 there, below the FP32
// rounding of the phase offsets it is applied to)
__device__ __forceinline__ void fast_sincos(float a, float *s, float *c) {
  const float r = fmaf(-6.28318530717958647692f, rintf(a * 0.15915494309189533577f), a);
  __sincosf(r, s, c);
}

// Bessi0c / Bessi1c (simulation_kernel.cu:15-73) in FP32; bessi0c also
// returns I0 - 1 without cancellation
__device__ inline float fbessi0c(float x, float *m1) {
  const float ax = fabsf(x);
  if (ax < 3.75f) {
    float cy = x * (1.0f / 3.75f);
    cy = cy * cy;
    const float s = cy * (3.5156229f + cy * (3.0899424f + cy * (1.2067492f + cy * (0.2659732f +
                    cy * (0.360768e-1f + cy * 0.45813e-2f)))));
    *m1 = s;
    return 1.0f + s;
  }
  const float cy = __fdividef(3.75f, ax);
  const float ans = (expf(ax) * rsqrtf(ax)) * (0.39894228f + cy * (0.1328592e-1f + cy * (0.225319e-2f +
                    cy * (-0.157565e-2f + cy * (0.916281e-2f + cy * (-0.2057706e-1f + cy * (0.2635537e-1f +
                    cy * (-0.1647633e-1f + cy * 0.392377e-2f))))))));
  *m1 = ans - 1.0f;
  return ans;
}
__device__ inline float fbessi1c(float x) {
  const float ax = fabsf(x);
  float ans;
  if (ax < 3.75f) {
    float cy = x * (1.0f / 3.75f);
    cy = cy * cy;
    ans = ax * (0.5f + cy * (0.87890594f + cy * (0.51498869f + cy * (0.15084934f + cy * (0.2658733e-1f +
          cy * (0.301532e-2f + cy * 0.32411e-3f))))));
  } else {
    const float cy = __fdividef(3.75f, ax);
    ans = 0.2282967e-1f + cy * (-0.2895312e-1f + cy * (0.1787654e-1f - cy * 0.420059e-2f));
    ans = 0.39894228f + cy * (-0.3988024e-1f + cy * (-0.362018e-2f + cy * (0.163801e-2f + cy *
          (-0.1031555e-1f + cy * ans))));
    ans = ans * (expf(ax) * rsqrtf(ax));
  }
  return x < 0.0f ? -ans : ans;
}

// RF gap second half (simulation_kernel.cu:310-497).  The synchronous
// particle's kick is formed on the host; a particle's is taken as the
// difference from it.  When the synchronous particle drifts through the
// gap (zero amplitude, or a CCL gap below the fit range) a kicked particle
// is measured from a hypothetical kicked synchronous particle (rh) and moved
// to the actual one by corr_phi / corr_w.
struct Gap2Map {
  RefK rin, rh;          // reference before the gap, reference after its (hypothetical) kick
  float dd2, drift_c;    // drift branch: phi += drift_c / beta
  float fbc, fbm, b0, tc[6], sc[6], inv2pifbc;  // T(beta), S(beta) as Taylor series about b0
  float beta_in, inv_beta_in, betag_ccl, gmg, inv_gmg, q, efl, efl_m, concomm, concomm1, con1, con2nex, inv_gmg2,
      inv_gmgcl, inv_fkis, fkr, sinps, cosps, X, ccl_dg;
  float sinF, cosF, prome1_r, sinP, cosP, tw_r, prome_r, K2;
  float dphi_ref, dw_ref;  // actual reference change
  float corr_phi, corr_w;  // hypothetical minus actual reference after the gap
  int ccl, amp0, ref_drift;
  __device__ uint32_t apply(Part &p) const {
    const Gap2Map &G = *this;
    float x = p.x, y = p.y, xp = p.xp, yp = p.yp;
    const float dphi = p.ph, dw = p.w;
    float g, beta, bg1;
    const float D = dinvb(dw, G.rin, g, beta, bg1);
    // GetTransitTimeFactors (simulation_kernel.cu:290-308) about the reference's beta
    float bcl = beta;
    if (beta > 1.1f * G.fbc) bcl = G.fbc;
    else if (beta < G.fbm) bcl = G.fbm;
    const float u = bcl - G.b0;
    const float dT = u * (tc[1] + u * (tc[2] + u * (tc[3] + u * (tc[4] + u * tc[5]))));
    const float t = tc[0] + dT;
    const float dTd = tc[1] + u * (2.0f * tc[2] + u * (3.0f * tc[3] + u * (4.0f * tc[4] + 5.0f * u * tc[5])));
    const float dSd = sc[1] + u * (2.0f * sc[2] + u * (3.0f * sc[3] + u * (4.0f * sc[4] + 5.0f * u * sc[5])));
    const float coef = bcl * bcl * G.inv2pifbc;
    const float tp = coef * dTd, sp = -coef * dSd;
    if (G.amp0 || (G.ccl && beta < G.fbm)) {
      p.x = fmaf(G.dd2, xp, x);
      p.y = fmaf(G.dd2, yp, y);
      if (G.ref_drift) {
        p.ph = fmaf(G.drift_c, D, dphi);
        return WR_X | WR_Y | WR_PH;
      }
      p.ph = dphi + G.drift_c / beta - G.dphi_ref;
      p.w = dw - G.dw_ref;
      return WR_X | WR_Y | WR_PH | WR_W;
    }
    float tw, dtw;
    if (G.ccl) {
      tw = t - F_TWOPI * tp * (__fdividef(G.beta_in, beta) - 1.0f) * G.betag_ccl * G.inv_beta_in;
      dtw = tw - G.tw_r;
    } else {
      tw = t;
      dtw = dT;
    }
    const float con5nex = G.concomm * (t * G.inv_fkis - G.X * tp * G.inv_gmg2);
    const float con5nex1 = G.concomm1 * t;
    const float con5nex2 = -G.con2nex * t * G.inv_fkis;
    const float delta = G.ccl ? dphi - G.ccl_dg * D : dphi;
    float sd, cd;
    fast_sincos(delta, &sd, &cd);
    const float sinp1 = G.sinF * cd + G.cosF * sd, cosp1 = G.cosF * cd - G.sinF * sd;
    const float prome1 = -G.con1 * (tp * (sinp1 - G.sinps) + sp * (cosp1 - G.cosps));
    const float eps = delta + (prome1 - G.prome1_r);
    // sin and cos of eps from those of eps/2 (one evaluation instead of two;
    // 2 sin^2(eps/2) = 1 - cos(eps) is the form dcos needs anyway)
    float sh, ch;
    fast_sincos(0.5f * eps, &sh, &ch);
    const float se = 2.0f * sh * ch, omc = 2.0f * sh * sh, ce = 1.0f - omc;
    const float sinp = G.sinP * ce + G.cosP * se, cosp = G.cosP * ce - G.sinP * se;
    const float dcos = -G.cosP * omc - G.sinP * se;
    const float rs_p = x * x + y * y, rrp = x * xp + y * yp;
    const float ris = sqrt_fast(rs_p), fkrris = G.fkr * ris;
    float b0m1;
    const float b0c = fbessi0c(fkrris, &b0m1);
    const float b1c = fbessi1c(fkrris);
    const float b1p = fkrris != 0.0f ? b0c - __fdividef(b1c, fkrris) : 0.5f;
    const float bes1covr = ris != 0.0f ? __fdividef(b1c, ris) : G.fkr * 0.5f;
    const float rest = ((tw - F_TWOPI * tp) * G.inv_gmg * bes1covr + tw * G.inv_gmg * G.fkr * b1p -
                        tw * G.gmg * bes1covr) * rrp * sinp;
    const float ddelte = G.q * G.efl * (tw * b0c * dcos + (dtw * b0c + G.tw_r * b0m1) * G.cosP + rest);
    const float dwh = dw + ddelte;
    float gh, betah, bg;
    const float Dh = dinvb(dwh, G.rh, gh, betah, bg);
    const float bgr = __fdividef(bg1, bg);
    const float onema = 1.0f - (con5nex * bes1covr + con5nex1 * b1p + con5nex2 * bes1covr) * cosp;
    const float dovbl = G.con2nex * bes1covr * tw * sinp;
    const float bgrovonema = __fdividef(bgr, onema);
    xp = -dovbl * x + bgrovonema * xp;
    x = x * onema + G.dd2 * xp;
    yp = -dovbl * y + bgrovonema * yp;
    y = y * onema + G.dd2 * yp;
    const float rpris = rs_p > 0.0f ? __fdividef(rrp, ris) : 0.0f;
    const float prome = 2.0f * G.con1 * (-tp * b0c + ris * tw * b1c * G.inv_gmgcl) * (sinp - G.sinps) -
                        G.efl_m * tw * b1c * rpris * (cosp - G.cosps);
    const float dphih = dphi + G.K2 * Dh + (prome - G.prome_r);
    const float wabs = G.rh.w + dwh;
    if (wabs <= 0.0f || x != x || y != y || xp != xp || yp != yp || dwh != dwh || dphih != dphih) {
      p.lo = 33333333u;
      return WR_LOSS;
    }
    p.x = x; p.y = y; p.xp = xp; p.yp = yp;
    p.ph = dphih + G.corr_phi;
    p.w = dwh + G.corr_w;
    return WR_X | WR_Y | WR_XP | WR_YP | WR_PH | WR_W;
  }
};

// SimulateBuncherKernel, simulation_kernel.cu:807-871
struct BunchMap {
  RefK r;
  float hr, sinB, cosB, k2q, qV, con1, beta_w, aper2;
  uint32_t eid;
  __device__ uint32_t apply(Part &p) const {
    const float x = p.x, y = p.y, dw = p.w;
    const float r2 = x * x + y * y;
    if (aper2 != 0.0f && r2 > aper2) { p.lo = eid; return WR_LOSS; }
    const float delta = hr * p.ph;
    float sd, cd;
    sincosf(delta, &sd, &cd);
    const float cosph = cosB * cd - sinB * sd, sinph = sinB * cd + cosB * sd;
    const float sh = sinf(0.5f * delta);
    const float dcos = -cosB * 2.0f * sh * sh - sinB * sd;
    const float arg = k2q * r2;
    const float poly = arg * (1.0f + arg * (0.25f + arg / 36.0f));
    const float dwi = qV * cosph * (1.0f + poly);
    const float ddw = qV * (dcos + cosph * poly);
    const float w = r.w + dw;
    const float wb_par = w + 0.5f * dwi, wf = w + dwi;
    if (wb_par <= 0.0f || wf <= 0.0f) { p.lo = eid; return WR_LOSS; }
    float gt = wb_par * r.minv;
    const float bav = sqrtf(gt * (gt + 2.0f)) / (gt + 1.0f);
    gt = fmaf(dw, r.minv, r.g);
    const float bg = sqrtf(gt * (gt + 2.0f));
    gt = wf * r.minv;
    const float rbgf = rsqrtf(gt * (gt + 2.0f));
    const float del = -con1 * sinph * (1.0f - bav * beta_w) * (0.5f + arg * (0.25f + arg / 24.0f)) / bav;
    p.xp = (p.xp * bg + del * x) * rbgf;
    p.yp = (p.yp * bg + del * y) * rbgf;
    p.w = dw + ddw;
    return WR_XP | WR_YP | WR_W;
  }
};

// SimulateRotationKernel, simulation_kernel.cu:511-529
struct RotMap {
  float cosa, sina;
  __device__ uint32_t apply(Part &p) const {
    const float x = p.x, y = p.y, xp = p.xp, yp = p.yp;
    p.x = x * cosa + y * sina;
    p.y = y * cosa - x * sina;
    p.xp = xp * cosa + yp * sina;
    p.yp = yp * cosa - xp * sina;
    return WR_X | WR_Y | WR_XP | WR_YP;
  }
};

// Simulate{First,Second}HalfDipoleKernel, simulation_kernel.cu:603-805
struct DipMap {
  float r11, r12, r16, r21, r22, r26, r33, r34, r43, r44, r51, r52, r56, e21, e43;
  float cdp, dpop_ref, cph;  // dpop_i = dpop_ref + cdp * dw; phase offset = cph * (...)
  int second;
  __device__ uint32_t apply(Part &p) const {
    float x = p.x, xp = p.xp, y = p.y, yp = p.yp;
    const float ddp = cdp * p.w;
    const float dpop = dpop_ref + ddp;
    if (!second) {
      xp += e21 * x;
      yp -= e43 * y;
      p.x = r11 * x + r12 * xp + r16 * dpop;
      p.xp = r21 * x + r22 * xp + r26 * dpop;
      p.y = r33 * y + r34 * yp;
      p.yp = r43 * y + r44 * yp;
      p.ph -= cph * (r51 * x + r52 * xp + r56 * ddp);
    } else {
      p.ph -= cph * (r51 * x + r52 * xp + r56 * ddp);
      const float xn = r11 * x + r12 * xp + r16 * dpop;
      xp = r21 * x + r22 * xp + r26 * dpop;
      const float yn = r33 * y + r34 * yp;
      yp = r43 * y + r44 * yp;
      p.x = xn;
      p.y = yn;
      p.xp = xp + e21 * xn;
      p.yp = yp - e43 * yn;
    }
    return WR_X | WR_Y | WR_XP | WR_YP | WR_PH;
  }
};

}  // namespace hps
