// sc32_kick.cuh -- the SCHEFF kick of one FP32 particle (ApplySpchKickKernel,
// src/simulation/inc/space_charge_kernel.cu:573-706), shared by the plain
// kick kernel (scheff32.cu) and the kernels that run the kick and the next
// element map in one sweep (push32.cu).
//
// The bunch-frame momentum p* = gamma_c (beta gamma - beta_c gamma) is formed
// as (gamma - gamma_c)(gamma + gamma_c) / (gamma_c (beta gamma + beta_c
// gamma)); with the exact inverse transform beta gamma = gamma_c (p* +
// beta_c sqrt(1 + p*^2)) the reference's change of beta gamma is
//   gamma_c (dp + beta_c [dp (2 p* + dp) / 2 + p*^4 / (4 (1 + p*^2/2 +
//   sqrt(1 + p*^2)))]),
// neither of which cancels in FP32.
#pragma once

#include "push32_maps.cuh"

namespace hps {

// everything one kick launch reads besides the particles
struct KickEnv {
  const float2 *fld;
  RefK r;  // synchronous particle at the kick
  float pag;  // origin of the relative phase: wrap(phi - pag)
  float phimc, xbar, ybar, epsq, inv_epsq, beta, gmg, inv_dr, inv_dzg, hl, rmesh, c2, xfac, yfac, cbgcoef, pl,
      er_c3, ez_c3, dwc;
  uint32_t nx, nz, adj, tbl_sz;
};

__device__ inline KickEnv kick_env(const ScState *sc, const ScTables &t, const RefK &r) {
  const Sc32Consts &kc = *t.c32;
  KickEnv e;
  e.fld = (const float2 *)t.ffld2;
  e.r = r;
  e.nx = sc->nx;
  e.nz = sc->nz;
  e.adj = sc->adj;
  e.tbl_sz = (e.nx + 1) * (e.nz + 1);
  e.cbgcoef = kc.cbg_per_onm * (float)sc->num_on_mesh;
  e.pag = kc.pag;
  e.phimc = kc.phimc; e.xbar = kc.xbar; e.ybar = kc.ybar; e.epsq = kc.epsq; e.inv_epsq = kc.inv_epsq;
  e.beta = kc.beta; e.gmg = kc.gmg; e.inv_dr = kc.inv_dr; e.inv_dzg = kc.inv_dzg; e.hl = kc.hl;
  e.rmesh = kc.rmesh; e.c2 = kc.c2; e.xfac = kc.xfac; e.yfac = kc.yfac; e.pl = kc.pl;
  e.er_c3 = kc.er_c3; e.ez_c3 = kc.ez_c3; e.dwc = kc.dwc;
  return e;
}

// wrap into [-pi, pi] by whole turns (space_charge_kernel.cu:160-166); the
// relative phases are already wrapped, so one turn at most is removed
__device__ inline float wrap_turns(float d) {
  const float pi = 3.14159265358979323846f, twopi = 6.28318530717958647692f;
  for (int guard = 0; (d > pi || d < -pi) && guard < 64; ++guard) d += d > 0.0f ? -twopi : twopi;
  return d;
}

// kick particle p (live, not longitudinally lost) whose relative phase is
// phi; returns the fields changed.  Quotients whose denominators are
// bounded away from zero and overflow use the two-ulp reciprocal-multiply
// (__fdividef), the square roots of the common path the hardware
// approximation (sqrt_fast).
__device__ inline uint32_t kick_particle(Part &p, float phi, const KickEnv &e) {
  const float dw = p.w;
  const float g = fmaf(dw, e.r.minv, e.r.g);
  const float gm = g + 1.0f;
  const float bgz = sqrt_fast(g * (g + 2.0f));
  float bgx = bgz * p.xp, bgy = bgz * p.yp;
  const float dgc = (dw + e.dwc) * e.r.minv;  // gm - gamma_c
  const float s0 = __fdividef(dgc * (gm + e.gmg), e.gmg * (bgz + e.beta * gm));
  const float xxbar = p.x - e.xbar, yybar = p.y - e.ybar;
  float rr = sqrt_fast(xxbar * xxbar * e.inv_epsq + yybar * yybar * e.epsq);
  if (rr == 0.0f) rr = 1.0e-8f;
  const float inv_rr = __fdividef(1.0f, rr);
  const float xovr = xxbar * e.xfac * inv_rr, yovr = yybar * e.yfac * inv_rr;
  float z = -e.c2 * wrap_turns(phi - e.phimc);
  float cbgr, cbgzs;
  if (rr > e.rmesh || fabsf(z) > e.hl) {
    z = -e.c2 * (phi - e.phimc);
    float d = sqrtf(z * z + rr * rr);
    float invd3 = 1.0f / (d * d * d);
    float rod3 = rr * invd3, zod3 = z * invd3;
    for (uint32_t nb = 1; nb <= e.adj; ++nb) {
      float xi = (float)nb;
      for (int lr = 0; lr < 2; ++lr) {
        const float sft = z + xi * e.pl;
        d = sqrtf(sft * sft + rr * rr);
        invd3 = 1.0f / (d * d * d);
        rod3 += rr * invd3;
        zod3 += sft * invd3;
        xi = -xi;
      }
    }
    cbgr = e.cbgcoef * rod3;
    cbgzs = e.cbgcoef * zod3;
  } else {
    const float ri = rr * e.inv_dr;
    const uint32_t i = 1 + (int)ri;
    const float a = ri - (float)(i - 1);
    const float bb = 1.0f - a;
    const float zi = (z + e.hl) * e.inv_dzg;
    const uint32_t j = 1 + (int)zi;
    const float c = zi - (float)(j - 1);
    const float d = 1.0f - c;
    uint32_t l = (j - 1) * (e.nx + 1) + i;
    uint32_t m = l + (e.nx + 1);
    if (m >= e.tbl_sz) m = e.tbl_sz - 1;
    if (l >= e.tbl_sz || l < 1) l = e.tbl_sz - 1;
    if (m < 1) m = 1;
    const float2 fl = e.fld[l], fl1 = e.fld[l - 1], fm = e.fld[m], fm1 = e.fld[m - 1];
    cbgr = e.er_c3 * (d * (a * fl.x + bb * fl1.x) + c * (a * fm.x + bb * fm1.x));
    cbgzs = e.ez_c3 * (d * (a * fl.y + bb * fl1.y) + c * (a * fm.y + bb * fm1.y));
  }
  bgx += cbgr * xovr;
  bgy += cbgr * yovr;
  // bgzf = gamma_c (p* + dp + beta_c (1 + (p* + dp)^2 / 2)) taken as
  // bgz + (bgzf - bgz): the change is formed without cancellation and bgz
  // comes straight from the particle's energy
  const float s2 = s0 * s0;
  const float dbgz = e.gmg * (cbgzs + e.beta * (0.5f * cbgzs * (2.0f * s0 + cbgzs) +
                                                __fdividef(s2 * s2, 4.0f * (1.0f + 0.5f * s2 + sqrt_fast(1.0f + s2)))));
  const float bgzf = bgz + dbgz;
  if (bgzf <= 0.0f) {
    p.lo = 9999u;
    return WR_LOSS;
  }
  const float inv_f = __fdividef(1.0f, bgzf);
  p.xp = bgx * inv_f;
  p.yp = bgy * inv_f;
  const float w = e.r.w + dw;
  p.w = dw + __fdividef(w * (gm + 1.0f) * dbgz, gm * bgz);
  return WR_XP | WR_YP | WR_W;
}

}  // namespace hps
