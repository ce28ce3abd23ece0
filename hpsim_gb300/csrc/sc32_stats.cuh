// sc32_stats.cuh -- the SCHEFF decision and the constants of an FP32 kick,
// taken by the one thread that finalises the statistics sweep: the sweeps
// of scheff32.cu, or an element map fused with the first of them (push32.cu).
#pragma once

#include "common.cuh"
#include "scheff_common.cuh"

namespace hps {
namespace {

// gamma, beta of the bunch-frame reference from <W>_good: gamma = 1 + W/m
// exactly, beta = sqrt(g (g + 2)) / (g + 1) without the 1 - 1/gamma^2
// cancellation at low energy
__device__ inline void sc32_kinematics(double ke, float inv_mass, float &gamma, float &beta) {
  const float g = (float)ke * inv_mass;
  gamma = 1.0f + g;
  beta = sqrtf(g * (g + 2.0f)) / gamma;
}

// UpdateScheffMeshSizeKernel (space_charge_kernel.cu:18-32) in FP32
__device__ inline void mesh_size32(ScState *s, float beta, float wave_len, float partial_r, float partial_z,
                                   float coef) {
  const float bl = beta * wave_len;
  s->dr = coef * partial_r / (float)s->nx;
  if (coef == 1.0f) s->dz = bl / (float)s->nz;
  else s->dz = coef * bl * partial_z / ((float)s->nz * 3.14159265358979f);
}

// Scheff::Start's decision (space_charge.cpp:86-138, as scheff_decide) in
// FP32 arithmetic; relative-change tests as |a - b| > threshold * b
__device__ void scheff_decide32(const BeamStats &st, const DevBeam &b, ScState *s, const Sc32Host &h, double freq,
                                double frac) {
  const uint32_t good_cnt = st.num_good;
  const float sigphi = b.n < 2 ? 0.0f : (float)st.st[PHI_SIG_GOOD];
  const float sigx = b.n < 2 ? 0.0f : (float)st.st[X_SIG_GOOD];
  const float sigy = b.n < 2 ? 0.0f : (float)st.st[Y_SIG_GOOD];
  const double ke = st.st[W_AVG_GOOD];
  float gamma, beta;
  sc32_kinematics(ke, h.inv_mass, gamma, beta);
  const float sigz = sigphi * (0.5f / 3.14159265f) * beta * h.wave_len;
  const float sigr = sqrtf(sigx * sigx + sigy * sigy);
  const float cratior = sigr * sigz, cratioz = sigz * sigz * gamma * gamma;
  const float sro = (float)s->sigr_old, szo = (float)s->sigz_old, gmo = (float)s->gm_old;
  const float cratior_old = sro * szo, cratioz_old = szo * szo * gmo * gmo;
  const uint32_t adj = (s->adj_bunch_w == 0.0 || ke < s->adj_bunch_w) ? s->adj_bunch : 0u;
  s->resized = 0;
  if (s->mesh_w != 0.0) {
    if (ke > s->mesh_w && (s->nx != s->nx_init / 2 || s->nz != s->nz_init / 2))
      set_mesh_size(s, s->nx_init / 2, s->nz_init / 2);
    else if (ke <= s->mesh_w && (s->nx != s->nx_init || s->nz != s->nz_init))
      set_mesh_size(s, s->nx_init, s->nz_init);
    if (ke > s->mesh_w && s->interval != s->interval_init * 4) s->interval = s->interval_init * 4;
    else if (ke <= s->mesh_w && s->interval != s->interval_init) s->interval = s->interval_init;
  }
  s->freq = freq;
  s->beta = beta;
  s->frac = frac;
  s->adj = adj;
  const float thr = (float)s->remesh_val;
  if (cratior_old == 0.0f || cratioz_old == 0.0f || fabsf(cratior - cratior_old) > thr * cratior_old ||
      fabsf(cratioz - cratioz_old) > thr * cratioz_old) {
    s->sigr_old = sigr;
    s->sigz_old = sigz;
    s->gm_old = gamma;
    s->good_cnt_old = good_cnt;
    s->remesh = 1;
    s->n_solves += 1;
    s->ratio_r = s->ratio_z = s->ratio_q = s->ratio_g = 1.0;
    // y branch of the pointer comparison (see scheff_decide)
    if (adj == 0) mesh_size32(s, beta, h.wave_len, sigy, sigphi, 3.0f);
  } else {
    s->remesh = 0;
    s->ratio_r = sigr / sro;
    s->ratio_z = sigz / szo;
    s->ratio_q = s->good_cnt_old ? (double)(good_cnt / s->good_cnt_old) : 0.0;
    s->ratio_g = gamma / gmo;
  }
}

// Constants of the kick about to run, from the statistics and the decision
// (ApplySpchKickKernel, space_charge_kernel.cu:573-620; UpdateFldTbl1Kernel,
// :39-60; DistributeParticleKernel, :123-150), once per kick.  The only FP64
// operations are the offsets of <W>_good and <phi>_good from the synchronous
// particle.
__device__ void sc32_consts(const BeamStats &st, const DevBeam &b, const ScState *s, Sc32Consts *c,
                            const Sc32Host &h) {
  const double ke = st.st[W_AVG_GOOD];
  float gmg, beta;
  sc32_kinematics(ke, h.inv_mass, gmg, beta);
  const float sx = (float)st.st[X_SIG_GOOD], sy = (float)st.st[Y_SIG_GOOD];
  const float epsq = sx / sy;
  const float dr0 = (float)s->dr, dzg0 = (float)s->dz * gmg;
  const float dr = dr0 * (float)s->ratio_r, dzg = dzg0 * (float)s->ratio_z;
  const float c3 = h.length / (beta * gmg);
  const float rr = (float)s->ratio_r, rz = (float)s->ratio_z, rq = (float)s->ratio_q, rg = (float)s->ratio_g;
  c->pag = (float)(st.st[PHI_AVG_GOOD] - b.phi_ref);
  c->phimc = (float)st.st[PHI_AVG_R];
  c->xbar = (float)st.st[X_AVG_GOOD];
  c->ybar = (float)st.st[Y_AVG_GOOD];
  c->epsq = epsq;
  c->inv_epsq = sy / sx;
  c->xfac = 2.0f / (epsq + 1.0f);
  c->yfac = epsq * c->xfac;
  c->beta = beta;
  c->gmg = gmg;
  c->pl = beta * gmg * h.wave_len;
  c->c2 = c->pl * (1.0f / 6.28318530717958647692f);
  c->dr = dr;
  c->dzg = dzg;
  c->inv_dr = 1.0f / dr;
  c->inv_dzg = 1.0f / dzg;
  c->hl = (float)s->nz * 0.5f * dzg;
  c->rmesh = (float)s->nx * dr;
  c->dr0 = dr0;
  c->dzg0 = dzg0;
  c->inv_dr0 = 1.0f / dr0;
  c->inv_dzg0 = 1.0f / dzg0;
  c->hl0 = (float)s->nz * 0.5f * dzg0;
  c->cbg_per_onm = h.c1 * c3 * (3.14159265358979f * 0.5f);
  c->er_c3 = rq / (rr * rz * rg * rg) * c3;
  c->ez_c3 = rq / (rz * rz) * c3;
  c->dwc = (float)(b.w_ref - ke);  // W_sync - W_c: gamma_c = 1 + <W>_good / m
  c->green_c1 = h.c1;
}

// The decision and the kick constants on local copies of the solver state:
// one burst of loads, one burst of stores, and no load waiting behind a
// store that might alias it.
__device__ void sc32_decide_consts(const BeamStats &st, const DevBeam &b, ScState *sc, Sc32Consts *c32,
                                   const Sc32Host &h, double freq, double frac) {
  ScState s = *sc;
  Sc32Consts c;
  scheff_decide32(st, b, &s, h, freq, frac);
  sc32_consts(st, b, &s, &c, h);
  *sc = s;
  *c32 = c;
}


// The SCHEFF moments from their totals s[0..7] (FP32 arithmetic, see
// Sc32Host), then, with a solver, the decision and the kick's constants
// (thread 0); the caller zeroes the tables afterwards.
__device__ void sc_moments_finish(const DevBeam &b, const double *s, ScState *sc, const ScTables &t, double freq,
                                  double frac, const Sc32Host &h) {
  BeamStats st = *b.st;  // local copy, written back once
  const float isv = 1.0f / (float)(uint32_t)(b.n - st.num_loss), ing = 1.0f / (float)st.num_good;
  st.st[PHI_AVG_R] = (float)s[0] * isv;
  const float pa = (float)s[1] * ing, pa2 = (float)s[2] * ing;
  st.st[PHI_SIG_GOOD] = sqrtf(pa2 - pa * pa);
  const float xa = (float)s[3] * isv, x2 = (float)s[4] * isv, ya = (float)s[5] * isv, y2 = (float)s[6] * isv;
  st.st[X_AVG_GOOD] = xa;
  st.st[X_SIG_GOOD] = sqrtf(x2 - xa * xa);
  st.st[Y_AVG_GOOD] = ya;
  st.st[Y_SIG_GOOD] = sqrtf(y2 - ya * ya);
  st.st[W_AVG_GOOD] = st.num_good > 0 ? (double)((float)s[7] * ing) + b.w_ref : -99999;
  *b.st = st;
  if (sc) sc32_decide_consts(st, b, sc, t.c32, h, freq, frac);
}

// the SCHEFF moments' per-particle terms: 0 mean relative phase of the live
// set, 1-2 phase, 3-6 x, x^2, y, y^2, 7 W of the good set
__device__ inline void sc_moments_add(float (&a)[12], float pr, uint32_t lo, uint32_t ll, float x, float y, float w) {
  const float alive = lo == 0u ? 1.0f : 0.0f;
  const float gd = (lo == 0u && ll == 0u) ? 1.0f : 0.0f;
  a[0] += alive * pr;
  a[1] += gd * pr; a[2] += gd * pr * pr;
  a[3] += gd * x; a[4] += gd * x * x; a[5] += gd * y; a[6] += gd * y * y;
  a[7] += gd * w;
}

}  // namespace
}  // namespace hps
