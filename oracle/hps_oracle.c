/*
 * hps_oracle.c -- FP64 CPU restatement of HPSim's per-element tracking path.
 *
 * TEST INFRASTRUCTURE ONLY (see hps_oracle.h).  Each function restates one
 * routine of the reference and cites it.  All file:line citations are
 * relative to the reference project root.
 *
 * Summation order: every reduction is split into ORC_NCHUNK fixed chunks
 * summed sequentially and merged in chunk order, so results do not depend on
 * the number of host threads.  The reference's own order (Harris tree
 * reductions, float/double atomics) is not reproducible either, so moment
 * parity is stated with a tolerance, loss flags are compared exactly.
 */
#define _GNU_SOURCE
#include "hps_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/util/inc/constant.h:7-11 */
#define CLIGHT 299.792458
#define PI 3.14159265358979323846
#define TWOPI (3.14159265358979323846 * 2.0)

#define ORC_NCHUNK 64

static inline uint64_t chunk_lo(uint32_t n, int c) { return (uint64_t)n * (uint64_t)c / ORC_NCHUNK; }

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* src/util/src/utility.cpp:7-16 */
static uint32_t next_pow2(uint32_t x) {
  --x;
  x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
  return ++x;
}

/* Beam::SetNumThreadsPerBlock, src/beam/src/beam.cpp:148-168 */
static void set_launch(orc_beam *b) {
  uint32_t nt = next_pow2(b->n);
  if (nt > 256) { b->grid_size = nt / 256; b->blck_size = 256; }
  else { b->grid_size = 1; b->blck_size = nt; }
}

static double *coord_ptr(const orc_beam *b, int c) {
  switch (c) {
    case HPS_COORD_X: return b->x;
    case HPS_COORD_XP: return b->xp;
    case HPS_COORD_Y: return b->y;
    case HPS_COORD_YP: return b->yp;
    case HPS_COORD_PHI: return b->phi;
    case HPS_COORD_W: return b->w;
    default: return b->phi_r;
  }
}

/* ------------------------------------------------------------------ */
/* Beam construction: src/beam/src/beam.cpp:124-134, beam.cu:24-112     */
/* ------------------------------------------------------------------ */
orc_beam *orc_beam_create(uint32_t n, double mass, double charge, double current) {
  orc_beam *b = (orc_beam *)calloc(1, sizeof(orc_beam));
  b->n = n; b->mass = mass; b->charge = charge; b->current = current;
  b->freq = 0.0; b->design_w = 0.0;
  size_t nd = (size_t)(n ? n : 1) * sizeof(double);
  size_t nu = (size_t)(n ? n : 1) * sizeof(uint32_t);
  b->x = (double *)calloc(1, nd); b->xp = (double *)calloc(1, nd);
  b->y = (double *)calloc(1, nd); b->yp = (double *)calloc(1, nd);
  b->phi = (double *)calloc(1, nd); b->phi_r = (double *)calloc(1, nd);
  b->w = (double *)calloc(1, nd);
  b->loss = (uint32_t *)calloc(1, nu); b->lloss = (uint32_t *)calloc(1, nu);
  set_launch(b);
  return b;
}

void orc_beam_free(orc_beam *b) {
  if (!b) return;
  free(b->x); free(b->xp); free(b->y); free(b->yp); free(b->phi); free(b->phi_r);
  free(b->w); free(b->loss); free(b->lloss);
  for (int s = 0; s < 2; ++s) {
    for (int k = 0; k < 6; ++k) free(b->save[s][k]);
    free(b->save_loss[s]); free(b->save_lloss[s]);
  }
  free(b);
}

/* UpdateBeamOnDevice, src/beam/src/beam.cu:197-218 */
static void upload(orc_beam *b, const double *x, const double *xp, const double *y,
                   const double *yp, const double *phi, const double *w,
                   const uint32_t *loss, const uint32_t *lloss) {
  size_t nd = (size_t)b->n * sizeof(double), nu = (size_t)b->n * sizeof(uint32_t);
  memcpy(b->x, x, nd); memcpy(b->xp, xp, nd); memcpy(b->y, y, nd);
  memcpy(b->yp, yp, nd); memcpy(b->phi, phi, nd); memcpy(b->w, w, nd);
  if (loss) memcpy(b->loss, loss, nu); else memset(b->loss, 0, nu);
  if (lloss) memcpy(b->lloss, lloss, nu); else memset(b->lloss, 0, nu);
}

/* Beam::InitPhiAvgGood, src/beam/src/beam.cpp:655-661 */
static void init_phi_avg_good(orc_beam *b) {
  orc_beam_update_loss(b);
  orc_beam_update_avg(b, HPS_COORD_PHI, 0);
  b->st[ORC_PHI_AVG_GOOD] = b->st[ORC_PHI_AVG];
}

/* Beam::InitBeamFromDistribution, src/beam/src/beam.cpp:317-368 */
void orc_beam_set_distribution(orc_beam *b, const double *x, const double *xp,
    const double *y, const double *yp, const double *phi, const double *w,
    const uint32_t *loss, const uint32_t *lloss) {
  upload(b, x, xp, y, yp, phi, w, loss, lloss);
  if (b->n) {
    b->x[0] = 0.0; b->xp[0] = 0.0; b->y[0] = 0.0; b->yp[0] = 0.0;
    if (loss) b->loss[0] = 0;
    if (lloss) b->lloss[0] = 0;
  }
  init_phi_avg_good(b);
}

/* Beam::InitWaterbagBeam, src/beam/src/beam.cpp:391-462.  Uses the C
 * library's rand() exactly as the reference's std::rand() (same glibc
 * sequence). */
void orc_beam_set_waterbag(orc_beam *b, double r_ax, double r_bx, double r_ex,
    double r_ay, double r_by, double r_ey, double r_az, double r_bz, double r_ez,
    double r_sync_phi, double r_sync_w, double r_freq, uint32_t r_seed) {
  uint32_t n = b->n;
  double *xh = b->x, *xph = b->xp, *yh = b->y, *yph = b->yp, *phih = b->phi, *wh = b->w;
  srand(r_seed ? r_seed : 1u);
  double rsq = 1.0;
  double gx = (1.0 + r_ax * r_ax) / r_bx;
  double xmx = sqrt(r_ex / gx);
  double xpmx = sqrt(r_ex * gx);
  double dx = -r_ax / gx;
  double gy = (1.0 + r_ay * r_ay) / r_by;
  double ymx = sqrt(r_ey / gy);
  double ypmx = sqrt(r_ey * gy);
  double dy = -r_ay / gy;
  double gz = (1.0 + r_az * r_az) / r_bz;
  double zmx = sqrt(r_ez / gz);
  double zpmx = r_ez / zmx;
  double dz = -r_az / gz;
  double wave_len = 29979.2458 / r_freq;
  b->freq = r_freq;
  double gm = r_sync_w / b->mass + 1.0;
  double beta = sqrt(1.0 - 1.0 / (gm * gm));
  for (uint32_t i = 0; i < n; ++i) {
    double r1, r2, r3, r4, r5, r6;
    do {
      do { r1 = 2.0 * rand() / RAND_MAX - 1.0; r2 = 2.0 * rand() / RAND_MAX - 1.0; }
      while (r1 * r1 + r2 * r2 > 1.0);
      do { r3 = 2.0 * rand() / RAND_MAX - 1.0; r4 = 2.0 * rand() / RAND_MAX - 1.0; }
      while (r3 * r3 + r4 * r4 > 1.0);
      do { r5 = 2.0 * rand() / RAND_MAX - 1.0; r6 = 2.0 * rand() / RAND_MAX - 1.0; }
      while (r5 * r5 + r6 * r6 > 1.0);
    } while (r1 * r1 + r2 * r2 + r3 * r3 + r4 * r4 + r5 * r5 + r6 * r6 > 1.0);
    r1 *= rsq; r2 *= rsq; r3 *= rsq; r4 *= rsq; r5 *= rsq; r6 *= rsq;
    xh[i] = 0.01 * (r1 * xmx + dx * r2 * xpmx);
    xph[i] = r2 * xpmx;
    yh[i] = 0.01 * (r3 * ymx + dy * r4 * ypmx);
    yph[i] = r4 * ypmx;
    phih[i] = -(r5 * zmx + dz * zpmx * r6) * 2.0 * M_PI / (beta * wave_len) + r_sync_phi;
    wh[i] = 2.0 * r_sync_w * zpmx * r6 + r_sync_w;
  }
  if (n) { xh[0] = 0.0; xph[0] = 0.0; yh[0] = 0.0; yph[0] = 0.0; }
  memset(b->loss, 0, (size_t)n * sizeof(uint32_t));
  memset(b->lloss, 0, (size_t)n * sizeof(uint32_t));
  init_phi_avg_good(b);
}

/* Beam::InitDCBeam, src/beam/src/beam.cpp:481-537 */
void orc_beam_set_dc(orc_beam *b, double r_ax, double r_bx, double r_ex, double r_ay,
    double r_by, double r_ey, double r_dphi, double r_sync_phi, double r_sync_w,
    uint32_t r_seed) {
  uint32_t n = b->n;
  srand(r_seed ? r_seed : 1u);
  double rsq = 1.0;
  double gx = (1.0 + r_ax * r_ax) / r_bx;
  double xmx = sqrt(r_ex / gx), xpmx = sqrt(r_ex * gx), dx = -r_ax / gx;
  double gy = (1.0 + r_ay * r_ay) / r_by;
  double ymx = sqrt(r_ey / gy), ypmx = sqrt(r_ey * gy), dy = -r_ay / gy;
  for (uint32_t i = 0; i < n; ++i) {
    double r1, r2, r3, r4, r5;
    do {
      do { r1 = 2.0 * rand() / RAND_MAX - 1.0; r2 = 2.0 * rand() / RAND_MAX - 1.0; }
      while (r1 * r1 + r2 * r2 > 1.0);
      do { r3 = 2.0 * rand() / RAND_MAX - 1.0; r4 = 2.0 * rand() / RAND_MAX - 1.0; }
      while (r3 * r3 + r4 * r4 > 1.0);
    } while (r1 * r1 + r2 * r2 + r3 * r3 + r4 * r4 > 1.0);
    r1 *= rsq; r2 *= rsq; r3 *= rsq; r4 *= rsq;
    r5 = 2.0 * (double)(i + 1.0) / (double)n - 1.0;
    b->x[i] = 0.01 * (r1 * xmx + dx * r2 * xpmx);
    b->xp[i] = r2 * xpmx;
    b->y[i] = 0.01 * (r3 * ymx + dy * r4 * ypmx);
    b->yp[i] = r4 * ypmx;
    b->phi[i] = r5 * r_dphi + r_sync_phi;
    b->w[i] = r_sync_w;
  }
  if (n) { b->x[0] = 0.0; b->xp[0] = 0.0; b->y[0] = 0.0; b->yp[0] = 0.0; }
  memset(b->loss, 0, (size_t)n * sizeof(uint32_t));
  memset(b->lloss, 0, (size_t)n * sizeof(uint32_t));
  init_phi_avg_good(b);
}

/* Beam::SetRefEnergy / SetRefPhase, src/beam/src/beam.cpp:1074-1089 */
void orc_beam_set_ref_w(orc_beam *b, double w) { if (b->n) b->w[0] = w; b->design_w = w; }
void orc_beam_set_ref_phi(orc_beam *b, double phi) { if (b->n) b->phi[0] = phi; }

/* Beam::Save*Beam / Restore*Beam, src/beam/src/beam.cpp:547-647 */
void orc_beam_save(orc_beam *b, int slot) {
  double *src[6] = {b->x, b->xp, b->y, b->yp, b->phi, b->w};
  size_t nd = (size_t)b->n * sizeof(double), nu = (size_t)b->n * sizeof(uint32_t);
  for (int k = 0; k < 6; ++k) {
    if (!b->save[slot][k]) b->save[slot][k] = (double *)malloc(nd ? nd : 8);
    memcpy(b->save[slot][k], src[k], nd);
  }
  if (!b->save_loss[slot]) b->save_loss[slot] = (uint32_t *)malloc(nu ? nu : 4);
  if (!b->save_lloss[slot]) b->save_lloss[slot] = (uint32_t *)malloc(nu ? nu : 4);
  memcpy(b->save_loss[slot], b->loss, nu);
  memcpy(b->save_lloss[slot], b->lloss, nu);
  b->save_design_w[slot] = b->design_w;
  b->save_freq[slot] = b->freq;
  b->save_current[slot] = b->current;
}

int orc_beam_restore(orc_beam *b, int slot) {
  if (!b->save_loss[slot]) return -1;
  upload(b, b->save[slot][0], b->save[slot][1], b->save[slot][2], b->save[slot][3],
         b->save[slot][4], b->save[slot][5], b->save_loss[slot], b->save_lloss[slot]);
  b->design_w = b->save_design_w[slot];
  b->freq = b->save_freq[slot];
  b->current = b->save_current[slot];
  orc_beam_update_avg(b, HPS_COORD_PHI, 1);
  orc_beam_update_relative_phi(b, 1);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Reductions and finalisers: src/beam/src/beam.cu:411-1255,           */
/* src/beam/inc/beam_kernel.cu:86-1446                                 */
/* ------------------------------------------------------------------ */

/* count of loss != 0 (LossReduceKernel, beam_kernel.cu:272-347) */
static uint32_t count_nonzero(const uint32_t *a, uint32_t n) {
  uint64_t part[ORC_NCHUNK];
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ORC_NCHUNK; ++c) {
    uint64_t s = 0;
    for (uint64_t i = chunk_lo(n, c); i < chunk_lo(n, c + 1); ++i) s += (a[i] != 0);
    part[c] = s;
  }
  uint64_t t = 0;
  for (int c = 0; c < ORC_NCHUNK; ++c) t += part[c];
  return (uint32_t)t;
}

/* mask: 0 -> loss==0 ; 1 -> loss+lloss==0 (uint add, as XReduceKernel) */
static inline int keep(const orc_beam *b, uint64_t i, int good) {
  uint32_t l = b->loss[i];
  if (good) l += b->lloss[i];
  return l == 0;
}

/* Masked sums of up to five products; kind selects the terms:
 *   1: sum a                 2: sum a, sum a^2
 *   4: sum a, a^2, c, c^2    5: sum a, a^2, c, c^2, a*c */
static void masked_sums(const orc_beam *b, const double *a, const double *c2,
                        int good, int kind, double out[5]) {
  double part[ORC_NCHUNK][5];
  uint32_t n = b->n;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ORC_NCHUNK; ++c) {
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
    for (uint64_t i = chunk_lo(n, c); i < chunk_lo(n, c + 1); ++i) {
      if (!keep(b, i, good)) continue;
      double u = a[i];
      s0 += u;
      if (kind >= 2) s1 += u * u;
      if (kind >= 4) { double v = c2[i]; s2 += v; s3 += v * v; if (kind >= 5) s4 += u * v; }
    }
    part[c][0] = s0; part[c][1] = s1; part[c][2] = s2; part[c][3] = s3; part[c][4] = s4;
  }
  for (int k = 0; k < 5; ++k) out[k] = 0.0;
  for (int c = 0; c < ORC_NCHUNK; ++c)
    for (int k = 0; k < 5; ++k) out[k] += part[c][k];
}

/* Beam::UpdateLoss -> UpdateLossCountKernelCall, beam.cu:493-516 */
void orc_beam_update_loss(orc_beam *b) { b->num_loss = count_nonzero(b->loss, b->n); }

/* UpdateGoodParticleCountKernelCall, beam.cu:1233-1255 */
void orc_beam_update_good_count(orc_beam *b) {
  uint64_t part[ORC_NCHUNK];
  uint32_t n = b->n;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ORC_NCHUNK; ++c) {
    uint64_t s = 0;
    for (uint64_t i = chunk_lo(n, c); i < chunk_lo(n, c + 1); ++i)
      s += ((uint32_t)(b->loss[i] + b->lloss[i]) == 0);
    part[c] = s;
  }
  uint64_t t = 0;
  for (int c = 0; c < ORC_NCHUNK; ++c) t += part[c];
  b->num_good = (uint32_t)t;
}

static int avg_slot(int coord, int good) {
  switch (coord) {
    case HPS_COORD_X: return good ? ORC_X_AVG_GOOD : ORC_X_AVG;
    case HPS_COORD_XP: return ORC_XP_AVG;
    case HPS_COORD_Y: return good ? ORC_Y_AVG_GOOD : ORC_Y_AVG;
    case HPS_COORD_YP: return ORC_YP_AVG;
    case HPS_COORD_PHI: return good ? ORC_PHI_AVG_GOOD : ORC_PHI_AVG;
    case HPS_COORD_W: return good ? ORC_W_AVG_GOOD : ORC_W_AVG;
    default: return ORC_PHI_AVG_R;
  }
}

/* UpdateAvgOfOneVariableKernelCall, beam.cu:411-436, with the finalisers
 * UpdateVariableAvgKernel (beam_kernel.cu:1413-1418: divides by
 * num - num_loss, num_loss being whatever the last UpdateLoss left) and
 * UpdateVariableAvgWithLlossKernel (beam_kernel.cu:1420-1426). */
static void avg_into(orc_beam *b, const double *v, int good, double *dst) {
  double s[5];
  masked_sums(b, v, NULL, good, 1, s);
  if (!good) {
    double surv = (double)(uint32_t)(b->n - b->num_loss);
    *dst = s[0] / surv;
  } else {
    if (b->num_good > 0) *dst = s[0] / b->num_good;
    else *dst = -99999;
  }
}

/* UpdateSigmaOfOneVariableKernelCall, beam.cu:651-678 with finalisers
 * beam_kernel.cu:1428-1446 */
static void sig_into(orc_beam *b, const double *v, int good, double *dst) {
  double s[5];
  masked_sums(b, v, NULL, good, 2, s);
  if (!good) {
    double surv = (double)(uint32_t)(b->n - b->num_loss);
    double avg = s[0] / surv, avg2 = s[1] / surv;
    *dst = sqrt(avg2 - avg * avg);
  } else {
    double avg = s[0] / b->num_good, avg2 = s[1] / b->num_good;
    *dst = sqrt(avg2 - avg * avg);
  }
}

/* Beam::UpdateAvg{X,Y,Phi,W,Xp,Yp,RelativePhi}, beam.cpp:796-882 */
void orc_beam_update_avg(orc_beam *b, int coord, int good_only) {
  int good = good_only;
  if (coord == HPS_COORD_XP || coord == HPS_COORD_YP) good = 0;
  avg_into(b, coord_ptr(b, coord), good, &b->st[avg_slot(coord, good)]);
}

/* Beam::UpdateSig{X,Y,Phi,RelativePhi,W,Xp,Yp}, beam.cpp:887-971.  Note the
 * good-only relative-phase sigma lands in phi_sig_good (beam.cpp:953). */
void orc_beam_update_sig(orc_beam *b, int coord, int good_only) {
  if (b->n <= 2) return;
  int slot;
  int good = good_only;
  switch (coord) {
    case HPS_COORD_X: slot = good ? ORC_X_SIG_GOOD : ORC_X_SIG; break;
    case HPS_COORD_XP: slot = ORC_XP_SIG; good = 0; break;
    case HPS_COORD_Y: slot = good ? ORC_Y_SIG_GOOD : ORC_Y_SIG; break;
    case HPS_COORD_YP: slot = ORC_YP_SIG; good = 0; break;
    case HPS_COORD_PHI: slot = ORC_PHI_SIG; good = 0; break;
    case HPS_COORD_W: slot = good ? ORC_W_SIG_GOOD : ORC_W_SIG; break;
    default: slot = good ? ORC_PHI_SIG_GOOD : ORC_PHI_SIG_R; break;
  }
  sig_into(b, coord_ptr(b, coord), good, &b->st[slot]);
}

/* UpdateRelativePhiKernel, beam_kernel.cu:1507-1525 (all particles) */
void orc_beam_update_relative_phi(orc_beam *b, int use_good) {
  uint32_t n = b->n;
  if (!n) return;
  double ref = use_good ? b->st[ORC_PHI_AVG_GOOD] : b->phi[0];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    double tmp = b->phi[i] - ref + PI;
    double sign = 1.0;
    if (tmp < 0) { sign = -1.0; tmp = -tmp; }
    b->phi_r[i] = sign * (fmod(tmp, TWOPI) - PI);
  }
}

/* Beam::UpdateLongitudinalLoss, beam.cpp:776-782; lloss kernel
 * beam_kernel.cu:1550-1559 */
void orc_beam_update_longitudinal_loss(orc_beam *b) {
  orc_beam_update_good_count(b);
  orc_beam_update_avg(b, HPS_COORD_PHI, 1);
  double lim = b->st[ORC_PHI_AVG_GOOD];
  uint32_t n = b->n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    if (b->phi[i] > lim + TWOPI + PI) b->lloss[i] = 1;
  b->num_lloss = count_nonzero(b->lloss, n);
}

/* UpdateAvgSigXYKernelCall, beam.cu:919-939; finaliser
 * UpdateHorizontalAvgSigKernel beam_kernel.cu:1397-1411 divides the
 * good-particle sums by num - num_loss. */
static void update_avg_sig_xy(orc_beam *b) {
  double s[5];
  masked_sums(b, b->x, b->y, 1, 4, s);
  double surv = (double)(uint32_t)(b->n - b->num_loss);
  double xavg = s[0] / surv, x2avg = s[1] / surv, yavg = s[2] / surv, y2avg = s[3] / surv;
  b->st[ORC_X_AVG_GOOD] = xavg;
  b->st[ORC_X_SIG_GOOD] = sqrt(x2avg - xavg * xavg);
  b->st[ORC_Y_AVG_GOOD] = yavg;
  b->st[ORC_Y_SIG_GOOD] = sqrt(y2avg - yavg * yavg);
}

/* UpdateAvgXYKernelCall, beam.cu:739-761; UpdateHorizontalAvgXYKernel
 * beam_kernel.cu:1386-1395 */
void orc_beam_update_avg_xy(orc_beam *b) {
  double s[5];
  masked_sums(b, b->x, b->y, 0, 4, s);
  double surv = (double)(uint32_t)(b->n - b->num_loss);
  b->st[ORC_X_AVG] = s[0] / surv;
  b->st[ORC_Y_AVG] = s[2] / surv;
}

/* UpdateMaxRPhiKernelCall, beam.cu:829-852; MaxR2PhiReduceKernel
 * beam_kernel.cu:794-931 (loss==0, relative to x_avg, y_avg, phi_avg_r) */
void orc_beam_update_max_r_phi(orc_beam *b) {
  double xa = b->st[ORC_X_AVG], ya = b->st[ORC_Y_AVG], pa = b->st[ORC_PHI_AVG_R];
  double r2max = 0, phimax = 0;
  for (uint32_t i = 0; i < b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double tx = b->x[i] - xa, ty = b->y[i] - ya;
    double r2 = tx * tx + ty * ty;
    double tp = b->phi_r[i] - pa;
    tp = tp > 0.0 ? tp : -tp;
    r2max = r2max < r2 ? r2 : r2max;
    phimax = phimax < tp ? tp : phimax;
  }
  b->st[ORC_R_MAX] = sqrt(r2max);
  b->st[ORC_ABS_PHI_MAX] = phimax;
}

/* transverse emittance finaliser, beam_kernel.cu:1334-1355 */
static void transverse_emit(orc_beam *b, const double *u, const double *up,
                            int s_avg, int s_sig, int s_pavg, int s_psig, int s_emit) {
  double s[5];
  masked_sums(b, u, up, 0, 5, s);
  double surv = (double)(uint32_t)(b->n - b->num_loss);
  double x = s[0] / surv, x2 = s[1] / surv, xp = s[2] / surv, xp2 = s[3] / surv,
         xxp = s[4] / surv;
  double gamma1 = b->w[0] / b->mass;
  double bg = sqrt(gamma1 * (gamma1 + 2.0));
  b->st[s_avg] = x;
  b->st[s_sig] = sqrt(x2 - x * x);
  b->st[s_pavg] = xp;
  b->st[s_psig] = sqrt(xp2 - xp * xp);
  b->st[s_emit] = sqrt((x2 - x * x) * (xp2 - xp * xp) - (xxp - x * xp) * (xxp - x * xp)) * bg;
}

/* Beam::UpdateEmittance, beam.cpp:985-995; kernels beam.cu:1007-1092 and
 * beam_kernel.cu:1334-1376 */
void orc_beam_update_emittance(orc_beam *b) {
  if (b->n <= 2) return;
  transverse_emit(b, b->x, b->xp, ORC_X_AVG, ORC_X_SIG, ORC_XP_AVG, ORC_XP_SIG, ORC_X_EMIT);
  transverse_emit(b, b->y, b->yp, ORC_Y_AVG, ORC_Y_SIG, ORC_YP_AVG, ORC_YP_SIG, ORC_Y_EMIT);
  orc_beam_update_relative_phi(b, 0);
  double s[5];
  masked_sums(b, b->phi_r, b->w, 0, 5, s);
  double surv = (double)(uint32_t)(b->n - b->num_loss);
  double phi = s[0] / surv, phi2 = s[1] / surv, w = s[2] / surv, w2 = s[3] / surv,
         phiw = s[4] / surv;
  double pv = phi2 - phi * phi, wv = w2 - w * w, cv = phiw - phi * w;
  b->st[ORC_PHI_AVG_R] = phi;
  b->st[ORC_W_AVG] = w;
  b->st[ORC_PHI_SIG_R] = sqrt(pv);
  b->st[ORC_W_SIG] = sqrt(wv);
  b->st[ORC_Z_EMIT] = sqrt(pv * wv - cv * cv);
}

/* Beam::UpdateStatForSpaceCharge, beam.cpp:1003-1016 */
void orc_beam_update_stat_for_sc(orc_beam *b) {
  if (b->n <= 2) return;
  orc_beam_update_longitudinal_loss(b);
  orc_beam_update_good_count(b);
  orc_beam_update_avg(b, HPS_COORD_PHI, 1);
  orc_beam_update_relative_phi(b, 1);
  avg_into(b, b->phi_r, 0, &b->st[ORC_PHI_AVG_R]);
  orc_beam_update_sig(b, HPS_COORD_PHI_R, 1);
  update_avg_sig_xy(b);
  orc_beam_update_avg(b, HPS_COORD_W, 1);
}

/* Beam::ChangeFrequency, beam.cpp:1658-1669 (ChangeFrequencyKernel
 * beam_kernel.cu:1532-1538 covers every particle) */
void orc_beam_change_frequency(orc_beam *b, double f) {
  b->current *= f / b->freq;
  double ratio = f / b->freq;
  for (uint32_t i = 0; i < b->n; ++i) b->phi[i] *= ratio;
  b->freq = f;
  orc_beam_update_avg(b, HPS_COORD_PHI, 0);
  orc_beam_update_relative_phi(b, 0);
  avg_into(b, b->phi_r, 0, &b->st[ORC_PHI_AVG_R]);
}

/* Beam::ApplyCut + CutBeamKernel, beam.cpp:1574-1587, beam_kernel.cu:1465-1481
 * (index 0 is skipped; a particle strictly inside (min,max) is marked) */
void orc_beam_apply_cut(orc_beam *b, char coord, double lo, double hi) {
  char c = (char)((coord >= 'A' && coord <= 'Z') ? coord + 32 : coord);
  double *v = NULL;
  if (c == 'x') v = b->x;
  if (c == 'y') v = b->y;
  if (c == 'w') v = b->w;
  if (c == 'p') v = b->phi;
  if (!v) return;
  for (uint32_t i = 1; i < b->n; ++i)
    if (b->loss[i] == 0 && v[i] < hi && v[i] > lo) b->loss[i] = 99999;
}

/* Beam::Shift* + ShiftVariableKernel, beam.cpp:1594-1648,
 * beam_kernel.cu:1491-1497 (index 0 is not shifted) */
void orc_beam_shift(orc_beam *b, int coord, double val) {
  double *v = coord_ptr(b, coord);
  for (uint32_t i = 1; i < b->n; ++i) v[i] += val;
  if (coord == HPS_COORD_PHI) init_phi_avg_good(b);
}

/* Side-effect-free statistics: what get_emittance_x() & co. report right
 * after UpdateLoss (wrap_beam.cpp:1188-1240); phi_r relative to particle 0. */
void orc_beam_monitor(const orc_beam *b, double *out) {
  uint32_t n = b->n;
  for (int k = 0; k < HPS_NMON; ++k) out[k] = 0.0;
  if (!n) return;
  double part[ORC_NCHUNK][17];
  double ref = b->phi[0];
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ORC_NCHUNK; ++c) {
    double s[17] = {0};
    for (uint64_t i = chunk_lo(n, c); i < chunk_lo(n, c + 1); ++i) {
      if ((uint32_t)(b->loss[i] + b->lloss[i]) == 0) s[16] += 1.0;
      if (b->loss[i] != 0) continue;
      double tmp = b->phi[i] - ref + PI, sign = 1.0;
      if (tmp < 0) { sign = -1.0; tmp = -tmp; }
      double pr = sign * (fmod(tmp, TWOPI) - PI);
      double x = b->x[i], xp = b->xp[i], y = b->y[i], yp = b->yp[i], w = b->w[i];
      s[0] += 1.0;
      s[1] += x; s[2] += x * x; s[3] += xp; s[4] += xp * xp; s[5] += x * xp;
      s[6] += y; s[7] += y * y; s[8] += yp; s[9] += yp * yp; s[10] += y * yp;
      s[11] += pr; s[12] += pr * pr; s[13] += w; s[14] += w * w; s[15] += pr * w;
    }
    for (int k = 0; k < 17; ++k) part[c][k] = s[k];
  }
  double s[17] = {0};
  for (int c = 0; c < ORC_NCHUNK; ++c)
    for (int k = 0; k < 17; ++k) s[k] += part[c][k];
  double m = s[0];
  out[HPS_MON_NALIVE] = m;
  out[HPS_MON_NGOOD] = s[16];
  double g1 = b->w[0] / b->mass, bg = sqrt(g1 * (g1 + 2.0));
  if (m > 0) {
    for (int pl = 0; pl < 2; ++pl) {
      const double *q = s + 1 + 5 * pl;
      double a = q[0] / m, a2 = q[1] / m, ap = q[2] / m, ap2 = q[3] / m, aap = q[4] / m;
      int base = pl ? HPS_MON_Y_AVG : HPS_MON_X_AVG;
      out[base + 0] = a;
      out[base + 1] = sqrt(a2 - a * a);
      out[base + 2] = ap;
      out[base + 3] = sqrt(ap2 - ap * ap);
      out[base + 4] = sqrt((a2 - a * a) * (ap2 - ap * ap) - (aap - a * ap) * (aap - a * ap)) * bg;
    }
    double p = s[11] / m, p2 = s[12] / m, w = s[13] / m, w2 = s[14] / m, pw = s[15] / m;
    double pv = p2 - p * p, wv = w2 - w * w, cv = pw - p * w;
    out[HPS_MON_PHIR_AVG] = p;
    out[HPS_MON_PHIR_SIG] = sqrt(pv);
    out[HPS_MON_W_AVG] = w;
    out[HPS_MON_W_SIG] = sqrt(wv);
    out[HPS_MON_Z_EMIT] = sqrt(pv * wv - cv * cv);
  }
  out[HPS_MON_W0] = b->w[0];
  out[HPS_MON_PHI0] = b->phi[0];
}

/* ------------------------------------------------------------------ */
/* SCHEFF: src/simulation/src/space_charge.{cpp,cu},                    */
/*         src/simulation/inc/space_charge_kernel.cu                    */
/* ------------------------------------------------------------------ */

/* Initialize, space_charge.cu:27-60: tables allocated and zeroed */
static void scheff_alloc(orc_scheff *s) {
  free(s->bin); free(s->fld1); free(s->fld2);
  s->bin = (double *)calloc((size_t)s->nx * s->nz, sizeof(double));
  s->fld1 = (double *)calloc((size_t)(s->nx + 1) * s->nx * s->nz * 2, sizeof(double));
  s->fld2 = (double *)calloc((size_t)(s->nz + 1) * (s->nx + 1) * 2, sizeof(double));
}

/* SpaceCharge::SpaceCharge + Scheff::Scheff, space_charge.cpp:13-40 */
orc_scheff *orc_scheff_create(uint32_t nr, uint32_t nz, uint32_t adj_bunch) {
  orc_scheff *s = (orc_scheff *)calloc(1, sizeof(orc_scheff));
  s->nx = nr; s->nz = nz; s->nx_init = nr; s->nz_init = nz;
  s->adj_bunch = adj_bunch; s->fraction = 1.0; s->interval = 0.01;
  s->interval_init = 0.01; s->adj_bunch_w = 0.0; s->mesh_w = 0.0;
  s->remesh_val = 0.05;
  scheff_alloc(s);
  return s;
}

void orc_scheff_free(orc_scheff *s) {
  if (!s) return;
  free(s->bin); free(s->fld1); free(s->fld2); free(s);
}

/* SpaceCharge::SetInterval, space_charge.h:59-63 */
void orc_scheff_set_interval(orc_scheff *s, double v) { s->interval = v; s->interval_init = v; }

/* Scheff::SetMeshSize, space_charge.cpp:61-73 */
void orc_scheff_set_mesh_size(orc_scheff *s, uint32_t nr, uint32_t nz) {
  if (nr != s->nx || nz != s->nz) {
    s->nx = nr; s->nz = nz;
    scheff_alloc(s);
  }
}

/* UpdateFldTbl1Kernel, space_charge_kernel.cu:39-100.  Launch geometry of
 * UpdateTblsKernelCall (space_charge.cu:160-170): block (nz, by),
 * grid (nr/by, nr+1), by = min(512/nz, nr); rows rs >= (nr/by)*by are not
 * written by the reference and are left untouched here too. */
void orc_scheff_green_table(orc_scheff *s, double r_beta, double r_freq,
                            uint32_t r_num_part, double r_current_ov_mc2,
                            uint32_t r_adj_bunch) {
  uint32_t nr = s->nx, nz = s->nz;
  uint32_t by = (512 / nz < nr) ? 512 / nz : nr;
  uint32_t gx = by ? nr / by : 0;
  uint32_t nrs = gx * by;
  double gm = 1.0 / sqrt(1.0 - r_beta * r_beta);
  double dr = s->dr;
  double dzg = s->dz * gm;
  double wave_len = CLIGHT / r_freq;
  double pl = r_beta * gm * wave_len;
  double c1 = 5721.67 * r_current_ov_mc2 / (r_freq * 1e6 * (double)r_num_part);
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t rpi = 0; rpi <= (int64_t)nr; ++rpi)
    for (int64_t k = 0; k < (int64_t)nrs; ++k) {
      for (uint32_t tz = 0; tz < nz; ++tz) {
        double rs = sqrt(0.5 * (double)(k * k + (k + 1) * (k + 1))) * dr;
        double zs = 0.5 * dzg;
        double zp = (tz + 1) * dzg;
        double rp = rpi * dr;
        size_t cnt = (size_t)rpi * nr * nz + (size_t)k * nz + tz;
        double d = zp - zs;
        double d2 = d * d;
        double c = (rp - rs) * (rp - rs);
        double b = (rp + rs) * (rp + rs);
        double rsrp = rs * rp;
        double a = 4.0 * rsrp / (b + d2);
        double g = 1.0 - a;
        double h = log(g);
        double ee = 1.0 + g * (0.4630106 - 0.2452740 * h + g * (0.1077857 - 0.04125321 * h));
        double ek = 1.38629436 - 0.5 * h + g * (0.1119697 - 0.1213486 * h + g * (0.07253230 - 0.02887472 * h));
        double er1 = 0.0;
        a = sqrt(b + d2);
        double rs2mrp2 = (rs * rs - rp * rp);
        if (rp != 0.0) er1 = (ek - (rs2mrp2 + d2) * ee / (c + d2)) / (2.0 * rp * a);
        double ez1 = d * ee / (a * (c + d2));
        for (uint32_t i = 1; i <= r_adj_bunch; ++i) {
          double xi = i;
          for (int j = 0; j < 2; ++j) {
            double d1 = d - xi * pl;
            d2 = d1 * d1;
            a = 4.0 * rsrp / (b + d2);
            g = 1.0 - a;
            h = log(g);
            ee = 1.0 + g * (0.4630106 - 0.2452740 * h + g * (0.1077857 - 0.04125321 * h));
            ek = 1.38629436 - 0.5 * h + g * (0.1119697 - 0.1213486 * h + g * (0.07253230 - 0.02887472 * h));
            a = sqrt(b + d2);
            if (rp != 0.0) er1 += (ek - (rs2mrp2 + d2) * ee / (c + d2)) / (2.0 * rp * a);
            ez1 += d1 * ee / (a * (c + d2));
            xi = -xi;
          }
        }
        s->fld1[2 * cnt] = c1 * er1;
        s->fld1[2 * cnt + 1] = c1 * ez1;
      }
    }
}

/* DistributeParticleKernel, space_charge_kernel.cu:123-224 (every particle
 * with loss == 0 && lloss == 0, including particle 0) */
void orc_scheff_deposit(orc_scheff *s, const orc_beam *bm, double r_beta, double r_freq) {
  uint32_t nx = s->nx, nz = s->nz, n = bm->n;
  size_t nb = (size_t)nx * nz;
  double *priv = (double *)calloc((size_t)ORC_NCHUNK * nb, sizeof(double));
  uint32_t onm[ORC_NCHUNK];
  double phimc = bm->st[ORC_PHI_AVG_R], xbar = bm->st[ORC_X_AVG_GOOD],
         ybar = bm->st[ORC_Y_AVG_GOOD];
  double epsq = bm->st[ORC_X_SIG_GOOD] / bm->st[ORC_Y_SIG_GOOD];
  double gm = 1.0 / sqrt(1.0 - r_beta * r_beta);
  double dr = s->dr;
  double dzg = s->dz * gm;
  double wave_len = CLIGHT / r_freq;
  double hl = nz * 0.5 * dzg;
  double c2 = r_beta * gm * wave_len / TWOPI;
#pragma omp parallel for schedule(static)
  for (int ch = 0; ch < ORC_NCHUNK; ++ch) {
    double *bin = priv + (size_t)ch * nb;
    uint32_t cnt = 0;
    for (uint64_t np = chunk_lo(n, ch); np < chunk_lo(n, ch + 1); ++np) {
      if (!(bm->loss[np] == 0 && bm->lloss[np] == 0)) continue;
      double x = bm->x[np], y = bm->y[np], z = bm->phi_r[np];
      double a, cc, rminsq, rmaxsq, bb, d;
      int i, jm1, i1, j1, k;
      double rsq_sh = (x - xbar) * (x - xbar) / epsq + (y - ybar) * (y - ybar) * epsq;
      i = (int)(sqrt(rsq_sh) / dr + 1);
      /* the reference compares int i with uint nx; i < 1 only arises from
       * NaN statistics and would index before the table */
      if (i >= 1 && (uint32_t)i <= nx) {
        double ddz = z - phimc;
        while (ddz > PI || ddz < -PI) {
          if (ddz > 0.0) ddz -= TWOPI;
          else ddz += TWOPI;
        }
        z = -c2 * ddz;
        if (fabs(z) < hl) {
          double zz = z + hl;
          jm1 = (int)(zz / dzg + 1);
          i1 = i + 1;
          double drdr = dr * dr;
          if (rsq_sh < 0.5 * drdr * (double)(i * i + (i - 1) * (i - 1))) i1 = i - 1;
          if (i1 < 1) i1 = 1;
          if (i1 > (int)nx) i1 = nx;
          j1 = jm1 + 1;
          if (zz < (jm1 - 1 + 0.5) * dzg) j1 = jm1 - 1;
          if (j1 < 1) j1 = 1;
          if (j1 > (int)nz) j1 = nz;
          if (i1 == i) a = 1.0;
          else {
            double sqrtmp = sqrt(4.0 * rsq_sh / drdr - 1.0);
            rminsq = 0.25 * drdr * (sqrtmp - 1.0) * (sqrtmp - 1.0);
            rmaxsq = rminsq + sqrtmp * drdr;
            if (i1 < i) a = (rmaxsq - (i - 1) * (i - 1) * drdr) / (rmaxsq - rminsq);
            else a = ((i1 - 1) * (i1 - 1) * drdr - rminsq) / (rmaxsq - rminsq);
          }
          cc = 1.0;
          if (j1 != jm1) cc = (zz - (j1 - 1 + 0.5) * dzg) / ((jm1 - j1) * dzg);
          bb = 1.0 - a;
          d = 1.0 - cc;
          k = (jm1 - 1) * nx + i;
          bin[k - 1] += a * cc;
          k += i1 - i;
          bin[k - 1] += bb * cc;
          k = (j1 - 1) * nx + i;
          bin[k - 1] += a * d;
          k += i1 - i;
          bin[k - 1] += bb * d;
          ++cnt;
        }
      }
    }
    onm[ch] = cnt;
  }
  uint32_t tot = 0;
  for (int ch = 0; ch < ORC_NCHUNK; ++ch) {
    const double *bin = priv + (size_t)ch * nb;
    for (size_t q = 0; q < nb; ++q) s->bin[q] += bin[q];
    tot += onm[ch];
  }
  s->num_on_mesh = tot;
  free(priv);
}

/* UpdateFldTbl2KernelDouble, space_charge_kernel.cu:472-568 launched as
 * <<<nr + 2, 1024>>> (space_charge.cu:203).  The bins a thread visits are
 * exactly those of the reference's partition, so bins the reference never
 * reads (remainders of the integer divisions) are skipped here too. */
void orc_scheff_contract(orc_scheff *s) {
  uint32_t nx = s->nx, nz = s->nz;
  uint32_t fld_sz = nx * nz;
  uint32_t nrow = nx + 1;
  /* blocks rp = 0..nx, zp = 0..nz-1 */
  uint32_t gnum = 1024 / nz;
  uint32_t gsz = gnum ? fld_sz / gnum : 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t rp = 0; rp <= (int64_t)nx; ++rp)
    for (int64_t zp = 0; zp < (int64_t)nz; ++zp) {
      double ax = 0.0, az = 0.0;
      for (uint32_t g = 0; g < gnum; ++g) {
        double tx = 0.0, tz = 0.0;
        for (uint32_t bi = g * gsz; bi < g * gsz + gsz; ++bi) {
          double bv = s->bin[bi];
          if (bv == 0.0) continue;
          uint32_t rs = bi % nx, zs = bi / nx;
          double sign = 1.0;
          uint32_t dz;
          if (zs >= (uint32_t)zp) { dz = zs - zp; sign = -1.0; }
          else dz = zp - zs - 1;
          size_t f1 = dz + (size_t)rs * nz + (size_t)rp * fld_sz;
          tx += bv * s->fld1[2 * f1];
          tz += sign * bv * s->fld1[2 * f1 + 1];
        }
        ax += tx; az += tz;
      }
      size_t o = (size_t)zp * nrow + rp;
      s->fld2[2 * o] += ax;
      s->fld2[2 * o + 1] += az;
    }
  /* last block: zp = nz, rp = 0..nx-1 */
  uint32_t gnum2 = 1024 / nx;
  uint32_t gsz2 = gnum2 ? fld_sz / gnum2 : 0;
  for (uint32_t rp = 0; rp < nx; ++rp) {
    double ax = 0.0, az = 0.0;
    for (uint32_t g = 0; g < gnum2; ++g) {
      double tx = 0.0, tz = 0.0;
      for (uint32_t bi = g * gsz2; bi < g * gsz2 + gsz2; ++bi) {
        double bv = s->bin[bi];
        if (bv == 0.0) continue;
        uint32_t rs = bi % nx, zs = bi / nx;
        uint32_t dz = nz - zs - 1;
        size_t f1 = dz + (size_t)rs * nz + (size_t)fld_sz * rp;
        tx += bv * s->fld1[2 * f1];
        tz += bv * s->fld1[2 * f1 + 1];
      }
      ax += tx; az += tz;
    }
    size_t o = (size_t)nz * nrow + rp;
    s->fld2[2 * o] += ax;
    s->fld2[2 * o + 1] += az;
  }
  /* the corner point (nz, nx): thread t sums bins t + i*1024, i < fld_sz/1024 */
  {
    uint32_t cnt = fld_sz / 1024;
    double ax = 0.0, az = 0.0;
    for (uint32_t t = 0; t < 1024; ++t) {
      double tx = 0.0, tz = 0.0;
      for (uint32_t i = 0; i < cnt; ++i) {
        uint32_t bi = t + i * 1024;
        double bv = s->bin[bi];
        if (bv == 0.0) continue;
        uint32_t rs = bi % nx, zs = bi / nx;
        uint32_t dz = nz - zs - 1;
        size_t f1 = dz + (size_t)rs * nz + (size_t)fld_sz * nx;
        tx += bv * s->fld1[2 * f1];
        tz += bv * s->fld1[2 * f1 + 1];
      }
      ax += tx; az += tz;
    }
    size_t o = (size_t)nz * nrow + nx;
    s->fld2[2 * o] += ax;
    s->fld2[2 * o + 1] += az;
  }
}

/* ApplySpchKickKernel, space_charge_kernel.cu:573-706, launched by
 * KickBeamKernelCall (space_charge.cu:220-244) as
 * <<<grid_size, blck_size/4>>>.  The loop `while(indx > 0 && ...)` ends
 * thread 0 before its first particle, so every particle whose index is a
 * multiple of the launch's thread count is never kicked. */
static void scheff_kick(orc_scheff *s, orc_beam *bm, double r_length, double r_ratio_r,
                        double r_ratio_z, double r_ratio_q, double r_ratio_gm) {
  uint32_t n = bm->n;
  uint64_t stride = (uint64_t)bm->grid_size * (bm->blck_size / 4);
  if (stride == 0) return;
  uint32_t nx = s->nx, nz = s->nz;
  double r_beta = s->beta, r_freq = s->sc_freq, r_mass = bm->mass;
  double r_current = bm->current * s->frac;
  double phimc = bm->st[ORC_PHI_AVG_R], xbar = bm->st[ORC_X_AVG_GOOD],
         ybar = bm->st[ORC_Y_AVG_GOOD];
  double epsq = bm->st[ORC_X_SIG_GOOD] / bm->st[ORC_Y_SIG_GOOD];
  double gmg = 1.0 / sqrt(1.0 - r_beta * r_beta);
  double dr = s->dr * r_ratio_r;
  double dzg = s->dz * gmg * r_ratio_z;
  double wave_len = CLIGHT / r_freq;
  double hl = nz * 0.5 * dzg;
  double c1 = 5721.67 * r_current / (r_freq * 1e6 * (double)n * r_mass);
  double c2 = r_beta * gmg * wave_len / TWOPI;
  double c3 = r_length / (r_beta * gmg);
  double xfac = 2.0 / (epsq + 1.0);
  double yfac = epsq * xfac;
  uint32_t adj = s->adj_cur;
  uint32_t onm = s->num_on_mesh;
  uint32_t tbl_sz = (nx + 1) * (nz + 1);
  const double *fld = s->fld2;
#pragma omp parallel for schedule(static)
  for (int64_t ii = 1; ii < (int64_t)n; ++ii) {
    uint64_t indx = (uint64_t)ii;
    if (indx % stride == 0) continue;
    if (!(bm->loss[indx] == 0 && bm->lloss[indx] == 0)) continue;
    double x = bm->x[indx], y = bm->y[indx], xp = bm->xp[indx], yp = bm->yp[indx];
    double phi = bm->phi_r[indx], w = bm->w[indx];
    double bgx, bgy, bgzstar, gstar, xxbar, yybar, r, xovr, yovr, ddz, z, d, rod3, zod3,
        cbgr, cbgzs, a, bb, c, bgzf, er_ratio, ez_ratio;
    uint32_t i, j, l, m;
    double gm = w / r_mass + 1.0;
    double bgz = sqrt((gm - 1.0) * (gm + 1.0));
    bgx = bgz * xp;
    bgy = bgz * yp;
    bgzstar = gmg * (bgz - r_beta * gm);
    gstar = gmg * (gm - r_beta * bgz);
    (void)gstar;
    xxbar = x - xbar;
    yybar = y - ybar;
    r = sqrt(xxbar * xxbar / epsq + yybar * yybar * epsq);
    if (r == 0.0) r = 1.0e-8;
    xovr = xxbar * xfac / r;
    yovr = yybar * yfac / r;
    ddz = phi - phimc;
    while (ddz > PI || ddz < -PI) {
      if (ddz > 0.0) ddz -= TWOPI;
      else ddz += TWOPI;
    }
    z = -c2 * ddz;
    if (r > nx * dr || fabs(z) > hl) {
      z = -c2 * (phi - phimc);
      d = sqrt(z * z + r * r);
      double invd3 = 1.0 / (d * d * d);
      rod3 = r * invd3;
      zod3 = z * invd3;
      double pl = r_beta * gmg * wave_len;
      for (uint32_t nb = 1; nb <= adj; ++nb) {
        int xi = (int)nb;
        for (int lr = 1; lr <= 2; ++lr) {
          double sft = z + xi * pl;
          d = sqrt(sft * sft + r * r);
          invd3 = 1.0 / (d * d * d);
          rod3 += r * invd3;
          zod3 += sft * invd3;
          xi = -xi;
        }
      }
      double cbgcoef = c1 * c3 * PI * 0.5 * onm;
      cbgr = cbgcoef * rod3;
      cbgzs = cbgcoef * zod3;
    } else {
      i = 1 + (int)(r / dr);
      a = r / dr - (i - 1.0);
      bb = 1.0 - a;
      j = 1 + (int)((z + hl) / dzg);
      c = (z + hl) / dzg - (j - 1.0);
      d = 1.0 - c;
      l = (j - 1) * (nx + 1) + i;
      m = l + (nx + 1);
      if (m >= tbl_sz) m = tbl_sz - 1;
      /* l can only leave the table for r == nx*dr and z == hl together, or
       * for NaN coordinates; the reference then reads outside the table */
      if (l >= tbl_sz || l < 1) l = tbl_sz - 1;
      if (m < 1) m = 1;
      er_ratio = r_ratio_q / (r_ratio_r * r_ratio_z * r_ratio_gm * r_ratio_gm);
      ez_ratio = r_ratio_q / (r_ratio_z * r_ratio_z);
      cbgr = er_ratio * c3 * (d * (a * fld[2 * l] + bb * fld[2 * (l - 1)]) +
                              c * (a * fld[2 * m] + bb * fld[2 * (m - 1)]));
      cbgzs = ez_ratio * c3 * (d * (a * fld[2 * l + 1] + bb * fld[2 * (l - 1) + 1]) +
                               c * (a * fld[2 * m + 1] + bb * fld[2 * (m - 1) + 1]));
    }
    bgx += cbgr * xovr;
    bgy += cbgr * yovr;
    bgzstar += cbgzs;
    gstar = 1.0 + 0.5 * bgzstar * bgzstar;
    bgzf = gmg * (bgzstar + r_beta * gstar);
    if (bgzf <= 0.0) bm->loss[indx] = 9999;
    else {
      bm->xp[indx] = bgx / bgzf;
      bm->yp[indx] = bgy / bgzf;
      bm->w[indx] *= 1.0 + (gm + 1.0) * (bgzf - bgz) / (gm * bgz);
    }
  }
}

/* UpdateScheffMeshSizeKernel, space_charge_kernel.cu:18-32 */
static void mesh_size(orc_scheff *s, double partial_r, double partial_z, double r_freq,
                      double r_beta, double r_coef) {
  double bl = r_beta * CLIGHT / r_freq;
  s->dr = r_coef * partial_r / s->nx;
  if (r_coef == 1.0) s->dz = bl / s->nz;
  else {
    if (partial_z * r_coef > PI) s->dz = bl / s->nz;
    s->dz = r_coef * bl * partial_z / (s->nz * PI);
  }
}

/* Scheff::Start, space_charge.cpp:82-139 (with the launcher glue of
 * space_charge.cu:77-244) */
void orc_scheff_start(orc_scheff *s, orc_beam *b, double r_length) {
  orc_beam_update_stat_for_sc(b);
  uint32_t good_cnt = b->num_good;
  double sigphi = b->n < 2 ? 0.0 : b->st[ORC_PHI_SIG_GOOD];
  double sigx = b->n < 2 ? 0.0 : b->st[ORC_X_SIG_GOOD];
  double sigy = b->n < 2 ? 0.0 : b->st[ORC_Y_SIG_GOOD];
  double ke = b->st[ORC_W_AVG_GOOD];
  double gamma = (double)ke / b->mass + 1.0;
  double beta = sqrt(1.0 - 1.0 / (gamma * gamma));
  double lmbd = 299.792458 / b->freq;
  double sigz = sigphi * 0.5 / 3.14159265 * beta * lmbd;
  double sigr = sqrt(sigx * sigx + sigy * sigy);
  double cratior = sigr * sigz;
  double cratioz = sigz * sigz * gamma * gamma;
  double cratior_old = s->sigr_old * s->sigz_old;
  double cratioz_old = s->sigz_old * s->sigz_old * s->gm_old * s->gm_old;
  uint32_t adj;
  if (s->adj_bunch_w == 0.0 || ke < s->adj_bunch_w) adj = s->adj_bunch;
  else adj = 0;
  if (s->mesh_w != 0.0) {
    if (ke > s->mesh_w && (s->nx != s->nx_init / 2 || s->nz != s->nz_init / 2))
      orc_scheff_set_mesh_size(s, s->nx_init / 2, s->nz_init / 2);
    else if (ke <= s->mesh_w && (s->nx != s->nx_init || s->nz != s->nz_init))
      orc_scheff_set_mesh_size(s, s->nx_init, s->nz_init);
    if (ke > s->mesh_w && s->interval != s->interval_init * 4)
      s->interval = s->interval_init * 4;
    else if (ke <= s->mesh_w && s->interval != s->interval_init)
      s->interval = s->interval_init;
  }
  /* SetParameters, space_charge.cu:77-86 */
  s->sc_freq = b->freq; s->beta = beta; s->frac = s->fraction; s->adj_cur = adj;

  if (cratior_old == 0.0 || cratioz_old == 0.0 ||
      fabs(cratior - cratior_old) / cratior_old > s->remesh_val ||
      fabs(cratioz - cratioz_old) / cratioz_old > s->remesh_val) {
    s->sigr_old = sigr; s->sigz_old = sigz; s->gm_old = gamma; s->good_cnt_old = good_cnt;
    memset(s->bin, 0, (size_t)s->nx * s->nz * sizeof(double));
    memset(s->fld2, 0, (size_t)(s->nx + 1) * (s->nz + 1) * 2 * sizeof(double));
    /* UpdateMeshKernelCall, space_charge.cu:122-138.  The reference picks
     * the sigma by comparing the device *pointers* x_sig_good > y_sig_good;
     * x_sig_good is allocated first (beam.cu:51,54), so the y branch runs. */
    if (adj != 0) {
      orc_beam_update_max_r_phi(b);
      mesh_size(s, b->st[ORC_R_MAX], 0.0, s->sc_freq, s->beta, 1.0);
    } else {
      mesh_size(s, b->st[ORC_Y_SIG_GOOD], b->st[ORC_PHI_SIG_GOOD], s->sc_freq, s->beta, 3.0);
    }
    orc_scheff_green_table(s, s->beta, s->sc_freq, b->n, b->current * s->frac / b->mass, adj);
    s->num_on_mesh = 0;
    if (b->blck_size / 4 > 0) orc_scheff_deposit(s, b, s->beta, s->sc_freq);
    orc_scheff_contract(s);
    scheff_kick(s, b, r_length, 1, 1, 1, 1.0);
    s->n_solves++;
  } else {
    double rq = s->good_cnt_old ? (double)(good_cnt / s->good_cnt_old) : 0.0;
    scheff_kick(s, b, r_length, sigr / s->sigr_old, sigz / s->sigz_old, rq, gamma / s->gm_old);
  }
}

/* ------------------------------------------------------------------ */
/* Element transfer maps: src/simulation/inc/simulation_kernel.cu       */
/* ------------------------------------------------------------------ */

/* Bessi0c / Bessi1c / Bessi1p, simulation_kernel.cu:15-73 */
static double bessi0c(double r_x) {
  double ans, cy, ax = fabs(r_x);
  if (ax < 3.75) {
    cy = r_x / 3.75;
    cy = cy * cy;
    ans = 1.0 + cy * (3.5156229 + cy * (3.0899424 + cy * (1.2067492 + cy * (0.2659732 +
          cy * (0.360768e-1 + cy * 0.45813e-2)))));
  } else {
    cy = 3.75 / ax;
    ans = (exp(ax) * (1.0 / sqrt(ax))) * (0.39894228 + cy * (0.1328592e-1 + cy * (0.225319e-2 +
          cy * (-0.157565e-2 + cy * (0.916281e-2 + cy * (-0.2057706e-1 + cy * (0.2635537e-1 +
          cy * (-0.1647633e-1 + cy * 0.392377e-2))))))));
  }
  return ans;
}
static double bessi1c(double r_x) {
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
    ans = ans * (exp(ax) * (1.0 / sqrt(ax)));
  }
  return r_x < 0.0 ? -ans : ans;
}
static double bessi1p(double r_x) {
  if (r_x != 0.0) return bessi0c(r_x) - bessi1c(r_x) / r_x;
  return 0.5;
}

/* GetTransitTimeFactors, simulation_kernel.cu:290-308 */
static void transit_time_factors(double *t, double *tp, double *sp, double r_beta,
    double r_betag, double r_betamin, const double *ta /* t0..t5 */, const double *sa /* s1..s5 */) {
  double beta = r_beta;
  if (r_beta > 1.1 * r_betag) beta = r_betag;
  else if (r_beta < r_betamin) beta = r_betamin;
  *t = ta[0] + beta * (ta[1] + beta * (ta[2] + beta * (ta[3] + beta * (ta[4] + beta * ta[5]))));
  double coef = beta * beta / (TWOPI * r_betag);
  *tp = coef * (ta[1] + beta * (2 * ta[2] + beta * (3 * ta[3] + beta * (4 * ta[4] + 5 * beta * ta[5]))));
  *sp = -coef * (sa[0] + beta * (2 * sa[1] + beta * (3 * sa[2] + beta * (4 * sa[3] + 5 * beta * sa[4]))));
}

typedef struct {
  double length, frequency, clbl, amplitude, phase_ref, phase_shift, energy_out,
      beta_center, dg, t, tp, sp, fbc, fbm, ta[6], sa[5];
} rfgap_t;

static void load_gap(const double *p, rfgap_t *g) {
  g->length = p[HPS_P_LENGTH];
  g->frequency = p[HPS_P_RF_FREQ];
  g->clbl = p[HPS_P_RF_CLBL];
  g->amplitude = p[HPS_P_RF_AMP];
  g->phase_ref = p[HPS_P_RF_PHASE_REF];
  g->phase_shift = p[HPS_P_RF_PHASE_SHIFT];
  g->energy_out = p[HPS_P_RF_ENERGY_OUT];
  g->beta_center = p[HPS_P_RF_BETA_CENTER];
  g->dg = p[HPS_P_RF_DG];
  g->t = p[HPS_P_RF_T]; g->tp = p[HPS_P_RF_TP]; g->sp = p[HPS_P_RF_SP];
  g->fbc = p[HPS_P_RF_FIT_BETA_CENTER]; g->fbm = p[HPS_P_RF_FIT_BETA_MIN];
  for (int k = 0; k < 6; ++k) g->ta[k] = p[HPS_P_RF_FIT_T0 + k];
  for (int k = 0; k < 5; ++k) g->sa[k] = p[HPS_P_RF_FIT_S1 + k];
}

/* SimulatePartialDriftKernel, simulation_kernel.cu:86-118 */
static void k_partial_drift(orc_beam *b, double wl, double hf, double aper, uint32_t eid) {
  double mass = b->mass;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double aper2 = aper * aper;
    double x = b->x[i], y = b->y[i];
    x += b->xp[i] * hf;
    y += b->yp[i] * hf;
    if (aper2 != 0.0 && x * x + y * y > aper2) b->loss[i] = eid;
    else {
      b->x[i] = x; b->y[i] = y;
      double gm1 = b->w[i] / mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b->phi[i] += TWOPI * hf / (wl * bt);
    }
  }
}

/* SimulateSteererKernel, simulation_kernel.cu:120-140 */
static void k_steerer(orc_beam *b, double blh, double blv) {
  double mass = b->mass, charge = b->charge;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double gm1 = b->w[i] / mass;
    double btgm = sqrt(gm1 * (gm1 + 2.0));
    double p = btgm * mass / CLIGHT;
    if (blh > 1e-10) b->xp[i] += blh * charge / p;
    if (blv > 1e-10) b->yp[i] += blv * charge / p;
  }
}

/* SimulateHalfQuadKernel, simulation_kernel.cu:142-218 */
static void k_half_quad(orc_beam *b, double wl, double len, double aper, double grad, uint32_t eid) {
  double aper2 = aper * aper;
  double qg = grad * b->charge, mass = b->mass;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double x = b->x[i], y = b->y[i], xp = b->xp[i], yp = b->yp[i], w = b->w[i];
    if (qg == 0) {
      b->x[i] = x + xp * len * 0.5;
      b->y[i] = y + yp * len * 0.5;
    } else {
      double gamma1 = w / mass;
      double bg = sqrt(gamma1 * (gamma1 + 2.0) * (1.0 + xp * xp + yp * yp));
      double absqg = qg > 0.0 ? qg : -qg;
      double k = sqrt(absqg / (bg * mass) * CLIGHT);
      double inv_k = 1.0 / k;
      double kds = len * 0.25 * k;
      double s, c, sh = sinh(kds), ch = cosh(kds);
      sincos(kds, &s, &c);
      double xx, yy, sovk = s * inv_k, shovk = sh * inv_k, sk = s * k, shk = sh * k;
      for (int rep = 0; rep < 2; ++rep) {
        if (qg > 0.0) {
          xx = c * x + sovk * xp; xp = -sk * x + c * xp; x = xx;
          yy = ch * y + shovk * yp; yp = shk * y + ch * yp; y = yy;
        } else {
          xx = ch * x + shovk * xp; xp = shk * x + ch * xp; x = xx;
          yy = c * y + sovk * yp; yp = -sk * y + c * yp; y = yy;
        }
      }
      b->x[i] = x; b->y[i] = y; b->xp[i] = xp; b->yp[i] = yp;
    }
    if (aper2 != 0 && x * x + y * y > aper2) b->loss[i] = eid;
    else {
      double gm1 = w / mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b->phi[i] += TWOPI * len * 0.5 / (wl * bt);
    }
  }
}

/* SimulateRFGapFirstHalfKernel, simulation_kernel.cu:226-288 */
static void k_gap_first(orc_beam *b, double *wl, double design_w_in, double phi_in,
                        const rfgap_t *g, double len, double q1, double q2, int ccl) {
  double mass = b->mass;
  int any = 0;
  for (uint32_t i = 0; i < b->n; ++i) if (b->loss[i] == 0) { any = 1; break; }
  double wave_len = CLIGHT / g->frequency;
  if (any) *wl = wave_len; /* d_wavelen is written by every live particle */
  double dwl = *wl;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double x = b->x[i], y = b->y[i], xp = b->xp[i], yp = b->yp[i], phi = b->phi[i], w = b->w[i];
    double cell_len = len + q1 * 0.5 + q2 * 0.5;
    double dd1 = 0.5 * cell_len - g->dg - 0.5 * q1;
    b->x[i] = x + dd1 * xp;
    b->y[i] = y + dd1 * yp;
    if (g->amplitude == 0.0) {
      double gm1 = w / mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b->phi[i] += TWOPI * dd1 / (dwl * bt);
    } else {
      double gam = design_w_in / mass;
      double beta_in = sqrt((gam + 2.0) * gam) / (gam + 1.0);
      gam = w / mass;
      double beta = sqrt((gam + 2.0) * gam) / (gam + 1.0);
      if (!ccl) {
        double dps = g->phase_ref - phi_in;
        double d_cell_len = cell_len - g->beta_center * wave_len;
        double dphi_qlen1 = TWOPI * 0.5 * q1 / (beta * wave_len);
        double dphi_clen = 0.0;
        if (d_cell_len > 1e-15 || d_cell_len < -1e-15) dphi_clen = PI * d_cell_len / (beta * wave_len);
        b->phi[i] = phi + (1.0 - (beta - beta_in) / beta) * (PI * g->clbl + dps) + dphi_clen - dphi_qlen1;
      } else {
        double dps = g->phase_ref - phi_in;
        double betag = cell_len / (g->clbl * wave_len);
        b->phi[i] = phi + (1.0 - (beta - beta_in) * betag / (beta * beta_in)) * (PI * g->clbl + dps);
      }
    }
  }
}

/* SimulateRFGapSecondHalfKernel, simulation_kernel.cu:310-497 */
static void k_gap_second(orc_beam *b, double wl, double design_w_in, double phi_in,
                         const rfgap_t *g, double len, uint32_t ccl_cell_num,
                         double q1, double q2, int ccl) {
  double mass = b->mass, charge = b->charge;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double cell_len = len + q1 * 0.5 + q2 * 0.5;
    double dd2 = 0.5 * cell_len + g->dg - q2 * 0.5;
    double x = b->x[i], y = b->y[i], xp = b->xp[i], yp = b->yp[i];
    double inv_mass = 1.0 / mass;
    double phi = b->phi[i], w = b->w[i];
    double gm_in = design_w_in * inv_mass + 1.0;
    double beta_in = sqrt(1.0 - 1.0 / (gm_in * gm_in));
    double gam = w * inv_mass;
    double bg1 = sqrt(gam * (gam + 2.0));
    double beta = bg1 / (gam + 1.0);
    double t_fac = g->t, tp_fac = g->tp, sp_fac = g->sp;
    transit_time_factors(&t_fac, &tp_fac, &sp_fac, beta, g->fbc, g->fbm, g->ta, g->sa);
    if (g->amplitude == 0.0 || (ccl && beta < g->fbm)) {
      b->x[i] = x + dd2 * xp;
      b->y[i] = y + dd2 * yp;
      double gm1 = b->w[i] / mass;
      double bt = sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
      b->phi[i] += TWOPI * dd2 / (wl * bt);
      continue;
    }
    double wave_len = CLIGHT / g->frequency;
    double cl = cell_len / g->clbl;
    double betag_ccl = cl / wave_len;
    double betag = ccl ? g->beta_center : betag_ccl;
    double betag2 = betag * betag;
    double gmg = 1.0 / sqrt(1.0 - betag2);
    double inv_gmg2 = 1.0 / (gmg * gmg);
    double q = charge;
    q = q > 0.0 ? q : -q;
    double gm_out = g->energy_out * inv_mass + 1.0;
    double beta_out = sqrt(1.0 - 1.0 / (gm_out * gm_out));
    double efl = g->amplitude * cell_len;
    double concomm = q * efl / (mass * betag2);
    double concomm1 = concomm * inv_gmg2 / gmg;
    double con1 = PI * concomm1;
    double con2nex = concomm * inv_gmg2;
    double con5nex, tw, inv_fkis, inv_gmgcl;
    if (ccl) {
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
    sincos(g->phase_ref, &sinps, &cosps);
    double phi1, sinp1, cosp1;
    if (ccl) phi1 = phi + g->phase_shift - TWOPI * g->dg / (beta * wave_len) + ccl_cell_num * PI;
    else phi1 = phi + g->phase_shift;
    sincos(phi1, &sinp1, &cosp1);
    double prome1 = -con1 * (tp_fac * (sinp1 - sinps) + sp_fac * (cosp1 - cosps));
    sincos(phi1 + prome1, &sinp1, &cosp1);
    double rs_p = x * x + y * y;
    double rrp = x * xp + y * yp;
    double ris, fkrris, rpris = 0.0, bes1covr;
    ris = sqrt(rs_p);
    fkrris = fkr * ris;
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
    if (ccl) {
      double dps = phi_in - g->phase_ref;
      phi_new = phi + (1.0 - (beta - beta_out) * betag_ccl / (beta * beta_out)) * (PI * g->clbl + dps) + prome;
    } else {
      double d_cell_len = cell_len - g->beta_center * wave_len;
      double dphi_qlen2 = TWOPI * 0.5 * q2 / (beta * wave_len);
      double dphi_clen = 0.0;
      if (d_cell_len > 1e-15 || d_cell_len < -1e-15) dphi_clen = PI * d_cell_len / (beta * wave_len);
      double dps = g->phase_ref - phi_in;
      phi_new = phi + (1.0 - (beta - beta_out) / beta) * (PI * g->clbl + dps) + prome + dphi_clen - dphi_qlen2;
    }
    if (w <= 0.0 || x != x || y != y || xp != xp || yp != yp || w != w || phi_new != phi_new) {
      b->loss[i] = 33333333;
    } else {
      b->x[i] = x; b->y[i] = y; b->xp[i] = xp; b->yp[i] = yp; b->w[i] = w; b->phi[i] = phi_new;
    }
  }
}

/* SimulateRotationKernel, simulation_kernel.cu:511-529 */
static void k_rotation(orc_beam *b, double angle) {
  double cosa = cos(angle), sina = sin(angle);
  for (uint32_t i = 0; i < b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double x = b->x[i], y = b->y[i], xp = b->xp[i], yp = b->yp[i];
    b->x[i] = x * cosa + y * sina;
    b->y[i] = y * cosa - x * sina;
    b->xp[i] = xp * cosa + yp * sina;
    b->yp[i] = yp * cosa - xp * sina;
  }
}

/* Simulate{Circular,Rectangular}ApertureKernel, simulation_kernel.cu:543-575
 * (index 0 is skipped) */
static void k_aperture(orc_beam *b, int rect, const double *p, uint32_t eid) {
  double cx = b->st[ORC_X_AVG], cy = b->st[ORC_Y_AVG];
  for (uint32_t i = 1; i < b->n; ++i) {
    if (b->loss[i] != 0) continue;
    if (!rect) {
      double aper2 = p[HPS_P_APERTURE] * p[HPS_P_APERTURE];
      double x = b->x[i] - cx, y = b->y[i] - cy;
      if (x * x + y * y > aper2) b->loss[i] = eid;
    } else {
      double xmin = cx - p[HPS_P_APT_XL], xmax = cx + p[HPS_P_APT_XR];
      double ymin = cy - p[HPS_P_APT_YB], ymax = cy + p[HPS_P_APT_YT];
      double x = b->x[i], y = b->y[i];
      if (x < xmin || x > xmax || y < ymin || y > ymax) b->loss[i] = eid;
    }
  }
}

/* SimulateBuncherKernel, simulation_kernel.cu:807-871 */
static void k_buncher(orc_beam *b, double wl, double w_ref, double freq, double voltage,
                      double phase, double aper, double freq_ratio, uint32_t eid) {
  double mass = b->mass, charge = b->charge;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double x = b->x[i], y = b->y[i], xp = b->xp[i], yp = b->yp[i];
    double phi = b->phi[i] * freq_ratio;
    double w = b->w[i];
    double r2 = x * x + y * y;
    double aper2 = aper * aper;
    if (aper2 != 0.0 && r2 > aper2) { b->loss[i] = eid; continue; }
    double h = freq * wl / CLIGHT;
    double gm1 = w_ref / mass;
    double gm = gm1 + 1.0;
    double btgm = sqrt(gm1 * (gm1 + 2.0));
    double beta = btgm / gm;
    double k = h * TWOPI / (btgm * wl);
    double k2 = k * k;
    double q = charge;
    q = q > 0.0 ? q : -q;
    double con1 = TWOPI * h * voltage * q / (beta * wl * mass);
    double arg = k2 * r2 * 0.25;
    double ph = h * phi + phase;
    double dw = q * voltage * cos(ph) * (1.0 + arg * (1.0 + arg * (0.25 + arg / 36.0)));
    double wb_par = w + 0.5 * dw;
    double wf = w + dw;
    if (wb_par <= 0.0 || wf <= 0.0) { b->loss[i] = eid; continue; }
    double gmtmp = wb_par / mass;
    double bav = sqrt(gmtmp * (gmtmp + 2.0)) / (gmtmp + 1.0);
    gmtmp = w / mass;
    double bg = sqrt(gmtmp * (gmtmp + 2.0));
    gmtmp = wf / mass;
    double rbgf = 1.0 / sqrt(gmtmp * (gmtmp + 2.0));
    double del = -con1 * sin(ph) * (1.0 - bav * beta) * (0.5 + arg * (0.25 + arg / 24.0)) / bav;
    b->xp[i] = (xp * bg + del * x) * rbgf;
    b->yp[i] = (yp * bg + del * y) * rbgf;
    b->w[i] = wf;
  }
}

/* Simulate{First,Second}HalfDipoleKernel, simulation_kernel.cu:603-805 */
static void dipole_body(const double *p, double mass, double *r11, double *r12, double *r16,
                        double *r21, double *r22, double *r26, double *r33, double *r34,
                        double *r43, double *r44, double *r51, double *r52, double *r56,
                        double *beta, double *dl, double *design_w) {
  double h = 1.0 / p[HPS_P_DIP_RADIUS];
  double findx = p[HPS_P_DIP_FIELD_INDEX];
  *design_w = p[HPS_P_DIP_KINETIC_ENERGY];
  double h2 = h * h;
  *dl = 0.5 * p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE];
  double yk2 = findx * h2;
  double yk = sqrt(fabs(yk2));
  double inv_yk = 1.0 / yk;
  double ykl = yk * *dl;
  double xk2 = h2 - yk2;
  double inv_xk2 = 1.0 / xk2;
  double xk = sqrt(fabs(xk2));
  double inv_xk = 1.0 / xk;
  double xkl = xk * *dl;
  double cxkl = 1.0, sxokx = *dl;
  if (xk2 > 0.0) { cxkl = cos(xkl); sxokx = sin(xkl) * inv_xk; }
  else if (xk2 < 0.0) { cxkl = cosh(xkl); sxokx = sinh(xkl) * inv_xk; }
  double cykl = 1.0, syoky = *dl;
  if (yk2 > 0.0) { cykl = cos(ykl); syoky = sin(ykl) * inv_yk; }
  else if (yk2 < 0.0) { cykl = cosh(ykl); syoky = sinh(ykl) * inv_yk; }
  *r11 = cxkl; *r12 = sxokx; *r21 = -xk2 * sxokx; *r22 = cxkl;
  *r33 = cykl; *r34 = syoky; *r43 = -yk2 * syoky; *r44 = cykl;
  *r26 = h * sxokx;
  *r16 = h * (1.0 - cxkl) * inv_xk2;
  *r51 = -*r26;
  *r52 = -*r16;
  double gamma = *design_w / mass + 1.0;
  double beta2 = 1.0 - 1.0 / (gamma * gamma);
  *beta = sqrt(beta2);
  *r56 = -h2 * (*dl * beta2 - sxokx) * inv_xk2 + *dl * (1.0 - h2 * inv_xk2) / (gamma * gamma);
}

static void k_dipole(orc_beam *b, double wl, const double *p, int second) {
  double mass = b->mass;
  double r11, r12, r16, r21, r22, r26, r33, r34, r43, r44, r51, r52, r56, beta, dl, design_w;
  dipole_body(p, mass, &r11, &r12, &r16, &r21, &r22, &r26, &r33, &r34, &r43, &r44, &r51,
              &r52, &r56, &beta, &dl, &design_w);
  double h = 1.0 / p[HPS_P_DIP_RADIUS];
  double hf_g = p[HPS_P_DIP_HALF_GAP], k1 = p[HPS_P_DIP_K1], k2 = p[HPS_P_DIP_K2];
  double bedge = second ? p[HPS_P_DIP_EDGE_OUT] : p[HPS_P_DIP_EDGE_IN];
  double c1 = 2.0 * hf_g * k1 * h;
  double sinb, cosb;
  if (!second) sincos(bedge, &sinb, &cosb);
  else { sinb = sin(bedge); cosb = cos(bedge); }
  double inv_cosb = 1.0 / cosb;
  double psi = c1 * (1.0 + sinb * sinb) * inv_cosb * (1.0 - c1 * k2 * sinb * inv_cosb);
  double e21 = tan(bedge) * h;
  double e43 = tan(bedge - psi) * h;
  for (uint32_t i = 0; i < b->n; ++i) {
    if (b->loss[i] != 0) continue;
    double x = b->x[i], xp = b->xp[i], y = b->y[i], yp = b->yp[i];
    double dpop = (design_w / mass + 1.0) / (design_w * ((design_w / mass + 1.0) + 1.0)) * (b->w[i] - design_w);
    if (!second) {
      xp += e21 * x;
      yp -= e43 * y;
      b->x[i] = r11 * x + r12 * xp + r16 * dpop;
      b->xp[i] = r21 * x + r22 * xp + r26 * dpop;
      b->y[i] = r33 * y + r34 * yp;
      b->yp[i] = r43 * y + r44 * yp;
      b->phi[i] += TWOPI * (-(r51 * x + r52 * xp + r56 * dpop) + dl) / (beta * wl);
    } else {
      b->phi[i] += TWOPI * (-(r51 * x + r52 * xp + r56 * dpop) + dl) / (beta * wl);
      double x_new = r11 * x + r12 * xp + r16 * dpop;
      xp = r21 * x + r22 * xp + r26 * dpop;
      double y_new = r33 * y + r34 * yp;
      yp = r43 * y + r44 * yp;
      b->x[i] = x_new; b->y[i] = y_new;
      b->xp[i] = xp + e21 * x_new;
      b->yp[i] = yp - e43 * y_new;
    }
  }
}

/* ------------------------------------------------------------------ */
/* Engine: src/simulation/src/simulation_engine.{cpp,cu}                */
/* ------------------------------------------------------------------ */

orc_sim *orc_sim_create(orc_beam *b, uint32_t nelem, const int *types, const double *params,
                        orc_scheff *spch) {
  orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
  s->beam = b; s->spch = spch; s->nelem = nelem; s->types = types; s->params = params;
  s->sc_on = spch != NULL;       /* SimulationEngine::InitEngine, :408-427 */
  s->prev_end = -1;              /* (int)numeric_limits<uint>::max() */
  orc_sim_reset(s);
  return s;
}
void orc_sim_free(orc_sim *s) { free(s); }
void orc_sim_set_monitor(orc_sim *s, double *mon) { s->mon = mon; }

/* Reset, simulation_engine.cu:101-111 */
void orc_sim_reset(orc_sim *s) {
  s->cur_id = 0; s->ccl_cell_num = 0;
  s->design_w = s->beam->design_w;
  s->wavelen = CLIGHT / s->beam->freq;
}

static const double *P(orc_sim *s, uint32_t i) { return s->params + (size_t)i * HPS_NPARAM; }
static int T(orc_sim *s, int64_t i) { return (i >= 0 && i < (int64_t)s->nelem) ? s->types[i] : 0; }

static void sc_start(orc_sim *s, double len) {
  if (s->sc_on && s->spch) orc_scheff_start(s->spch, s->beam, len);
}

/* PrepSimulateRFGap, simulation_engine.cu:163-175 */
static void prep_gap(orc_sim *s, const rfgap_t *g) {
  if (s->beam->freq != g->frequency) {
    s->wavelen = CLIGHT / g->frequency;
    orc_beam_change_frequency(s->beam, g->frequency);
  }
}

static int visit(orc_sim *s, uint32_t i) {
  orc_beam *b = s->beam;
  const double *p = P(s, i);
  uint32_t eid = s->cur_id;
  switch (s->types[i]) {
    case HPS_ELEM_DRIFT: { /* SimulateDrift, :125-145 */
      int nk = 1;
      double length = p[HPS_P_LENGTH];
      if (s->sc_on && s->spch) nk = (int)ceil(length / s->spch->interval);
      double hf = 0.5 * length / nk;
      for (int k = 0; k < nk; ++k) {
        k_partial_drift(b, s->wavelen, hf, p[HPS_P_APERTURE], eid);
        sc_start(s, 2.0 * hf);
        k_partial_drift(b, s->wavelen, hf, p[HPS_P_APERTURE], eid);
      }
      break;
    }
    case HPS_ELEM_QUAD: /* SimulateQuad, :147-161 (block = blck_size/2) */
      if (b->blck_size / 2 > 0)
        k_half_quad(b, s->wavelen, p[HPS_P_LENGTH], p[HPS_P_APERTURE], p[HPS_P_GRADIENT], eid);
      sc_start(s, p[HPS_P_LENGTH]);
      if (b->blck_size / 2 > 0)
        k_half_quad(b, s->wavelen, p[HPS_P_LENGTH], p[HPS_P_APERTURE], p[HPS_P_GRADIENT], eid);
      break;
    case HPS_ELEM_RFGAP_DTL: { /* SimulateDTLRFGap, :182-241 */
      rfgap_t g; load_gap(p, &g);
      prep_gap(s, &g);
      double phi_in = 0.0;
      uint32_t sz = s->nelem, c = s->cur_id;
      if (c == 1 || (c > 1 && T(s, c - 2) != HPS_ELEM_RFGAP_DTL)) {
        if (c + 2 < sz && T(s, c + 2) == HPS_ELEM_RFGAP_DTL)
          phi_in = g.phase_ref - 0.5 * (P(s, c + 2)[HPS_P_RF_PHASE_REF] - g.phase_ref);
        else if (c + 1 >= sz) return -1;
        else phi_in = g.phase_ref;
      } else if (c > 1) {
        phi_in = 0.5 * (P(s, c - 2)[HPS_P_RF_PHASE_REF] + g.phase_ref);
      } else return -1;
      if (T(s, (int64_t)c - 1) != HPS_ELEM_QUAD || T(s, (int64_t)c + 1) != HPS_ELEM_QUAD) return -1;
      double q1 = P(s, c - 1)[HPS_P_LENGTH], q2 = P(s, c + 1)[HPS_P_LENGTH];
      if (b->blck_size / 2 > 0)
        k_gap_first(b, &s->wavelen, s->design_w, phi_in, &g, g.length, q1, q2, 0);
      sc_start(s, g.length);
      if (b->blck_size / 2 > 0)
        k_gap_second(b, s->wavelen, s->design_w, phi_in, &g, g.length, 0, q1, q2, 0);
      s->design_w = g.energy_out;
      b->design_w = s->design_w;
      break;
    }
    case HPS_ELEM_RFGAP_CCL: { /* SimulateCCLRFGap, :243-293 */
      rfgap_t g; load_gap(p, &g);
      prep_gap(s, &g);
      uint32_t c = s->cur_id;
      if (c == 0 || T(s, (int64_t)c - 1) != HPS_ELEM_RFGAP_CCL) s->ccl_cell_num = 0;
      double phi_in, phi_out, cur = g.phase_ref;
      if (s->ccl_cell_num == 0) {
        if (!(T(s, c + 1) == HPS_ELEM_RFGAP_CCL || T(s, c + 1) == HPS_ELEM_RFGAP_DTL)) return -1;
        double nxt = P(s, c + 1)[HPS_P_RF_PHASE_REF];
        phi_in = cur - 0.5 * (nxt - cur);
        phi_out = 0.5 * (nxt + cur);
      } else if (T(s, c + 1) != HPS_ELEM_RFGAP_CCL) {
        double prv = P(s, c - 1)[HPS_P_RF_PHASE_REF];
        phi_in = 0.5 * (cur + prv);
        phi_out = cur + 0.5 * (cur - prv);
      } else {
        phi_in = 0.5 * (cur + P(s, c - 1)[HPS_P_RF_PHASE_REF]);
        phi_out = 0.5 * (cur + P(s, c + 1)[HPS_P_RF_PHASE_REF]);
      }
      uint32_t gcb = b->blck_size / 4 > 1 ? b->blck_size / 4 : b->blck_size;
      if (gcb > 0) k_gap_first(b, &s->wavelen, s->design_w, phi_in, &g, g.length, 0.0, 0.0, 1);
      sc_start(s, g.length);
      if (gcb > 0)
        k_gap_second(b, s->wavelen, s->design_w, phi_out, &g, g.length, s->ccl_cell_num, 0.0, 0.0, 1);
      s->ccl_cell_num++;
      s->design_w = g.energy_out;
      b->design_w = s->design_w;
      break;
    }
    case HPS_ELEM_ROTATION:
      k_rotation(b, p[HPS_P_ROT_ANGLE]);
      break;
    case HPS_ELEM_SPCHCOMP:
      if (s->sc_on && s->spch) s->spch->fraction = p[HPS_P_SPC_FRACTION];
      break;
    case HPS_ELEM_APERTURE_C:
    case HPS_ELEM_APERTURE_R:
      if (p[HPS_P_APT_IN] == 0.0) break;
      orc_beam_update_loss(b);
      orc_beam_update_avg_xy(b);
      k_aperture(b, s->types[i] == HPS_ELEM_APERTURE_R, p, eid);
      break;
    case HPS_ELEM_DIAGNOSTICS:
      break;
    case HPS_ELEM_STEERER: {
      double blh = p[HPS_P_STR_BLH], blv = p[HPS_P_STR_BLV];
      if (blh > 1e-10 || blv > 1e-10) k_steerer(b, blh, blv);
      break;
    }
    case HPS_ELEM_BUNCHER: {
      if (p[HPS_P_BUN_ON] == 0.0) break;
      double bf = p[HPS_P_BUN_FREQ];
      s->wavelen = CLIGHT / bf;
      k_buncher(b, s->wavelen, s->design_w, bf, p[HPS_P_BUN_VOLTAGE], p[HPS_P_BUN_PHASE],
                p[HPS_P_APERTURE], bf / b->freq, eid);
      break;
    }
    case HPS_ELEM_DIPOLE:
      if (b->blck_size / 4 > 0) k_dipole(b, s->wavelen, p, 0);
      sc_start(s, p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE]);
      if (b->blck_size / 4 > 0) k_dipole(b, s->wavelen, p, 1);
      break;
    default:
      return -1;
  }
  return 0;
}

/* SimulationEngine::Simulate, simulation_engine.cpp:447-469 (indices
 * instead of names; -1 selects the first / last element) */
int orc_sim_simulate(orc_sim *s, int start, int end) {
  int start_index = start < 0 ? 0 : start;
  int end_index = end < 0 ? (int)s->nelem - 1 : end;
  /* prev_end_element_index_ is an int (simulation_engine.h:66) holding
   * UINT_MAX, i.e. -1: the first call does not reset */
  if (start_index < s->prev_end) orc_sim_reset(s);
  s->prev_end = end_index;
  for (int i = 0; i <= end_index; ++i) {
    if (i >= start_index || s->types[i] == HPS_ELEM_SPCHCOMP) {
      s->cur_id = (uint32_t)i;
      uint32_t solves0 = s->spch ? s->spch->n_solves : 0;
      if (visit(s, (uint32_t)i) != 0) { s->error = 1; return -1; }
      if (s->mon) {
        double *m = s->mon + (size_t)i * HPS_NMON;
        orc_beam_monitor(s->beam, m);
        if (s->spch) {
          m[HPS_MON_SC_DR] = s->spch->dr;
          m[HPS_MON_SC_DZ] = s->spch->dz;
          m[HPS_MON_SC_REMESH] = (double)(s->spch->n_solves - solves0);
          m[HPS_MON_SC_ONMESH] = (double)s->spch->num_on_mesh;
        }
        m[HPS_MON_ELEM] = (double)i;
      }
    }
  }
  return 0;
}
