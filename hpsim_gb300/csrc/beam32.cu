// beam32.cu -- beam moments, loss counts and the small per-particle beam
// kernels for FP32 beams (same operations as beam_ops.cu).
//
// FP32 beams hold x, x', y, y' as FP32 and phi, W as FP32 offsets from the
// synchronous particle (DevBeam::phi_ref, w_ref, FP64 on the host).  Every
// statistic is stored in the beam's FP64 statistics block in the reference's
// absolute units: sums are taken over the offsets (per thread and per warp in
// FP32, across warps and blocks in FP64) and the anchor is added to the
// averages in FP64; central moments are shift-invariant, so they are taken
// from the offset sums directly.  Divisors follow beam_ops.cu.
#include "internal.h"
#include "reduce.cuh"

namespace hps {

namespace {

struct NoCtx {};

__device__ inline float *fcoord(const DevBeam &b, int c) {
  switch (c) {
    case HPS_COORD_X: return b.fx;
    case HPS_COORD_XP: return b.fxp;
    case HPS_COORD_Y: return b.fy;
    case HPS_COORD_YP: return b.fyp;
    case HPS_COORD_PHI: return b.fphi;
    case HPS_COORD_W: return b.fw;
    default: return b.fphi_r;
  }
}
__host__ __device__ inline double anchor(const DevBeam &b, int c) {
  return c == HPS_COORD_PHI ? b.phi_ref : c == HPS_COORD_W ? b.w_ref : 0.0;
}

__device__ inline double surv(const DevBeam &b) { return (double)(uint32_t)(b.n - b.st->num_loss); }

__device__ inline int avg_slot(int c, int g) {
  switch (c) {
    case HPS_COORD_X: return g ? X_AVG_GOOD : X_AVG;
    case HPS_COORD_XP: return XP_AVG;
    case HPS_COORD_Y: return g ? Y_AVG_GOOD : Y_AVG;
    case HPS_COORD_YP: return YP_AVG;
    case HPS_COORD_PHI: return g ? PHI_AVG_GOOD : PHI_AVG;
    case HPS_COORD_W: return g ? W_AVG_GOOD : W_AVG;
    default: return PHI_AVG_R;
  }
}
__device__ inline int sig_slot(int c, int g) {
  switch (c) {
    case HPS_COORD_X: return g ? X_SIG_GOOD : X_SIG;
    case HPS_COORD_XP: return XP_SIG;
    case HPS_COORD_Y: return g ? Y_SIG_GOOD : Y_SIG;
    case HPS_COORD_YP: return YP_SIG;
    case HPS_COORD_PHI: return PHI_SIG;
    case HPS_COORD_W: return g ? W_SIG_GOOD : W_SIG;
    default: return g ? PHI_SIG_GOOD : PHI_SIG_R;
  }
}

// XReduceKernel / XX2ReduceKernel + their finalisers (beam_kernel.cu:84-166,
// 384-494, 1413-1446)
struct Op32Moment {
  static constexpr int K = 2;
  using Comb = SumComb;
  using Ctx = NoCtx;
  struct P { uint32_t lo, ll; float v; };
  DevBeam b;
  int coord, good_only, sigma;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {}; }
  __device__ P load(uint32_t i) const { return {b.loss[i], good_only ? b.lloss[i] : 0u, fcoord(b, coord)[i]}; }
  __device__ void use(uint32_t, const P &p, float (&a)[K], const Ctx &) const {
    bool keep = (uint32_t)(p.lo + p.ll) == 0u;
    float v = keep ? p.v : 0.0f;
    a[0] += v;
    a[1] += v * v;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    double off = anchor(b, coord);
    if (!sigma) {
      double *dst = &b.st->st[avg_slot(coord, good_only)];
      if (!good_only) *dst = t[0] / surv(b) + off;
      else *dst = b.st->num_good > 0 ? t[0] / b.st->num_good + off : -99999;
    } else {
      double d = good_only ? (double)b.st->num_good : surv(b);
      double avg = t[0] / d, avg2 = t[1] / d;
      b.st->st[sig_slot(coord, good_only)] = sqrt(avg2 - avg * avg);
    }
  }
};

// UpdateEmittance (beam.cpp:985-995) in one sweep, as OpEmittance
struct Op32Emittance {
  static constexpr int K = 15;
  using Comb = SumComb;
  struct Ctx { float phi0; };
  struct P { uint32_t lo; float x, xp, y, yp, ph, w; };
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {b.fphi[0]}; }
  __device__ P load(uint32_t i) const { return {b.loss[i], b.fx[i], b.fxp[i], b.fy[i], b.fyp[i], b.fphi[i], b.fw[i]}; }
  __device__ void use(uint32_t i, const P &p, float (&a)[K], const Ctx &c) const {
    float pr = rel_phase_f(p.ph - c.phi0);
    b.fphi_r[i] = pr;
    if (p.lo != 0u) return;
    float x = p.x, xp = p.xp, y = p.y, yp = p.yp, w = p.w;
    a[0] += x; a[1] += x * x; a[2] += xp; a[3] += xp * xp; a[4] += x * xp;
    a[5] += y; a[6] += y * y; a[7] += yp; a[8] += yp * yp; a[9] += y * yp;
    a[10] += pr; a[11] += pr * pr; a[12] += w; a[13] += w * w; a[14] += pr * w;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    double sv = surv(b);
    double g1 = (b.w_ref + (double)b.fw[0]) / b.mass, bg = sqrt(g1 * (g1 + 2.0));
    for (int pl = 0; pl < 2; ++pl) {
      const double *q = t + 5 * pl;
      double x = q[0] / sv, x2 = q[1] / sv, xp = q[2] / sv, xp2 = q[3] / sv, xxp = q[4] / sv;
      double *s = b.st->st;
      s[pl ? Y_AVG : X_AVG] = x;
      s[pl ? Y_SIG : X_SIG] = sqrt(x2 - x * x);
      s[pl ? YP_AVG : XP_AVG] = xp;
      s[pl ? YP_SIG : XP_SIG] = sqrt(xp2 - xp * xp);
      s[pl ? Y_EMIT : X_EMIT] = sqrt((x2 - x * x) * (xp2 - xp * xp) - (xxp - x * xp) * (xxp - x * xp)) * bg;
    }
    double phi = t[10] / sv, phi2 = t[11] / sv, w = t[12] / sv, w2 = t[13] / sv, pw = t[14] / sv;
    double pv = phi2 - phi * phi, wv = w2 - w * w, cv = pw - phi * w;
    b.st->st[PHI_AVG_R] = phi;
    b.st->st[W_AVG] = w + b.w_ref;
    b.st->st[PHI_SIG_R] = sqrt(pv);
    b.st->st[W_SIG] = sqrt(wv);
    b.st->st[Z_EMIT] = sqrt(pv * wv - cv * cv);
  }
};

struct Op32AvgXY {
  static constexpr int K = 2;
  using Comb = SumComb;
  using Ctx = NoCtx;
  struct P { uint32_t lo; float x, y; };
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {}; }
  __device__ P load(uint32_t i) const { return {b.loss[i], b.fx[i], b.fy[i]}; }
  __device__ void use(uint32_t, const P &p, float (&a)[K], const Ctx &) const {
    if (p.lo != 0u) return;
    a[0] += p.x;
    a[1] += p.y;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[X_AVG] = t[0] / surv(b);
    b.st->st[Y_AVG] = t[1] / surv(b);
  }
};

struct Op32MaxRPhi {
  static constexpr int K = 2;
  using Comb = MaxComb;
  struct Ctx { float xa, ya, pa; };
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const {
    return {(float)b.st->st[X_AVG], (float)b.st->st[Y_AVG], (float)b.st->st[PHI_AVG_R]};
  }
  struct P { uint32_t lo; float x, y, pr; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.fx[i], b.fy[i], b.fphi_r[i]}; }
  __device__ void use(uint32_t, const P &p, float (&a)[K], const Ctx &c) const {
    if (p.lo != 0u) return;
    float tx = p.x - c.xa, ty = p.y - c.ya;
    float r2 = tx * tx + ty * ty;
    float tp = fabsf(p.pr - c.pa);
    a[0] = fmaxf(a[0], r2);
    a[1] = fmaxf(a[1], tp);
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[R_MAX] = sqrt(t[0]);
    b.st->st[ABS_PHI_MAX] = t[1];
  }
};

struct Op32FreqAverages {
  static constexpr int K = 2;
  using Comb = SumComb;
  struct Ctx { float phi0; };
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {b.fphi[0]}; }
  struct P { uint32_t lo; float ph; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.fphi[i]}; }
  __device__ void use(uint32_t i, const P &p, float (&a)[K], const Ctx &c) const {
    float pr = rel_phase_f(p.ph - c.phi0);
    b.fphi_r[i] = pr;
    if (p.lo != 0u) return;
    a[0] += p.ph;
    a[1] += pr;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[PHI_AVG] = t[0] / surv(b) + b.phi_ref;
    b.st->st[PHI_AVG_R] = t[1] / surv(b);
  }
};

struct Op32Monitor {
  static constexpr int K = 17;
  using Comb = SumComb;
  struct Ctx { float phi0; };
  DevBeam b;
  const ScState *sc;
  double *out;
  uint32_t elem;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {b.fphi[0]}; }
  struct P { uint32_t lo, ll; float x, xp, y, yp, ph, w; };
  __device__ P load(uint32_t i) const {
    return {b.loss[i], b.lloss[i], b.fx[i], b.fxp[i], b.fy[i], b.fyp[i], b.fphi[i], b.fw[i]};
  }
  __device__ void use(uint32_t, const P &p, float (&a)[K], const Ctx &c) const {
    if ((uint32_t)(p.lo + p.ll) == 0u) a[16] += 1.0f;
    if (p.lo != 0u) return;
    float pr = rel_phase_f(p.ph - c.phi0);
    float x = p.x, xp = p.xp, y = p.y, yp = p.yp, w = p.w;
    a[0] += 1.0f;
    a[1] += x; a[2] += x * x; a[3] += xp; a[4] += xp * xp; a[5] += x * xp;
    a[6] += y; a[7] += y * y; a[8] += yp; a[9] += yp * yp; a[10] += y * yp;
    a[11] += pr; a[12] += pr * pr; a[13] += w; a[14] += w * w; a[15] += pr * w;
  }
  __device__ void finalize(const double *s, int tid, int) const {
    if (tid) return;
    double *o = out;
    for (int k = 0; k < HPS_NMON; ++k) o[k] = 0.0;
    double m = s[0];
    o[HPS_MON_NALIVE] = m;
    o[HPS_MON_NGOOD] = s[16];
    double w0 = b.w_ref + (double)b.fw[0];
    double g1 = w0 / b.mass, bg = sqrt(g1 * (g1 + 2.0));
    if (m > 0) {
      for (int pl = 0; pl < 2; ++pl) {
        const double *q = s + 1 + 5 * pl;
        double a = q[0] / m, a2 = q[1] / m, ap = q[2] / m, ap2 = q[3] / m, aap = q[4] / m;
        int base = pl ? HPS_MON_Y_AVG : HPS_MON_X_AVG;
        o[base] = a;
        o[base + 1] = sqrt(a2 - a * a);
        o[base + 2] = ap;
        o[base + 3] = sqrt(ap2 - ap * ap);
        o[base + 4] = sqrt((a2 - a * a) * (ap2 - ap * ap) - (aap - a * ap) * (aap - a * ap)) * bg;
      }
      double p = s[11] / m, p2 = s[12] / m, w = s[13] / m, w2 = s[14] / m, pw = s[15] / m;
      double pv = p2 - p * p, wv = w2 - w * w, cv = pw - p * w;
      o[HPS_MON_PHIR_AVG] = p;
      o[HPS_MON_PHIR_SIG] = sqrt(pv);
      o[HPS_MON_W_AVG] = w + b.w_ref;
      o[HPS_MON_W_SIG] = sqrt(wv);
      o[HPS_MON_Z_EMIT] = sqrt(pv * wv - cv * cv);
    }
    o[HPS_MON_W0] = w0;
    o[HPS_MON_PHI0] = b.phi_ref + (double)b.fphi[0];
    if (sc) {
      o[HPS_MON_SC_DR] = sc->dr;
      o[HPS_MON_SC_DZ] = sc->dz;
      o[HPS_MON_SC_REMESH] = (double)sc->n_solves;
      o[HPS_MON_SC_ONMESH] = (double)sc->num_on_mesh;
    }
    o[HPS_MON_ELEM] = (double)elem;
  }
};

#define PARTICLES(b) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (b).n; i += gridDim.x * blockDim.x)

// UpdateRelativePhiKernel (beam_kernel.cu:1507-1525)
__global__ void k32_relative_phi(DevBeam b, int use_good) {
  float ref = use_good ? (float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref) : b.fphi[0];
  PARTICLES(b) b.fphi_r[i] = rel_phase_f(b.fphi[i] - ref);
}

// UpdateLongitudinalLossCoordinateKernel (beam_kernel.cu:1550-1559)
__global__ void k32_lloss(DevBeam b) {
  float lim = (float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref + TWOPI + PI);
  PARTICLES(b) if (b.fphi[i] > lim) b.lloss[i] = 1u;
}

__global__ void k32_scale_phi(DevBeam b, float r) {
  PARTICLES(b) b.fphi[i] *= r;
}

// CutBeamKernel (beam_kernel.cu:1465-1481): compared in absolute units
__global__ void k32_cut(DevBeam b, int coord, double lo, double hi) {
  const float *v = fcoord(b, coord);
  double off = anchor(b, coord);
  PARTICLES(b) {
    if (i == 0 || b.loss[i] != 0u) continue;
    double x = off + (double)v[i];
    if (x < hi && x > lo) b.loss[i] = 99999u;
  }
}

// ShiftVariableKernel (beam_kernel.cu:1491-1497)
__global__ void k32_shift(DevBeam b, int coord, float val) {
  float *v = fcoord(b, coord);
  PARTICLES(b) if (i > 0) v[i] += val;
}

// move the anchor of phi or W: every offset changes by delta, particle 0
// becomes the anchor itself
__global__ void k32_reanchor(DevBeam b, int coord, float delta) {
  float *v = fcoord(b, coord);
  PARTICLES(b) v[i] = i == 0 ? 0.0f : v[i] + delta;
}

__global__ void k32_from_double(DevBeam b, const double *x, const double *xp, const double *y, const double *yp,
                                const double *phi, const double *w) {
  PARTICLES(b) {
    b.fx[i] = (float)x[i];
    b.fxp[i] = (float)xp[i];
    b.fy[i] = (float)y[i];
    b.fyp[i] = (float)yp[i];
    b.fphi[i] = (float)(phi[i] - b.phi_ref);
    b.fw[i] = (float)(w[i] - b.w_ref);
  }
}

__global__ void k32_to_double(DevBeam b, int coord, double *out) {
  const float *v = fcoord(b, coord);
  double off = anchor(b, coord);
  PARTICLES(b) out[i] = off + (double)v[i];
}

}  // namespace

void beam32_update_avg(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st) {
  if (coord == HPS_COORD_XP || coord == HPS_COORD_YP) good = 0;
  launch_pass_f(Op32Moment{b, coord, good, 0}, b.n, s, st); note_launch();
}
void beam32_update_sig(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st) {
  if (b.n <= 2) return;
  if (coord == HPS_COORD_XP || coord == HPS_COORD_YP || coord == HPS_COORD_PHI) good = 0;
  launch_pass_f(Op32Moment{b, coord, good, 1}, b.n, s, st); note_launch();
}
void beam32_update_emittance(const DevBeam &b, PassScratch s, cudaStream_t st) {
  if (b.n <= 2) return;
  launch_pass_f(Op32Emittance{b}, b.n, s, st); note_launch();
}
void beam32_update_relative_phi(const DevBeam &b, int use_good, cudaStream_t st) {
  k32_relative_phi<<<grid_for(b.n), kBlock, 0, st>>>(b, use_good); note_launch();
}
void beam32_update_longitudinal_loss(const DevBeam &b, PassScratch s, cudaStream_t st) {
  beam_update_good_count(b, s, st);
  beam32_update_avg(b, HPS_COORD_PHI, 1, s, st);
  k32_lloss<<<grid_for(b.n), kBlock, 0, st>>>(b); note_launch();
  beam_update_lloss_count(b, s, st);
}
void beam32_update_avg_xy(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass_f(Op32AvgXY{b}, b.n, s, st); note_launch();
}
void beam32_update_max_r_phi(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass_f(Op32MaxRPhi{b}, b.n, s, st); note_launch();
}
// the anchor phase scales with the offsets: phi_ref *= ratio on the host
void beam32_change_frequency(DevBeam &b, double ratio, PassScratch s, cudaStream_t st) {
  b.phi_ref *= ratio;
  k32_scale_phi<<<grid_for(b.n), kBlock, 0, st>>>(b, (float)ratio); note_launch();
  launch_pass_f(Op32FreqAverages{b}, b.n, s, st); note_launch();
}
void beam32_apply_cut(const DevBeam &b, int coord, double lo, double hi, cudaStream_t st) {
  k32_cut<<<grid_for(b.n), kBlock, 0, st>>>(b, coord, lo, hi); note_launch();
}
void beam32_shift(const DevBeam &b, int coord, double val, cudaStream_t st) {
  k32_shift<<<grid_for(b.n), kBlock, 0, st>>>(b, coord, (float)val); note_launch();
}
// Beam::SetRefEnergy / SetRefPhase (beam.cpp): particle 0 takes the value;
// the anchor moves to it so that particle 0 stays exact
void beam32_set_ref(DevBeam &b, int coord, double val, cudaStream_t st) {
  double old = coord == HPS_COORD_PHI ? b.phi_ref : b.w_ref;
  if (coord == HPS_COORD_PHI) b.phi_ref = val;
  else b.w_ref = val;
  k32_reanchor<<<grid_for(b.n), kBlock, 0, st>>>(b, coord, (float)(old - val)); note_launch();
}
void beam32_monitor(const DevBeam &b, const ScState *sc, double *mon_dev, uint32_t elem, PassScratch s,
                    cudaStream_t st) {
  launch_pass_f(Op32Monitor{b, sc, mon_dev, elem}, b.n, s, st); note_launch();
}
// staged FP64 coordinates -> FP32 state; the anchor is set by the caller
void beam32_from_double(const DevBeam &b, const double *const *src, cudaStream_t st) {
  k32_from_double<<<grid_for(b.n), kBlock, 0, st>>>(b, src[0], src[1], src[2], src[3], src[4], src[5]);
  note_launch();
}
void beam32_to_double(const DevBeam &b, int coord, double *out, cudaStream_t st) {
  k32_to_double<<<grid_for(b.n), kBlock, 0, st>>>(b, coord, out); note_launch();
}

}  // namespace hps
