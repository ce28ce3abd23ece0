// beam_ops.cu -- beam moments, loss counts and the small per-particle beam
// kernels of src/beam/ (beam.cpp, beam.cu, beam_kernel.cu).
//
// Every reduction is one pass_kernel launch (reduce.cuh) whose finaliser
// applies the formula of the reference's <<<1,1>>> finaliser kernel,
// including its divisors: masked sums over "transversely good" particles are
// divided by num_particle - num_loss with num_loss as the last UpdateLoss
// left it, sums over "good" particles by num_good.
#include "internal.h"
#include "reduce.cuh"

namespace hps {

namespace {

__device__ inline double *coord_of(const DevBeam &b, int c) {
  switch (c) {
    case HPS_COORD_X: return b.x;
    case HPS_COORD_XP: return b.xp;
    case HPS_COORD_Y: return b.y;
    case HPS_COORD_YP: return b.yp;
    case HPS_COORD_PHI: return b.phi;
    case HPS_COORD_W: return b.w;
    default: return b.phi_r;
  }
}

__device__ inline bool alive(const DevBeam &b, uint32_t i) { return b.loss[i] == 0u; }
// XReduceKernel's lloss mask: tmploss = loss + lloss (uint add), == 0
__device__ inline bool good(const DevBeam &b, uint32_t i) { return (uint32_t)(b.loss[i] + b.lloss[i]) == 0u; }

__device__ inline double surv(const DevBeam &b) { return (double)(uint32_t)(b.n - b.st->num_loss); }

// LossReduceKernel (beam_kernel.cu:270-347): count of nonzero entries
struct OpCount {
  static constexpr int K = 1;
  using Comb = SumComb;
  DevBeam b;
  int which;  // 0 loss -> num_loss, 1 lloss -> num_lloss, 2 good -> num_good
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    if (which == 0) a[0] += b.loss[i] != 0u;
    else if (which == 1) a[0] += b.lloss[i] != 0u;
    else a[0] += good(b, i);
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t v = (uint32_t)t[0];
    if (which == 0) b.st->num_loss = v;
    else if (which == 1) b.st->num_lloss = v;
    else b.st->num_good = v;
  }
};

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

// XReduceKernel + UpdateVariableAvg[WithLloss]Kernel (beam_kernel.cu:84-166,
// 1413-1426) and XX2ReduceKernel + UpdateVariableSigma[WithLloss]Kernel
// (beam_kernel.cu:384-494, 1428-1446)
struct OpMoment {
  static constexpr int K = 2;
  using Comb = SumComb;
  DevBeam b;
  int coord, good_only, sigma;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    bool keep = good_only ? good(b, i) : alive(b, i);
    double v = keep ? coord_of(b, coord)[i] : 0.0;
    a[0] += v;
    a[1] += v * v;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    if (!sigma) {
      double *dst = &b.st->st[avg_slot(coord, good_only)];
      if (!good_only) *dst = t[0] / surv(b);
      else *dst = b.st->num_good > 0 ? t[0] / b.st->num_good : -99999;
    } else {
      double d = good_only ? (double)b.st->num_good : surv(b);
      double avg = t[0] / d, avg2 = t[1] / d;
      b.st->st[sig_slot(coord, good_only)] = sqrt(avg2 - avg * avg);
    }
  }
};

// UpdateEmittance (beam.cpp:985-995): horizontal and vertical
// EmittanceReduceKernel + UpdateTransverseEmittanceKernel (normalised by
// beta*gamma of w[0]), UpdateRelativePhi() relative to particle 0, then the
// longitudinal emittance of (phi_r, w).  One sweep: phi_r is written and
// the 15 sums over loss == 0 are taken together.
struct OpEmittance {
  static constexpr int K = 15;
  using Comb = SumComb;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    double pr = rel_phase(b.phi[i], b.phi[0]);
    b.phi_r[i] = pr;
    if (!alive(b, i)) return;
    double x = b.x[i], xp = b.xp[i], y = b.y[i], yp = b.yp[i], w = b.w[i];
    a[0] += x; a[1] += x * x; a[2] += xp; a[3] += xp * xp; a[4] += x * xp;
    a[5] += y; a[6] += y * y; a[7] += yp; a[8] += yp * yp; a[9] += y * yp;
    a[10] += pr; a[11] += pr * pr; a[12] += w; a[13] += w * w; a[14] += pr * w;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    double sv = surv(b);
    double g1 = b.w[0] / b.mass, bg = sqrt(g1 * (g1 + 2.0));
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
    b.st->st[W_AVG] = w;
    b.st->st[PHI_SIG_R] = sqrt(pv);
    b.st->st[W_SIG] = sqrt(wv);
    b.st->st[Z_EMIT] = sqrt(pv * wv - cv * cv);
  }
};

// XYReduceKernel + UpdateHorizontalAvgXYKernel (beam_kernel.cu:612-722, 1386-1395)
struct OpAvgXY {
  static constexpr int K = 2;
  using Comb = SumComb;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    if (!alive(b, i)) return;
    a[0] += b.x[i];
    a[1] += b.y[i];
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[X_AVG] = t[0] / surv(b);
    b.st->st[Y_AVG] = t[1] / surv(b);
  }
};

// MaxR2PhiReduceKernel + UpdateMaxRPhiKernel (beam_kernel.cu:793-931, 1378-1384)
struct OpMaxRPhi {
  static constexpr int K = 2;
  using Comb = MaxComb;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    if (!alive(b, i)) return;
    double tx = b.x[i] - b.st->st[X_AVG], ty = b.y[i] - b.st->st[Y_AVG];
    double r2 = tx * tx + ty * ty;
    double tp = b.phi_r[i] - b.st->st[PHI_AVG_R];
    tp = tp > 0.0 ? tp : -tp;
    a[0] = a[0] < r2 ? r2 : a[0];
    a[1] = a[1] < tp ? tp : a[1];
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[R_MAX] = sqrt(t[0]);
    b.st->st[ABS_PHI_MAX] = t[1];
  }
};

// ChangeFrequency (beam.cpp:1658-1669) after the phase rescale:
// UpdateAvgPhi() then UpdateRelativePhi() and UpdateAvgRelativePhi().  The
// relative phase depends on phi[0] only, so one sweep computes both sums.
struct OpFreqAverages {
  static constexpr int K = 2;
  using Comb = SumComb;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    double pr = rel_phase(b.phi[i], b.phi[0]);
    b.phi_r[i] = pr;
    if (!alive(b, i)) return;
    a[0] += b.phi[i];
    a[1] += pr;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[PHI_AVG] = t[0] / surv(b);
    b.st->st[PHI_AVG_R] = t[1] / surv(b);
  }
};

// Side-effect-free statistics record (HPS_MON_*)
struct OpMonitor {
  static constexpr int K = 17;
  using Comb = SumComb;
  DevBeam b;
  const ScState *sc;
  double *out;
  uint32_t elem;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    if (good(b, i)) a[16] += 1.0;
    if (!alive(b, i)) return;
    double pr = rel_phase(b.phi[i], b.phi[0]);
    double x = b.x[i], xp = b.xp[i], y = b.y[i], yp = b.yp[i], w = b.w[i];
    a[0] += 1.0;
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
    double g1 = b.w[0] / b.mass, bg = sqrt(g1 * (g1 + 2.0));
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
      o[HPS_MON_W_AVG] = w;
      o[HPS_MON_W_SIG] = sqrt(wv);
      o[HPS_MON_Z_EMIT] = sqrt(pv * wv - cv * cv);
    }
    o[HPS_MON_W0] = b.w[0];
    o[HPS_MON_PHI0] = b.phi[0];
    if (sc) {
      o[HPS_MON_SC_DR] = sc->dr;
      o[HPS_MON_SC_DZ] = sc->dz;
      o[HPS_MON_SC_REMESH] = (double)sc->n_solves;  // cumulative; the host takes differences
      o[HPS_MON_SC_ONMESH] = (double)sc->num_on_mesh;
    }
    o[HPS_MON_ELEM] = (double)elem;
  }
};

// ---- plain per-particle kernels ------------------------------------------

// UpdateRelativePhiKernel, beam_kernel.cu:1507-1525 (every particle)
__global__ void k_relative_phi(DevBeam b, int use_good) {
  double ref = use_good ? b.st->st[PHI_AVG_GOOD] : b.phi[0];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += gridDim.x * blockDim.x)
    b.phi_r[i] = rel_phase(b.phi[i], ref);
}

// UpdateLongitudinalLossCoordinateKernel, beam_kernel.cu:1550-1559
__global__ void k_lloss(DevBeam b) {
  double lim = b.st->st[PHI_AVG_GOOD];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += gridDim.x * blockDim.x)
    if (b.phi[i] > lim + TWOPI + PI) b.lloss[i] = 1u;
}

// ChangeFrequencyKernel, beam_kernel.cu:1532-1538
__global__ void k_scale_phi(DevBeam b, double r) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += gridDim.x * blockDim.x)
    b.phi[i] *= r;
}

// CutBeamKernel, beam_kernel.cu:1465-1481 (index 0 skipped)
__global__ void k_cut(DevBeam b, int coord, double lo, double hi) {
  const double *v = coord_of(b, coord);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += gridDim.x * blockDim.x) {
    if (i == 0) continue;
    if (b.loss[i] == 0u) {
      double x = v[i];
      if (x < hi && x > lo) b.loss[i] = 99999u;
    }
  }
}

// ShiftVariableKernel, beam_kernel.cu:1491-1497 (index 0 skipped)
__global__ void k_shift(DevBeam b, int coord, double val) {
  double *v = coord_of(b, coord);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += gridDim.x * blockDim.x)
    if (i > 0) v[i] += val;
}

__global__ void k_set0(DevBeam b, int coord, double val) {
  if (b.n) coord_of(b, coord)[0] = val;
}

}  // namespace

void beam_update_loss(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass(OpCount{b, 0}, b.n, s, st); note_launch();
}
void beam_update_lloss_count(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass(OpCount{b, 1}, b.n, s, st); note_launch();
}
void beam_update_good_count(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass(OpCount{b, 2}, b.n, s, st); note_launch();
}
void beam_update_avg(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st) {
  if (coord == HPS_COORD_XP || coord == HPS_COORD_YP) good = 0;
  launch_pass(OpMoment{b, coord, good, 0}, b.n, s, st); note_launch();
}
void beam_update_sig(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st) {
  if (b.n <= 2) return;  // Beam::UpdateSig*: num_particle > 2
  if (coord == HPS_COORD_XP || coord == HPS_COORD_YP || coord == HPS_COORD_PHI) good = 0;
  launch_pass(OpMoment{b, coord, good, 1}, b.n, s, st); note_launch();
}
void beam_update_emittance(const DevBeam &b, PassScratch s, cudaStream_t st) {
  if (b.n <= 2) return;
  launch_pass(OpEmittance{b}, b.n, s, st); note_launch();
}
void beam_update_relative_phi(const DevBeam &b, int use_good, cudaStream_t st) {
  k_relative_phi<<<grid_for(b.n), kBlock, 0, st>>>(b, use_good); note_launch();
}
// Beam::UpdateLongitudinalLoss, beam.cpp:776-782
void beam_update_longitudinal_loss(const DevBeam &b, PassScratch s, cudaStream_t st) {
  beam_update_good_count(b, s, st);
  beam_update_avg(b, HPS_COORD_PHI, 1, s, st);
  k_lloss<<<grid_for(b.n), kBlock, 0, st>>>(b); note_launch();
  beam_update_lloss_count(b, s, st);
}
void beam_update_avg_xy(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass(OpAvgXY{b}, b.n, s, st); note_launch();
}
void beam_update_max_r_phi(const DevBeam &b, PassScratch s, cudaStream_t st) {
  launch_pass(OpMaxRPhi{b}, b.n, s, st); note_launch();
}
void beam_change_frequency(const DevBeam &b, double ratio, PassScratch s, cudaStream_t st) {
  k_scale_phi<<<grid_for(b.n), kBlock, 0, st>>>(b, ratio); note_launch();
  launch_pass(OpFreqAverages{b}, b.n, s, st); note_launch();
}
void beam_apply_cut(const DevBeam &b, int coord, double lo, double hi, cudaStream_t st) {
  k_cut<<<grid_for(b.n), kBlock, 0, st>>>(b, coord, lo, hi); note_launch();
}
void beam_shift(const DevBeam &b, int coord, double val, cudaStream_t st) {
  k_shift<<<grid_for(b.n), kBlock, 0, st>>>(b, coord, val); note_launch();
}
void beam_set_ref(const DevBeam &b, int coord, double val, cudaStream_t st) {
  k_set0<<<1, 1, 0, st>>>(b, coord, val); note_launch();
}
void beam_monitor(const DevBeam &b, const ScState *sc, double *mon_dev, uint32_t elem, PassScratch s,
                  cudaStream_t st) {
  launch_pass(OpMonitor{b, sc, mon_dev, elem}, b.n, s, st); note_launch();
}

}  // namespace hps
