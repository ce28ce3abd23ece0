// push32.cu -- element transfer maps on FP32 particle state: host side.
//
// The synchronous particle (on axis, never kicked by space charge) is
// advanced on the host in FP64 through the same formulas the FP64 kernels
// apply (simulation_kernel.cu), so absolute phases (hundreds of radians
// after a DTL) and energies never pass through FP32.  Each launcher forms
// its element's map (push32_maps.cuh) from the synchronous particle before
// the element, moves the synchronous particle, and launches the map in one
// of three forms: alone; followed by the statistics of the space-charge
// kick that follows, taken from the new state in the same sweep; or preceded
// by the space-charge kick (sc32_kick.cuh), so that a kick and the element
// half after it are one sweep over the particles.
//
// Lost particles keep their absolute phase and energy (the reference's
// kernels skip them): every sweep moves their offsets against the
// synchronous particle's step through the element.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <unordered_map>

#include "internal.h"
#include "push32_maps.cuh"
#include "reduce.cuh"
#include "sc32_kick.cuh"
#include "sc32_stats.cuh"

namespace hps {

namespace {

#define PARTICLES(b) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (b).n; i += gridDim.x * blockDim.x)

double beta_of(double w, double mass) {
  double gm1 = w / mass;
  return sqrt(gm1 * (gm1 + 2.0)) / (gm1 + 1.0);
}

// the synchronous particle's step through an element, in FP32
struct Shift {
  float dph, dw;
};

// offsets of a lost particle after the element: absolute phase and energy kept
__device__ inline uint32_t keep_lost(Part &p, uint32_t w, const Shift &s) {
  if (s.dph != 0.0f) { p.ph -= s.dph; w |= WR_PH; }
  if (s.dw != 0.0f) { p.w -= s.dw; w |= WR_W; }
  return w;
}

// the map on a live particle, the shift on a lost one (or one the map loses)
template <class Map>
__device__ inline uint32_t step(Part &p, const Map &m, const Shift &s) {
  if (p.lo != 0u) return keep_lost(p, 0u, s);
  const uint32_t w = m.apply(p);
  return p.lo != 0u ? keep_lost(p, w, s) : w;
}

// Particle sweeps run on a grid that is resident at once (the SMs times the
// kernel's occupancy); a thread loads kSweepBatch particles before it works
// on the first, so each SM keeps enough loads in flight to cover latency.
constexpr int kSweepBatch = 2;

// cap: at most this many blocks per SM (0: as many as the SM holds)
int sweep_grid(const void *kernel, uint32_t n, uint32_t cap) {
  static std::mutex m;
  static std::unordered_map<const void *, int> resident;
  static int sms = 0;
  int r;
  {
    std::lock_guard<std::mutex> lock(m);
    if (!sms && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) sms = 152;
    int &rr = resident[kernel];
    if (!rr && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rr, kernel, kBlock, 0) != cudaSuccess || rr < 1)) rr = 1;
    r = rr;
  }
  if (cap && (uint32_t)r > cap) r = (int)cap;
  const uint64_t need = ((uint64_t)n + (uint64_t)kSweepBatch * kBlock - 1) / ((uint64_t)kSweepBatch * kBlock);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)r * sms));
}

template <class Map>
__device__ __forceinline__ void push_body(const DevBeam &b, const Map &m, const Shift &sh, uint32_t bid,
                                          uint32_t nblk) {
  const bool moves = sh.dph != 0.0f || sh.dw != 0.0f;
  const uint32_t stride = nblk * blockDim.x;
  for (uint32_t base = bid * blockDim.x + threadIdx.x; base < b.n; base += kSweepBatch * stride) {
    Part p[kSweepBatch];
#pragma unroll
    for (int u = 0; u < kSweepBatch; ++u)
      if (base + u * stride < b.n) p[u] = load_part(b, base + u * stride);
#pragma unroll
    for (int u = 0; u < kSweepBatch; ++u) {
      const uint32_t i = base + u * stride;
      if (i >= b.n || (p[u].lo != 0u && !moves)) continue;
      store_part(b, i, p[u], step(p[u], m, sh));
    }
  }
}

template <class Map>
__global__ void __launch_bounds__(kBlock) k32_push(DevBeam b, Map m, Shift sh) {
  push_body(b, m, sh, blockIdx.x, gridDim.x);
}

// The map, then every statistic the SCHEFF kick after it takes from the new
// state (UpdateStatForSpaceCharge and the longitudinal-loss test of
// Scheff::Start, space_charge.cpp:86-101; beam.cpp:776-852, 1008-1009) in
// the same sweep, and in the finaliser the decision and the kick's
// constants.  Phase sums are taken about s, the offset of <phi>_good from
// the synchronous particle at the last kick of this simulation call (zero at
// its first), an estimate of the new one: <phi>_good from the raw offsets,
// sigma_phi and the mean relative phase of the live particles from the
// phases wrapped about s, shifted.  Two max slots certify that these are the
// separate sweeps' answers: no particle lies above <phi>_good + 3 pi (the
// loss test flags none) and no relative phase lies within |<phi>_good - s|
// of a wrap boundary (it wraps about <phi>_good as about s).  Without the
// certificate the finaliser records the counts and <phi>_good and sets
// sc_redo = 2 for the loss-test and moments sweeps (one grid-wide launch
// after this one, sc32_stats_after_push); so it does when s lies more than 4
// sigma_phi from <phi>_good, where sigma_phi^2 as a difference of FP32
// moments about s would lose precision.
template <class Map>
struct OpPushScStats {
  // 0 good count, 1 sum d (raw, for <phi>_good), 2-3 sum f, f^2 (wrapped, for
  // sigma_phi), 4-8 x, x^2, y, y^2, W of the good set; 9 sum f, 10 count of the
  // live set; 11 lloss count; 12 max |f| over the live set; 13 max phi over
  // lloss != 1.  d = phi - s, f = wrap(d).
  static constexpr int K = 14;
  static constexpr int kMaxFrom = 12;
  static constexpr int kBatch = 4;
  static constexpr bool kFast = true;
  using Comb = SumComb;
  struct Ctx { float s; };
  struct P { Part p; uint32_t ll; };
  DevBeam b;  // carries the synchronous particle after the element
  Map m;
  Shift sh;
  int s_last;  // s from the last kick's <phi>_good offset (else 0)
  ScState *sc;
  ScTables tb;
  double freq, frac;
  Sc32Host h;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const {
    const float e = s_last ? tb.c32->pag : 0.0f;
    return {fabsf(e) < 3.14159265f ? e : 0.0f};
  }
  __device__ P load(uint32_t i) const { return {load_part(b, i), b.lloss[i]}; }
  __device__ void use(uint32_t i, const P &q, float (&a)[K], const Ctx &c) const {
    Part p = q.p;
    const uint32_t w = step(p, m, sh);
    if (w) store_part(b, i, p, w);
    const bool alive = p.lo == 0u, g = alive && q.ll == 0u;
    const float d = p.ph - c.s, f = rel_phase_f(d);
    a[0] += g ? 1.0f : 0.0f;
    a[1] += g ? d : 0.0f;
    a[2] += g ? f : 0.0f;
    a[3] += g ? f * f : 0.0f;
    a[4] += g ? p.x : 0.0f;
    a[5] += g ? p.x * p.x : 0.0f;
    a[6] += g ? p.y : 0.0f;
    a[7] += g ? p.y * p.y : 0.0f;
    a[8] += g ? p.w : 0.0f;
    a[9] += alive ? f : 0.0f;
    a[10] += alive ? 1.0f : 0.0f;
    a[11] += q.ll != 0u ? 1.0f : 0.0f;
    if (alive) a[12] = fmaxf(a[12], fabsf(f));
    if (q.ll != 1u) a[13] = fmaxf(a[13], p.ph);
  }
  __device__ void finalize(const double *t, int tid, int nth) const {
    __shared__ int ok;
    if (tid == 0) {
      BeamStats &st = *b.st;
      const float s = setup().s;
      const uint32_t ng = (uint32_t)t[0];
      const double pag_abs = ng > 0 ? (double)(s + (float)t[1] / (float)ng) + b.phi_ref : -99999.0;
      st.num_good = ng;
      st.num_lloss = (uint32_t)t[11];
      st.st[PHI_AVG_GOOD] = pag_abs;
      // the loss test's limit and the relative-phase origin, as the sweeps take them
      const float lim = (float)(pag_abs - b.phi_ref + TWOPI + PI);
      const float dm = (float)(pag_abs - b.phi_ref) - s;
      // sigma_phi^2 = <f^2> - <f>^2 keeps FP32 precision while |<f>| <= 4 sigma
      const float ing = 1.0f / (float)ng, mf = (float)t[2] * ing, var = (float)t[3] * ing - mf * mf;
      ok = ng > 0 && (float)t[13] <= lim && (float)t[12] < 3.14159265f - fabsf(dm) - 1.0e-3f &&
           mf * mf <= 16.0f * var;
      if (ok) {
        // wrap(phi - <phi>_good) = f - dm on the live set: the totals of the
        // moments sweep (sigma_phi from the f moments, shift-invariant)
        double sm[8];
        sm[0] = (float)t[9] - (float)t[10] * dm;
        for (int k = 1; k < 8; ++k) sm[k] = t[k + 1];
        st.sc_redo = 0u;
        sc_moments_finish(b, sm, sc, tb, freq, frac, h);
      } else {
        st.sc_redo = 2u;
      }
    }
    __syncthreads();
    if (ok) zero_mesh_tables(sc, tb, tid, nth);
  }
};

// ApplySpchKickKernel on the particles it kicks (alive, not longitudinally
// lost, outside the skipped set), then the map on every live particle
template <class Map>
__device__ __forceinline__ void kick_push_body(const DevBeam &b, const ScState *sc, const ScTables &t, const RefK &rk,
                                               uint64_t skip_mask, const Map &m, const Shift &sh, uint32_t bid,
                                               uint32_t nblk) {
  const KickEnv e = kick_env(sc, t, rk);
  const bool moves = sh.dph != 0.0f || sh.dw != 0.0f;
  const uint32_t stride = nblk * blockDim.x;
  for (uint32_t base = bid * blockDim.x + threadIdx.x; base < b.n; base += kSweepBatch * stride) {
    Part p[kSweepBatch];
    uint32_t ll[kSweepBatch];
#pragma unroll
    for (int u = 0; u < kSweepBatch; ++u) {
      const uint32_t i = base + u * stride;
      if (i < b.n) {
        p[u] = load_part(b, i);
        ll[u] = b.lloss[i];
      }
    }
#pragma unroll
    for (int u = 0; u < kSweepBatch; ++u) {
      const uint32_t i = base + u * stride;
      if (i >= b.n || (p[u].lo != 0u && !moves)) continue;
      uint32_t w = 0;
      if (p[u].lo == 0u && ll[u] == 0u && ((uint64_t)i & skip_mask) != 0)
        w = kick_particle(p[u], rel_phase_f(p[u].ph - e.pag), e);
      w |= step(p[u], m, sh);
      store_part(b, i, p[u], w);
    }
  }
}

template <class Map>
__global__ void __launch_bounds__(kBlock) k32_kick_push(DevBeam b, const ScState *sc, ScTables t, RefK rk,
                                                       uint64_t skip_mask, Map m, Shift sh) {
  kick_push_body(b, sc, t, rk, skip_mask, m, sh, blockIdx.x, gridDim.x);
}

// lockstep forms: one beam's share of a merged launch
template <class Map>
struct PushSeg {
  DevBeam b;
  Map m;
  Shift sh;
};
template <class Map, int B>
__global__ void __launch_bounds__(kBlock) k32_push_seg(const __grid_constant__ SegArgs<PushSeg<Map>, B> a) {
  uint32_t bid, nblk;
  const PushSeg<Map> &p = a.p[seg_find(a, blockIdx.x, bid, nblk)];
  push_body(p.b, p.m, p.sh, bid, nblk);
}
template <class Map>
struct KickPushSeg {
  DevBeam b;
  const ScState *sc;
  ScTables t;
  RefK rk;
  uint64_t skip_mask;
  Map m;
  Shift sh;
};
template <class Map, int B>
__global__ void __launch_bounds__(kBlock) k32_kick_push_seg(const __grid_constant__ SegArgs<KickPushSeg<Map>, B> a) {
  uint32_t bid, nblk;
  const KickPushSeg<Map> &p = a.p[seg_find(a, blockIdx.x, bid, nblk)];
  kick_push_body(p.b, p.sc, p.t, p.rk, p.skip_mask, p.m, p.sh, bid, nblk);
}
template <class Map>
void push_merge(const std::vector<const Rec *> &recs, SegFork &, cudaStream_t st, cudaStream_t) {
  seg_chunks<PushSeg<Map>>(recs, [&](const auto &a, uint32_t blocks) {
    k32_push_seg<Map, std::decay_t<decltype(a)>::kB><<<blocks, kBlock, 0, st>>>(a);
  });
}
template <class Map>
void kick_push_merge(const std::vector<const Rec *> &recs, SegFork &, cudaStream_t st, cudaStream_t) {
  seg_chunks<KickPushSeg<Map>>(recs, [&](const auto &a, uint32_t blocks) {
    k32_kick_push_seg<Map, std::decay_t<decltype(a)>::kB><<<blocks, kBlock, 0, st>>>(a);
  });
}

// b carries the synchronous particle after the element; rk is it before
// (the kick of PUSH_AFTER_KICK happens there), phi0 / w0 its phase and energy
template <class Map>
void launch_map(const DevBeam &b, const Map &m, const RefK &rk, double phi0, double w0, cudaStream_t st,
                const PushFuse *pf) {
  const Shift sh{(float)(b.phi_ref - phi0), (float)(b.w_ref - w0)};
  if (recorder()) {  // a lockstep range is being recorded
    if (!pf) {
      record("push", &push_merge<Map>, (uint32_t)sweep_grid((const void *)k32_push<Map>, b.n, b.sweep_cap),
             PushSeg<Map>{b, m, sh});
    } else if (pf->mode == PUSH_SCSTATS) {
      launch_pass_f(OpPushScStats<Map>{b, m, sh, pf->s_last, pf->sc, pf->t, pf->freq, pf->frac, pf->h}, b.n, pf->scr,
                    st, b.sweep_cap, "push_scstats");
    } else {
      record("kick_push", &kick_push_merge<Map>,
             (uint32_t)sweep_grid((const void *)k32_kick_push<Map>, b.n, b.sweep_cap),
             KickPushSeg<Map>{b, (const ScState *)pf->sc, pf->t, rk, pf->skip_mask, m, sh});
    }
    return;
  }
  if (!pf) {
    launch_k(k32_push<Map>, dim3(sweep_grid((const void *)k32_push<Map>, b.n, b.sweep_cap)), dim3(kBlock), 0, st, b,
             m, sh);
  } else if (pf->mode == PUSH_SCSTATS) {
    launch_pass_f(OpPushScStats<Map>{b, m, sh, pf->s_last, pf->sc, pf->t, pf->freq, pf->frac, pf->h}, b.n, pf->scr,
                  st, b.sweep_cap);
  } else {
    launch_k(k32_kick_push<Map>, dim3(sweep_grid((const void *)k32_kick_push<Map>, b.n, b.sweep_cap)), dim3(kBlock),
             0, st, b, (const ScState *)pf->sc, pf->t, rk, pf->skip_mask, m, sh);
  }
  note_launch();
}

struct AptArgs {
  DevBeam b;
  int rect;
  float aper, xl, xr, yt, yb;
  uint32_t eid;
};
__device__ __forceinline__ void aperture_body(const AptArgs &a, uint32_t bid, uint32_t nblk) {
  const DevBeam &b = a.b;
  const float cx = (float)b.st->st[X_AVG], cy = (float)b.st->st[Y_AVG];
  const int rect = a.rect;
  const float aper = a.aper, xl = a.xl, xr = a.xr, yt = a.yt, yb = a.yb;
  const uint32_t eid = a.eid;
  for (uint32_t i = bid * blockDim.x + threadIdx.x; i < b.n; i += nblk * blockDim.x) {
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
__global__ void k32_aperture(AptArgs a) { aperture_body(a, blockIdx.x, gridDim.x); }
template <int B>
__global__ void k32_aperture_seg(const __grid_constant__ SegArgs<AptArgs, B> a) {
  uint32_t bid, nblk;
  aperture_body(a.p[seg_find(a, blockIdx.x, bid, nblk)], bid, nblk);
}
void aperture_merge(const std::vector<const Rec *> &recs, SegFork &, cudaStream_t st, cudaStream_t) {
  seg_chunks<AptArgs>(recs, [&](const auto &a, uint32_t blocks) {
    k32_aperture_seg<std::decay_t<decltype(a)>::kB><<<blocks, kBlock, 0, st>>>(a);
  });
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
// launchers: FP64 reference update on the host, FP32 map for the particles
// ---------------------------------------------------------------------------
void push32_partial_drift(DevBeam &b, double wl, double hf, double aper, uint32_t eid, cudaStream_t st,
                          const PushFuse *pf) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const RefK r = make_refk(b.w_ref, b.mass);
  const DriftMap m{r, (float)hf, (float)(aper * aper), (float)(TWOPI * hf / wl), eid};
  b.phi_ref += TWOPI * hf / (wl * beta_of(b.w_ref, b.mass));
  launch_map(b, m, r, phi0, w0, st, pf);
}

void push32_half_quad(DevBeam &b, double wl, double len, double aper, double grad, uint32_t eid, cudaStream_t st,
                      const PushFuse *pf) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const RefK r = make_refk(b.w_ref, b.mass);
  const double qg = grad * b.charge;
  QuadMap m{};
  m.r = r;
  m.len = (float)len;
  m.aper2 = (float)(aper * aper);
  m.qg = (float)qg;
  m.c = (float)(TWOPI * len * 0.5 / wl);
  m.eid = eid;
  if (qg != 0.0) {  // the synchronous particle's k ds / 4 and its functions, in FP64
    const double kcoef = fabs(qg) * CLIGHT / b.mass;
    const double gr = b.w_ref / b.mass;
    const double kds = len * 0.25 * sqrt(kcoef / sqrt(gr * (gr + 2.0)));
    m.sk0 = (float)sqrt(kcoef);
    m.isk0 = (float)(1.0 / sqrt(kcoef));
    m.kds_r = (float)kds;
    m.s_r = (float)sin(kds);
    m.c_r = (float)cos(kds);
    m.sh_r = (float)sinh(kds);
    m.ch_r = (float)cosh(kds);
  }
  b.phi_ref += TWOPI * len * 0.5 / (wl * beta_of(b.w_ref, b.mass));
  launch_map(b, m, r, phi0, w0, st, pf);
}

void push32_steerer(DevBeam &b, double blh, double blv, cudaStream_t st) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const RefK r = make_refk(b.w_ref, b.mass);
  const float kh = blh > 1e-10 ? (float)(blh * b.charge * CLIGHT / b.mass) : 0.0f;
  const float kv = blv > 1e-10 ? (float)(blv * b.charge * CLIGHT / b.mass) : 0.0f;
  launch_map(b, SteerMap{r, kh, kv}, r, phi0, w0, st, nullptr);
}

void push32_gap_first(DevBeam &b, const GapArgs &g, cudaStream_t st, const PushFuse *pf) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const RefK r = make_refk(b.w_ref, b.mass);
  const double mass = b.mass;
  const double wave_len = CLIGHT / g.frequency;
  const double cell_len = g.length + g.q1 * 0.5 + g.q2 * 0.5;
  const double dd1 = 0.5 * cell_len - g.dg - 0.5 * g.q1;
  double K, dphi_ref;
  const double bref = beta_of(b.w_ref, mass);
  if (g.amplitude == 0.0) {
    K = TWOPI * dd1 / wave_len;
    dphi_ref = TWOPI * dd1 / (wave_len * bref);
  } else {
    double gam = g.design_w_in / mass;
    const double beta_in = sqrt((gam + 2.0) * gam) / (gam + 1.0);
    gam = b.w_ref / mass;
    const double beta = sqrt((gam + 2.0) * gam) / (gam + 1.0);
    const double dps = g.phase_ref - g.phi_in;
    const double A = PI * g.clbl + dps;
    if (!g.ccl) {
      const double d_cell_len = cell_len - g.beta_center * wave_len;
      const double dphi_qlen1 = TWOPI * 0.5 * g.q1 / (beta * wave_len);
      double dphi_clen = 0.0;
      const bool dc = d_cell_len > 1e-15 || d_cell_len < -1e-15;
      if (dc) dphi_clen = PI * d_cell_len / (beta * wave_len);
      dphi_ref = (1.0 - (beta - beta_in) / beta) * A + dphi_clen - dphi_qlen1;
      K = beta_in * A + (dc ? PI * d_cell_len / wave_len : 0.0) - PI * g.q1 / wave_len;
    } else {
      const double betag = cell_len / (g.clbl * wave_len);
      dphi_ref = (1.0 - (beta - beta_in) * betag / (beta * beta_in)) * A;
      K = betag * A;
    }
  }
  b.phi_ref += dphi_ref;
  launch_map(b, Gap1Map{r, (float)dd1, (float)K}, r, phi0, w0, st, pf);
}

void push32_gap_second(DevBeam &b, const GapArgs &g, cudaStream_t st, const PushFuse *pf) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const double mass = b.mass;
  const RefK rkick = make_refk(b.w_ref, mass);
  Gap2Map G{};
  G.rin = rkick;
  const double cell_len = g.length + g.q1 * 0.5 + g.q2 * 0.5;
  const double dd2 = 0.5 * cell_len + g.dg - g.q2 * 0.5;
  G.dd2 = (float)dd2;
  G.drift_c = (float)(TWOPI * dd2 / g.wl);
  const double inv_mass = 1.0 / mass;
  const double gm_in = g.design_w_in * inv_mass + 1.0;
  const double beta_in = sqrt(1.0 - 1.0 / (gm_in * gm_in));
  const double gam = b.w_ref * inv_mass;
  const double bg1 = sqrt(gam * (gam + 2.0));
  const double beta = bg1 / (gam + 1.0);
  // transit-time factors of the reference, as in the FP64 kernel
  double bcl = beta;
  if (beta > 1.1 * g.fbc) bcl = g.fbc;
  else if (beta < g.fbm) bcl = g.fbm;
  const double *ta = g.ta, *sa = g.sa;
  const double t_r = ta[0] + bcl * (ta[1] + bcl * (ta[2] + bcl * (ta[3] + bcl * (ta[4] + bcl * ta[5]))));
  const double coef = bcl * bcl / (TWOPI * g.fbc);
  const double tp_r = coef * (ta[1] + bcl * (2 * ta[2] + bcl * (3 * ta[3] + bcl * (4 * ta[4] + 5 * bcl * ta[5]))));
  const double sp_r = -coef * (sa[0] + bcl * (2 * sa[1] + bcl * (3 * sa[2] + bcl * (4 * sa[3] + 5 * bcl * sa[4]))));
  double tcoef[6], scoef[6];
  const double sfull[6] = {0.0, sa[0], sa[1], sa[2], sa[3], sa[4]};
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
  const bool ref_drift = g.amplitude == 0.0 || (g.ccl && beta < g.fbm);
  G.ref_drift = ref_drift;
  const double dphi_drift_ref = TWOPI * dd2 / (g.wl * beta);
  double phi_h, w_h;  // reference after a kick (hypothetical if it drifts)
  const double wave_len = CLIGHT / g.frequency;
  if (g.amplitude != 0.0) {
    const double cl = cell_len / g.clbl;
    const double betag_ccl = cl / wave_len;
    const double betag = g.ccl ? g.beta_center : betag_ccl;
    const double betag2 = betag * betag;
    const double gmg = 1.0 / sqrt(1.0 - betag2);
    const double inv_gmg2 = 1.0 / (gmg * gmg);
    const double q = fabs(b.charge);
    const double gm_out = g.energy_out * inv_mass + 1.0;
    const double beta_out = sqrt(1.0 - 1.0 / (gm_out * gm_out));
    const double efl = g.amplitude * cell_len;
    const double concomm = q * efl / (mass * betag2);
    const double concomm1 = concomm * inv_gmg2 / gmg;
    const double con1 = PI * concomm1;
    const double con2nex = concomm * inv_gmg2;
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
    const double fkr = TWOPI * inv_gmgcl;
    const double sinps = sin(g.phase_ref), cosps = cos(g.phase_ref);
    double phi1;
    if (g.ccl) phi1 = b.phi_ref + g.phase_shift - TWOPI * g.dg / (beta * wave_len) + g.ccl_cell_num * PI;
    else phi1 = b.phi_ref + g.phase_shift;
    const double sinp1 = sin(phi1), cosp1 = cos(phi1);
    const double prome1 = -con1 * (tp_r * (sinp1 - sinps) + sp_r * (cosp1 - cosps));
    const double P = phi1 + prome1;
    const double sinP = sin(P), cosP = cos(P);
    // on axis: b0c = 1, b1c = 0, b1p = 0.5, rrp = 0
    const double delte = q * efl * (tw * cosP);
    w_h = b.w_ref + delte;
    const double gh = w_h * inv_mass;
    const double bgh = sqrt(gh * (gh + 2.0));
    const double beta_h = bgh / (gh + 1.0);
    const double prome = 2.0 * con1 * (-tp_r) * (sinP - sinps);
    const double A = PI * g.clbl + (g.ccl ? (g.phi_in - g.phase_ref) : (g.phase_ref - g.phi_in));
    double K2;
    if (g.ccl) {
      phi_h = b.phi_ref + (1.0 - (beta_h - beta_out) * betag_ccl / (beta_h * beta_out)) * A + prome;
      K2 = betag_ccl * A;
    } else {
      const double d_cell_len = cell_len - g.beta_center * wave_len;
      const double dphi_qlen2 = TWOPI * 0.5 * g.q2 / (beta_h * wave_len);
      const bool dc = d_cell_len > 1e-15 || d_cell_len < -1e-15;
      const double dphi_clen = dc ? PI * d_cell_len / (beta_h * wave_len) : 0.0;
      phi_h = b.phi_ref + (1.0 - (beta_h - beta_out) / beta_h) * A + prome + dphi_clen - dphi_qlen2;
      K2 = beta_out * A + (dc ? PI * d_cell_len / wave_len : 0.0) - PI * g.q2 / wave_len;
    }
    G.beta_in = (float)beta_in; G.inv_beta_in = (float)(1.0 / beta_in); G.betag_ccl = (float)betag_ccl;
    G.gmg = (float)gmg; G.inv_gmg = (float)(1.0 / gmg); G.q = (float)q;
    G.efl = (float)efl; G.efl_m = (float)(efl * inv_mass); G.concomm = (float)concomm;
    G.concomm1 = (float)concomm1; G.con1 = (float)con1; G.con2nex = (float)con2nex;
    G.inv_gmg2 = (float)inv_gmg2; G.inv_gmgcl = (float)inv_gmgcl; G.inv_fkis = (float)inv_fkis;
    G.fkr = (float)fkr; G.sinps = (float)sinps; G.cosps = (float)cosps; G.X = (float)X;
    G.ccl_dg = (float)(TWOPI * g.dg / wave_len);
    const double F = fmod(phi1, TWOPI), Pm = fmod(P, TWOPI);
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
  const double phi_new = ref_drift ? b.phi_ref + dphi_drift_ref : phi_h;
  const double w_new = ref_drift ? b.w_ref : w_h;
  G.dphi_ref = (float)(phi_new - b.phi_ref);
  G.dw_ref = (float)(w_new - b.w_ref);
  G.corr_phi = (float)(phi_h - phi_new);
  G.corr_w = (float)(w_h - w_new);
  b.phi_ref = phi_new;
  b.w_ref = w_new;
  launch_map(b, G, rkick, phi0, w0, st, pf);
}

void push32_buncher(DevBeam &b, double wl, double w_ref_design, double freq, double voltage, double phase,
                    double aper, double freq_ratio, uint32_t eid, cudaStream_t st) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const double mass = b.mass;
  BunchMap B{};
  B.r = make_refk(b.w_ref, mass);
  const double h = freq * wl / CLIGHT;
  const double gm1 = w_ref_design / mass;
  const double gm = gm1 + 1.0;
  const double btgm = sqrt(gm1 * (gm1 + 2.0));
  const double beta = btgm / gm;
  const double k = h * TWOPI / (btgm * wl);
  const double q = fabs(b.charge);
  const double con1 = TWOPI * h * voltage * q / (beta * wl * mass);
  const double ph = fmod(h * b.phi_ref * freq_ratio + phase, TWOPI);
  B.hr = (float)(h * freq_ratio);
  B.sinB = (float)sin(ph);
  B.cosB = (float)cos(ph);
  B.k2q = (float)(k * k * 0.25);
  B.qV = (float)(q * voltage);
  B.con1 = (float)con1;
  B.beta_w = (float)beta;
  B.aper2 = (float)(aper * aper);
  B.eid = eid;
  b.w_ref += q * voltage * cos(h * b.phi_ref * freq_ratio + phase);
  launch_map(b, B, B.r, phi0, w0, st, nullptr);
}

void push32_rotation(DevBeam &b, double angle, cudaStream_t st) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  launch_map(b, RotMap{(float)cos(angle), (float)sin(angle)}, RefK{}, phi0, w0, st, nullptr);
}

void push32_aperture(DevBeam &b, int rect, const double *p, uint32_t eid, cudaStream_t st) {
  const AptArgs a{b, rect, (float)p[HPS_P_APERTURE], (float)p[HPS_P_APT_XL], (float)p[HPS_P_APT_XR],
                  (float)p[HPS_P_APT_YT], (float)p[HPS_P_APT_YB], eid};
  if (recorder()) {
    record("aperture", &aperture_merge, (uint32_t)grid_for(b.n), a);
    return;
  }
  launch_k(k32_aperture, dim3(grid_for(b.n)), dim3(kBlock), 0, st, a);
  note_launch();
}

void push32_dipole(DevBeam &b, const double *p, double wl, int second, cudaStream_t st, const PushFuse *pf) {
  const double phi0 = b.phi_ref, w0 = b.w_ref;
  const double mass = b.mass;
  const RefK rkick = make_refk(b.w_ref, mass);
  const double h = 1.0 / p[HPS_P_DIP_RADIUS];
  const double findx = p[HPS_P_DIP_FIELD_INDEX];
  const double design_w = p[HPS_P_DIP_KINETIC_ENERGY];
  const double h2 = h * h;
  const double dl = 0.5 * p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE];
  const double yk2 = findx * h2, yk = sqrt(fabs(yk2)), inv_yk = 1.0 / yk, ykl = yk * dl;
  const double xk2 = h2 - yk2, inv_xk2 = 1.0 / xk2, xk = sqrt(fabs(xk2)), inv_xk = 1.0 / xk, xkl = xk * dl;
  double cxkl = 1.0, sxokx = dl;
  if (xk2 > 0.0) { cxkl = cos(xkl); sxokx = sin(xkl) * inv_xk; }
  else if (xk2 < 0.0) { cxkl = cosh(xkl); sxokx = sinh(xkl) * inv_xk; }
  double cykl = 1.0, syoky = dl;
  if (yk2 > 0.0) { cykl = cos(ykl); syoky = sin(ykl) * inv_yk; }
  else if (yk2 < 0.0) { cykl = cosh(ykl); syoky = sinh(ykl) * inv_yk; }
  const double gamma = design_w / mass + 1.0;
  const double beta2 = 1.0 - 1.0 / (gamma * gamma);
  const double beta = sqrt(beta2);
  const double r26 = h * sxokx, r16 = h * (1.0 - cxkl) * inv_xk2;
  const double r56 = -h2 * (dl * beta2 - sxokx) * inv_xk2 + dl * (1.0 - h2 * inv_xk2) / (gamma * gamma);
  const double bedge = second ? p[HPS_P_DIP_EDGE_OUT] : p[HPS_P_DIP_EDGE_IN];
  const double c1 = 2.0 * p[HPS_P_DIP_HALF_GAP] * p[HPS_P_DIP_K1] * h;
  const double sinb = sin(bedge), inv_cosb = 1.0 / cos(bedge);
  const double psi = c1 * (1.0 + sinb * sinb) * inv_cosb * (1.0 - c1 * p[HPS_P_DIP_K2] * sinb * inv_cosb);
  const double cdp = gamma / (design_w * (gamma + 1.0));
  const double dpop_ref = cdp * (b.w_ref - design_w);
  DipMap d;
  d.r11 = (float)cxkl; d.r12 = (float)sxokx; d.r16 = (float)r16; d.r21 = (float)(-xk2 * sxokx); d.r22 = (float)cxkl;
  d.r26 = (float)r26; d.r33 = (float)cykl; d.r34 = (float)syoky; d.r43 = (float)(-yk2 * syoky); d.r44 = (float)cykl;
  d.r51 = (float)(-r26); d.r52 = (float)(-r16); d.r56 = (float)r56;
  d.e21 = (float)(tan(bedge) * h); d.e43 = (float)(tan(bedge - psi) * h);
  d.cdp = (float)cdp; d.dpop_ref = (float)dpop_ref; d.cph = (float)(TWOPI / (beta * wl));
  d.second = second;
  b.phi_ref += TWOPI * (-(r56 * dpop_ref) + dl) / (beta * wl);
  launch_map(b, d, rkick, phi0, w0, st, pf);
}

}  // namespace hps
