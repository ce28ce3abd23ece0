// scheff32.cu -- the SCHEFF 2D r-z space-charge kick on FP32 particle state.
//
// Same launch sequence and device-side decision as scheff.cu (Scheff::Start,
// src/simulation/src/space_charge.cpp:82-139; kernels of
// src/simulation/inc/space_charge_kernel.cu).  Differences:
//  * statistics sweeps accumulate offsets in FP32 per thread and warp, FP64
//    across warps and blocks (reduce.cuh: pass_kernel_f);
//  * the thread that takes the space-charge decision also forms every
//    constant the FP32 kernels of the kick need (Sc32Consts), in FP32
//    arithmetic from host-side constants, so no particle kernel and no
//    finaliser does FP64 arithmetic beyond a few adds (GB300 runs FP64 at
//    1/64 rate, and a dependent FP64 divide costs about a microsecond);
//  * ahead of a kick on four or more particles, the element half before it
//    takes every statistics sweep in its own sweep (push32.cu,
//    OpPushScStats) and certifies that the loss test flags no particle
//    and that no relative phase wraps; only when it cannot, the loss test
//    and the moments run here in one small launch (Op32LlossScStats, whose
//    last block sweeps the moments again when the good set changed).  The
//    kick runs inside the element half after it;
//  * relative phases are not stored: the deposit and the kick form
//    wrap(phi - <phi>_good) from the phase offset and Sc32Consts::pag;
//  * the deposit keeps a 32-bit fixed-point histogram per block in shared
//    memory (scale chosen from the block's particle count so that no bin can
//    overflow) and adds it to the 2^-36 global table as integers, so the
//    charge table is independent of arrival order;
//  * the Green's table is evaluated in FP32 with the elliptic-integral fits
//    rearranged so the far field is not a difference of O(1) terms, and the
//    ring-to-mesh contraction runs in FP32 from shared-memory tiles;
//  * the kick forms the bunch-frame momentum p* = gamma_c (beta gamma -
//    beta_c gamma) and the lab momentum change from differences that do not
//    cancel in FP32: p* = (gamma - gamma_c)(gamma + gamma_c) /
//    (gamma_c (beta gamma + beta_c gamma)), and with the exact inverse
//    transform beta gamma = gamma_c (p* + beta_c sqrt(1 + p*^2)), the
//    reference's bgzf - bgz = gamma_c (dp + beta_c [dp (2 p* + dp) / 2 +
//    p*^4 / (4 (1 + p*^2/2 + sqrt(1 + p*^2)))]).
// Particle kernels load a particle's flags and coordinates together and
// predicate the stores, so each particle costs one memory round trip.
#include <cooperative_groups.h>

#include <algorithm>
#include <vector>

#include "../../include/hpsim_gb300.h"
#include "internal.h"
#include "reduce.cuh"
#include "sc32_kick.cuh"
#include "contract.cuh"
#include "contract_tc.cuh"
#include "green32.cuh"
#include "sc32_stats.cuh"
#include "scheff_common.cuh"

namespace hps {

namespace {

struct NoCtx {};

// UpdateGoodParticleCount + UpdateAvgPhi(true)
struct Op32GoodPhi {
  static constexpr int K = 2;
  static constexpr bool kFast = true;
  using Comb = SumComb;
  using Ctx = NoCtx;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {}; }
  struct P { uint32_t lo, ll; float ph; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.lloss[i], b.fphi[i]}; }
  __device__ void use(uint32_t, const P &p, float (&a)[K], const Ctx &) const {
    bool g = (uint32_t)(p.lo + p.ll) == 0u;
    a[0] += g ? 1.0f : 0.0f;
    a[1] += g ? p.ph : 0.0f;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t ng = (uint32_t)t[0];
    b.st->num_good = ng;
    b.st->st[PHI_AVG_GOOD] = ng > 0 ? (double)((float)t[1] / (float)ng) + b.phi_ref : -99999;
  }
};

// longitudinal-loss test + lloss count + good count + <phi>_good
struct Op32LlossGoodPhi {
  static constexpr int K = 3;
  static constexpr bool kFast = true;
  using Comb = SumComb;
  struct Ctx { float lim; };
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {(float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref + TWOPI + PI)}; }
  struct P { uint32_t lo, ll; float ph; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.lloss[i], b.fphi[i]}; }
  __device__ void use(uint32_t i, const P &p, float (&a)[K], const Ctx &c) const {
    uint32_t ll = p.ll;
    if (p.ph > c.lim && ll != 1u) {
      ll = 1u;
      b.lloss[i] = 1u;
    }
    bool g = (uint32_t)(p.lo + ll) == 0u;
    a[0] += ll != 0u ? 1.0f : 0.0f;
    a[1] += g ? 1.0f : 0.0f;
    a[2] += g ? p.ph : 0.0f;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t ng = (uint32_t)t[1];
    b.st->num_lloss = (uint32_t)t[0];
    b.st->num_good = ng;
    b.st->st[PHI_AVG_GOOD] = ng > 0 ? (double)((float)t[2] / (float)ng) + b.phi_ref : -99999;
  }
};

// accumulate particle p into the SCHEFF moments (pr: its relative phase)
// relative phase about <phi>_good, the SCHEFF moments, the decision and the
// kick's constants (as OpScStats in scheff.cu).  With redo_only it runs only
// when the loss-test sweep below changed the good set (sc_redo == 1).
struct Op32ScStats {
  static constexpr int K = 8;
  static constexpr bool kFast = true;
  using Comb = SumComb;
  struct Ctx { float pag; };
  DevBeam b;
  ScState *sc;
  ScTables t;
  double freq, frac;
  Sc32Host h;
  int redo_only;
  __device__ bool enabled() const { return !redo_only || b.st->sc_redo == 1u; }
  __device__ Ctx setup() const { return {(float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref)}; }
  struct P { uint32_t lo, ll; float ph, x, y, w; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.lloss[i], b.fphi[i], b.fx[i], b.fy[i], b.fw[i]}; }
  __device__ void use(uint32_t i, const P &p, float (&a)[K], const Ctx &c) const {
    const float pr = rel_phase_f(p.ph - c.pag);
    b.fphi_r[i] = pr;
    const float alive = p.lo == 0u ? 1.0f : 0.0f;
    const float gd = (p.lo == 0u && p.ll == 0u) ? 1.0f : 0.0f;
    a[0] += alive * pr;
    a[1] += gd * pr; a[2] += gd * pr * pr;
    a[3] += gd * p.x; a[4] += gd * p.x * p.x; a[5] += gd * p.y; a[6] += gd * p.y * p.y;
    a[7] += gd * p.w;
  }
  __device__ void finalize(const double *s, int tid, int nth) const {
    if (tid == 0) {
      sc_moments_finish(b, s, sc, t, freq, frac, h);
      b.st->sc_redo = 0u;
    }
    if (!sc) return;
    __syncthreads();
    zero_mesh_tables(sc, t, tid, nth);
  }
};

// The longitudinal-loss test (UpdateLongitudinalLossCoordinateKernel with the
// lloss and good counts and <phi>_good, beam.cpp:780-781, 1008-1009) and the
// SCHEFF moments in one sweep, when the element map before the kick could
// not certify its own statistics (sc_redo == 2).  The relative phases are
// taken about the <phi>_good that sweep recorded; when the test flags no
// particle of the good set, that is the <phi>_good the separate sweeps would
// have used, and the totals are the same ones in the same order.  Otherwise
// the sweep records the new <phi>_good and asks for the moments sweep again
// (sc_redo = 1).
struct Op32LlossScStats {
  static constexpr int K = 12;
  static constexpr bool kFast = true;
  using Comb = SumComb;
  struct Ctx { float lim, pag; };
  DevBeam b;
  ScState *sc;
  ScTables t;
  double freq, frac;
  Sc32Host h;
  __device__ bool enabled() const { return b.st->sc_redo == 2u; }
  __device__ Ctx setup() const {
    const double pag = b.st->st[PHI_AVG_GOOD] - b.phi_ref;
    return {(float)(pag + TWOPI + PI), (float)pag};
  }
  struct P { uint32_t lo, ll; float ph, x, y, w; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.lloss[i], b.fphi[i], b.fx[i], b.fy[i], b.fw[i]}; }
  __device__ void use(uint32_t i, const P &p, float (&a)[K], const Ctx &c) const {
    uint32_t ll = p.ll;
    float newly = 0.0f;
    if (p.ph > c.lim && ll != 1u) {
      if (p.lo == 0u && ll == 0u) newly = 1.0f;
      ll = 1u;
      b.lloss[i] = 1u;
    }
    const float pr = rel_phase_f(p.ph - c.pag);
    b.fphi_r[i] = pr;
    sc_moments_add(a, pr, p.lo, ll, p.x, p.y, p.w);
    const bool g = (uint32_t)(p.lo + ll) == 0u;
    a[8] += ll != 0u ? 1.0f : 0.0f;
    a[9] += g ? 1.0f : 0.0f;
    a[10] += g ? p.ph : 0.0f;
    a[11] += newly;
  }
  __device__ void finalize(const double *s, int tid, int nth) const {
    __shared__ int redo;
    __shared__ float red[kBlock / 32][8];
    __shared__ double mom[8];
    if (tid == 0) {
      sc->n_stat_sweeps += 1;
      BeamStats &st = *b.st;
      const uint32_t ng = (uint32_t)s[9];
      st.num_lloss = (uint32_t)s[8];
      st.num_good = ng;
      redo = s[11] != 0.0;
      if (redo) {
        st.st[PHI_AVG_GOOD] = ng > 0 ? (double)((float)s[10] / (float)ng) + b.phi_ref : -99999;
      } else {
        sc_moments_finish(b, s, sc, t, freq, frac, h);
        st.sc_redo = 0u;
      }
    }
    __syncthreads();
    if (redo) {
      // the loss test changed the good set: the moments again about the new
      // <phi>_good (Op32ScStats), swept by this last block alone -- a rare
      // path, kept out of a launch of its own; thread order, then a fixed
      // shuffle tree and the warps in order
      const float pag = (float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref);
      float a[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = 0.0f;
      for (uint32_t i = tid; i < b.n; i += nth) {
        const float pr = rel_phase_f(b.fphi[i] - pag);
        b.fphi_r[i] = pr;
        float a12[12];
#pragma unroll
        for (int k = 0; k < 8; ++k) a12[k] = a[k];
        sc_moments_add(a12, pr, b.loss[i], b.lloss[i], b.fx[i], b.fy[i], b.fw[i]);
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = a12[k];
      }
      const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        float v = a[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp][k] = v;
      }
      __syncthreads();
      if (tid < 8) {
        double v = 0.0;
        for (int w = 0; w < nth / 32; ++w) v += (double)red[w][tid];
        mom[tid] = v;
      }
      __syncthreads();
      if (tid == 0) {
        sc_moments_finish(b, mom, sc, t, freq, frac, h);
        b.st->sc_redo = 0u;
      }
      __syncthreads();
    }
    zero_mesh_tables(sc, t, tid, nth);
  }
};

struct Op32AdjMesh {
  static constexpr int K = 2;
  static constexpr bool kFast = true;
  using Comb = MaxComb;
  struct Ctx { float xa, ya, pa, pag; };
  DevBeam b;
  ScState *sc;
  Sc32Consts *c32;
  Sc32Host h;
  __device__ bool enabled() const { return sc->remesh && sc->adj != 0u; }
  __device__ Ctx setup() const {
    return {(float)b.st->st[X_AVG], (float)b.st->st[Y_AVG], (float)b.st->st[PHI_AVG_R], c32->pag};
  }
  struct P { uint32_t lo; float x, y, ph; };
  __device__ P load(uint32_t i) const { return {b.loss[i], b.fx[i], b.fy[i], b.fphi[i]}; }
  __device__ void use(uint32_t, const P &p, float (&a)[K], const Ctx &c) const {
    if (p.lo != 0u) return;
    float tx = p.x - c.xa, ty = p.y - c.ya;
    a[0] = fmaxf(a[0], tx * tx + ty * ty);
    a[1] = fmaxf(a[1], fabsf(rel_phase_f(p.ph - c.pag) - c.pa));
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    const float rmax = sqrtf((float)t[0]);
    BeamStats st = *b.st;
    st.st[R_MAX] = rmax;
    st.st[ABS_PHI_MAX] = t[1];
    *b.st = st;
    ScState s = *sc;
    Sc32Consts c;
    mesh_size32(&s, (float)s.beta, h.wave_len, rmax, 0.0f, 1.0f);
    sc32_consts(st, b, &s, &c, h);
    *sc = s;
    *c32 = c;
  }
};

__global__ void k32_decide_only(DevBeam b, ScState *sc, ScTables t, double freq, double frac, Sc32Host h) {
  if (threadIdx.x == 0) sc32_decide_consts(*b.st, b, sc, t.c32, h, freq, frac);
  __syncthreads();
  zero_mesh_tables(sc, t, threadIdx.x, blockDim.x);
}

// ---- Green's table ---------------------------------------------------------
// green_term (green32.cuh): UpdateFldTbl1Kernel's entry in FP32.
// blocks [bid0, bid0 + nblk) of the launch evaluate the table
__device__ void green_blocks(const ScState *sc, const ScTables &t, uint32_t bid, uint32_t nblk) {
  const uint32_t nr = sc->nx, nz = sc->nz;
  const uint32_t by = (512 / nz < nr) ? 512 / nz : nr;
  const uint32_t nrs = by ? (nr / by) * by : 0;
  const uint32_t total = (nr + 1) * nrs * nz;
  const Sc32Consts &k = *t.c32;
  const float dr = k.dr0, dzg = k.dzg0, pl = k.pl, c1 = k.green_c1;
  const uint32_t adj = sc->adj;
  float2 *out = (float2 *)t.ffld1;
  // a tensor-core mesh also gets the folded split-BF16 MMA tiles (rp < nr)
  const bool tc = t.tcg != nullptr && nr == t.tc_nr && nz == t.tc_nz;
  for (uint32_t e = bid * blockDim.x + threadIdx.x; e < total; e += nblk * blockDim.x) {
    uint32_t tz = e % nz;
    uint32_t kk = (e / nz) % nrs;
    uint32_t rpi = e / (nz * nrs);
    float rs = sqrtf(0.5f * (float)(kk * kk + (kk + 1) * (kk + 1))) * dr;
    float rp = (float)rpi * dr;
    float d = ((float)tz + 0.5f) * dzg;  // zp - zs with zs = dzg / 2, zp = (tz + 1) dzg
    GreenTerm g = green_term(rs, rp, d);
    for (uint32_t i = 1; i <= adj; ++i) {
      GreenTerm g1 = green_term(rs, rp, d - (float)i * pl), g2 = green_term(rs, rp, d + (float)i * pl);
      g.er += g1.er + g2.er;
      g.ez += g1.ez + g2.ez;
    }
    // stored [rp][dz][rs] (rs fastest) for the contraction's lanes
    const float2 v = make_float2(c1 * g.er, c1 * g.ez);
    out[((size_t)rpi * nz + tz) * nr + kk] = v;
    if (tc) tc_put_green(t, nr, nz, rpi, kk, tz, v.x, v.y);
  }
}

__global__ void k32_green(const ScState *sc, ScTables t) {
  if (!sc->remesh || sc->sur_accepted) return;
  green_blocks(sc, t, blockIdx.x, gridDim.x);
}

// lockstep form: grid y over the beams
template <int B>
__global__ void k32_green_seg(const __grid_constant__ SegArgs<MeshSeg, B> a) {
  const MeshSeg &p = a.p[blockIdx.y];
  if (!p.sc->remesh || p.sc->sur_accepted) return;
  green_blocks(p.sc, p.t, blockIdx.x, gridDim.x);
}

// ---- deposit -----------------------------------------------------------------
struct DepQ {
  float scale;   // 2^s: fixed-point scale of the per-block histogram
  int shift;     // 36 - s: to the global table's 2^36 scale
  int smem;      // per-block histogram in shared memory (else global atomics)
  int agg;       // warp-aggregated shared-memory adds (a launch-shape choice)
};

// Add w to bin k of the block's histogram.  Aggregated: the warp's lanes
// with the same bin (__match_any_sync) sum their weights (__reduce_add_sync,
// exact integer sums) and the lowest of them adds the total, one shared-
// memory atomic per distinct bin per warp instead of one per particle --
// the beam core's few bins take most particles.  Every lane of the warp
// calls it (invalid lanes with k = -1 and w = 0).
__device__ __forceinline__ void hist_add(int *hist32, int k, int w, bool agg) {
  if (!agg) {
    if (w) atomicAdd(hist32 + k, w);
    return;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, k);
  const int tot = (int)__reduce_add_sync(peers, (unsigned)w);
  if (k >= 0 && tot && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) atomicAdd(hist32 + k, tot);
}

// Deposit blocks run in clusters of kDepCluster CTAs: each CTA fills its own
// shared-memory histogram, then CTA r of the cluster sums slice r of the
// cluster's histograms through distributed shared memory and adds it to the
// global table, so a bin takes one global atomic per cluster, not per block.
constexpr int kDepCluster = 8;
// deposit threads per block: 256, 512 or 1024 (a launch-shape choice; the
// kernels take up to 1024, at most 64 registers a thread)
constexpr int kDepBlockMax = 1024;
// particles a thread loads before it deposits them.  Measured on the whole
// step: 2 (51 registers) ties 4 on 1M-particle beams but is 3.5% slower on a
// 16M-particle beam (fewer loads in flight); 8 is 3% slower on 1M particles
constexpr int kDepBatch = 4;

struct DepIn {
  uint32_t lo, ll;
  float x, y, ph;
};

// DistributeParticleKernel (space_charge_kernel.cu:123-224) in FP32, on
// blocks [0, nblk) of the launch (nblk a multiple of kDepCluster)
__device__ void deposit_blocks(const DevBeam &bm, ScState *sc, const ScTables &t, const DepQ &q, uint32_t bid,
                               uint32_t nblk) {
  extern __shared__ int hist32[];
  namespace cg = cooperative_groups;
  const uint32_t nx = sc->nx, nz = sc->nz, nb = nx * nz;
  if (q.smem) {
    if (nb % 4 == 0)
      for (uint32_t k = threadIdx.x; k < nb / 4; k += blockDim.x) ((int4 *)hist32)[k] = make_int4(0, 0, 0, 0);
    else
      for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) hist32[k] = 0;
    __syncthreads();
  }
  const Sc32Consts &kc = *t.c32;
  const float phimc = kc.phimc, xbar = kc.xbar, ybar = kc.ybar, epsq = kc.epsq, inv_epsq = kc.inv_epsq;
  const float dr = kc.dr0, dzg = kc.dzg0, inv_dr = kc.inv_dr0, inv_dzg = kc.inv_dzg0, hl = kc.hl0, c2 = kc.c2;
  const float pag = kc.pag;
  const float drdr = dr * dr, inv_drdr = inv_dr * inv_dr;
  const long long m = 1ll << q.shift;
  const uint32_t stride = nblk * blockDim.x;
  const bool agg = q.smem && q.agg;
  uint32_t cnt = 0;
  // particle in -> its four bins and fixed-point weights; false when it is
  // not deposited (lost, longitudinally lost, off the mesh)
  auto weigh = [&](const DepIn &in, int (&k)[4], int (&w)[4]) -> bool {
    if (in.lo != 0u || in.ll != 0u) return false;
    const float pz = rel_phase_f(in.ph - pag);
    const float dx = in.x - xbar, dy = in.y - ybar;
    const float rsq_sh = dx * dx * inv_epsq + dy * dy * epsq;
    const int i = (int)(sqrt_fast(rsq_sh) * inv_dr + 1.0f);
    const float z = -c2 * wrap_turns(pz - phimc);
    if (!(i >= 1 && (uint32_t)i <= nx)) return false;
    if (!(fabsf(z) < hl)) return false;
    const float zz = z + hl;
    const int jm1 = (int)(zz * inv_dzg + 1.0f);
    if (jm1 < 1 || jm1 > (int)nz) return false;
    int i1 = i + 1;
    if (rsq_sh < 0.5f * drdr * (float)(i * i + (i - 1) * (i - 1))) i1 = i - 1;
    i1 = min(max(i1, 1), (int)nx);
    int j1 = jm1 + 1;
    if (zz < ((float)jm1 - 0.5f) * dzg) j1 = jm1 - 1;
    j1 = min(max(j1, 1), (int)nz);
    // area weights in units of dr^2 (rmax^2 - rmin^2 = sqrtmp dr^2), and the
    // z weight with (jm1 - j1) dz = +-dz
    float a = 1.0f;
    if (i1 != i) {
      const float sqrtmp = sqrt_fast(4.0f * rsq_sh * inv_drdr - 1.0f);
      const float rmin_n = 0.25f * (sqrtmp - 1.0f) * (sqrtmp - 1.0f);
      const float rmax_n = rmin_n + sqrtmp;
      if (i1 < i) a = __fdividef(rmax_n - (float)((i - 1) * (i - 1)), sqrtmp);
      else a = __fdividef((float)((i1 - 1) * (i1 - 1)) - rmin_n, sqrtmp);
    }
    float cc = 1.0f;
    if (j1 != jm1) cc = (zz - ((float)j1 - 0.5f) * dzg) * (j1 < jm1 ? inv_dzg : -inv_dzg);
    const float bb = 1.0f - a, d = 1.0f - cc;
    k[0] = (jm1 - 1) * (int)nx + i - 1;
    k[1] = k[0] + (i1 - i);
    k[2] = (j1 - 1) * (int)nx + i - 1;
    k[3] = k[2] + (i1 - i);
    w[0] = __float2int_rn(a * cc * q.scale);
    w[1] = __float2int_rn(bb * cc * q.scale);
    w[2] = __float2int_rn(a * d * q.scale);
    w[3] = __float2int_rn(bb * d * q.scale);
    return true;
  };
  if (agg) {
    // warp-uniform iterations (a lane past the end carries no particle), so
    // that every lane takes part in the aggregated adds
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t wbase = bid * blockDim.x + (threadIdx.x & ~31u); wbase < bm.n; wbase += kDepBatch * stride) {
      DepIn in[kDepBatch];
#pragma unroll
      for (int u = 0; u < kDepBatch; ++u) {
        const uint32_t np = wbase + lane + u * stride;
        if (np < bm.n) in[u] = {bm.loss[np], bm.lloss[np], bm.fx[np], bm.fy[np], bm.fphi[np]};
        else in[u].lo = 1u;
      }
#pragma unroll
      for (int u = 0; u < kDepBatch; ++u) {
        int k[4] = {-1, -1, -1, -1}, w[4] = {0, 0, 0, 0};
        if (weigh(in[u], k, w)) ++cnt;
        else k[0] = k[1] = k[2] = k[3] = -1, w[0] = w[1] = w[2] = w[3] = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) hist_add(hist32, k[e], w[e], true);
      }
    }
  } else {
    for (uint32_t base = bid * blockDim.x + threadIdx.x; base < bm.n; base += kDepBatch * stride) {
      DepIn in[kDepBatch];
#pragma unroll
      for (int u = 0; u < kDepBatch; ++u) {
        const uint32_t np = base + u * stride;
        if (np < bm.n) in[u] = {bm.loss[np], bm.lloss[np], bm.fx[np], bm.fy[np], bm.fphi[np]};
        else in[u].lo = 1u;
      }
#pragma unroll
      for (int u = 0; u < kDepBatch; ++u) {
        int k[4], w[4];
        if (!weigh(in[u], k, w)) continue;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (!w[e]) continue;
          if (q.smem) atomicAdd(hist32 + k[e], w[e]);
          else atomicAdd(t.bin_fx + k[e], (unsigned long long)((long long)w[e] * m));
        }
        ++cnt;
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&sc->num_on_mesh, cnt);
  if (!q.smem) return;  // uniform over the launch
  cg::cluster_group cl = cg::this_cluster();
  cl.sync();  // every histogram of the cluster is complete
  const uint32_t nc = cl.num_blocks(), r = cl.block_rank();
  if (nc == (uint32_t)kDepCluster && nb % (4 * kDepCluster) == 0) {
    // slice r of the cluster's histograms, four bins per 16-byte load from
    // every CTA of the cluster at once (all loads in flight together), the
    // CTAs summed in rank order
    const uint32_t per = nb / kDepCluster, k0 = r * per;
    const int4 *src[kDepCluster];
#pragma unroll
    for (int c = 0; c < kDepCluster; ++c) src[c] = (const int4 *)cl.map_shared_rank(hist32 + k0, c);
    for (uint32_t k4 = threadIdx.x; k4 < per / 4; k4 += blockDim.x) {
      int4 v[kDepCluster];
#pragma unroll
      for (int c = 0; c < kDepCluster; ++c) v[c] = src[c][k4];
      long long s0 = 0, s1 = 0, s2 = 0, s3 = 0;  // up to 8 block sums of < 2^30 each
#pragma unroll
      for (int c = 0; c < kDepCluster; ++c) {
        s0 += v[c].x; s1 += v[c].y; s2 += v[c].z; s3 += v[c].w;
      }
      unsigned long long *dst = t.bin_fx + k0 + 4 * k4;
      if (s0) atomicAdd(dst, (unsigned long long)(s0 * m));
      if (s1) atomicAdd(dst + 1, (unsigned long long)(s1 * m));
      if (s2) atomicAdd(dst + 2, (unsigned long long)(s2 * m));
      if (s3) atomicAdd(dst + 3, (unsigned long long)(s3 * m));
    }
  } else {
    const uint32_t per = (nb + nc - 1) / nc, k0 = r * per, k1 = min(nb, k0 + per);
    for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      long long v = 0;  // up to nc block sums of < 2^30 each
      for (uint32_t c = 0; c < nc; ++c) v += *cl.map_shared_rank(hist32 + k, c);
      if (v) atomicAdd(t.bin_fx + k, (unsigned long long)(v * m));
    }
  }
  cl.sync();  // no CTA leaves while the others read its histogram
}

// The deposit and the Green's table are independent: one launch, blocks
// [0, ndep) deposit, blocks [ndep, ndep + ngreen) evaluate the table (both
// multiples of the cluster size, so no cluster mixes the two).
__global__ void __cluster_dims__(kDepCluster, 1, 1) __launch_bounds__(kDepBlockMax)
    k32_green_deposit(DevBeam bm, ScState *sc, ScTables t, DepQ q, uint32_t ndep, uint32_t ngreen) {
  if (!sc->remesh) return;
  if (blockIdx.x < ndep) deposit_blocks(bm, sc, t, q, blockIdx.x, ndep);
  else green_blocks(sc, t, blockIdx.x - ndep, ngreen);
}

// lockstep form of the deposit: every beam's blocks (whole clusters, so a
// cluster never spans two beams) in one flat launch
struct DepSeg {
  DevBeam bm;
  ScState *sc;
  ScTables t;
  DepQ q;
  size_t hb;  // shared-memory histogram bytes (the same for every beam of a batch)
  uint32_t threads;  // block size (the same for every beam of a merged launch)
};
template <int B>
__global__ void __cluster_dims__(kDepCluster, 1, 1) __launch_bounds__(kDepBlockMax)
    k32_deposit_seg(const __grid_constant__ SegArgs<DepSeg, B> a) {
  uint32_t bid, nblk;
  const DepSeg &p = a.p[seg_find(a, blockIdx.x, bid, nblk)];
  if (!p.sc->remesh) return;
  deposit_blocks(p.bm, p.sc, p.t, p.q, bid, nblk);
}

// the side-stream branch: fork, the Green's tables of every beam, join
void green_merge(const std::vector<const Rec *> &recs, SegFork &a, cudaStream_t st, cudaStream_t side) {
  uint32_t blocks = 0;  // the table entries are independent of the block count
  for (const Rec *r : recs) blocks = std::max(blocks, r->blocks);
  cudaEventRecord(a.ev_fork, st);
  cudaStreamWaitEvent(side, a.ev_fork, 0);
  seg_chunks<MeshSeg>(recs, [&](const auto &g, uint32_t) {
    k32_green_seg<std::decay_t<decltype(g)>::kB><<<dim3(blocks, g.nb), kBlock, 0, side>>>(g);
  });
  cudaEventRecord(a.ev_join, side);
}
// the deposit on the main stream, then the join of the Green's branch
void deposit_merge(const std::vector<const Rec *> &recs, SegFork &a, cudaStream_t st, cudaStream_t) {
  size_t hb = 0;  // the largest histogram of the beams that deposit through shared memory
  for (const Rec *r : recs) {
    DepSeg d;
    std::memcpy(&d, r->p.data(), sizeof(DepSeg));
    if (d.q.smem) hb = std::max(hb, d.hb);
  }
  seg_chunks<DepSeg>(recs, [&](const auto &g, uint32_t blocks) {
    launch_k(k32_deposit_seg<std::decay_t<decltype(g)>::kB>, dim3(blocks), dim3(g.p[0].threads), hb, st, g);
  });
  cudaStreamWaitEvent(st, a.ev_join, 0);
}

// ---- kick ----------------------------------------------------------------------
// ApplySpchKickKernel (space_charge_kernel.cu:573-706) in FP32.  The skipped
// set (i % skip_stride == 0) is tested as i & skip_mask == 0: the reference's
// launch geometry (NextPow2 grid and block) makes the stride a power of two.
__global__ void __launch_bounds__(kBlock) k32_kick(DevBeam bm, const ScState *sc, ScTables t, RefK r,
                                                  uint64_t skip_mask) {
  const KickEnv e = kick_env(sc, t, r);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < bm.n; i += gridDim.x * blockDim.x) {
    Part p = load_part(bm, i);
    const uint32_t ll = bm.lloss[i];
    if (((uint64_t)i & skip_mask) == 0 || p.lo != 0u || ll != 0u) continue;
    store_part(bm, i, p, kick_particle(p, rel_phase_f(p.ph - e.pag), e));
  }
}

DepQ dep_quant(uint32_t n, int grid, uint32_t threads, size_t hist_bytes) {
  DepQ q{};
  uint32_t per = (uint32_t)grid * threads;
  uint32_t iters = (n + per - 1) / per;
  uint64_t p = (uint64_t)iters * threads;  // particles one block can deposit
  int bits = 0;
  while ((1ull << bits) <= p) ++bits;
  int s = 30 - bits;
  if (s > 30) s = 30;
  q.smem = hist_bytes > 0;
  if (!q.smem || s < 8) { s = 28; q.smem = 0; }  // global 64-bit atomics: no per-block limit
  q.scale = (float)(1u << s);
  q.shift = 36 - s;
  return q;
}

constexpr size_t kMaxHistSmem = 96 * 1024;

}  // namespace

void beam32_update_stat_for_sc(const DevBeam &b, PassScratch s, cudaStream_t st) {
  if (b.n <= 2) return;
  launch_pass_f(Op32GoodPhi{b}, b.n, s, st);
  launch_pass_f(Op32LlossGoodPhi{b}, b.n, s, st);
  launch_pass_f(Op32ScStats{b, nullptr, ScTables{}, 0.0, 0.0, Sc32Host{}, 0}, b.n, s, st);
  note_launch(3);
}

static ScTables tables32(const ScTables &t) {
  ScTables u = t;
  u.fld2 = nullptr;  // FP32 beams use ffld1 / ffld2
  return u;
}

Sc32Host sc32_host(const DevBeam &b, const ScKickArgs &a) {
  Sc32Host h;
  h.inv_mass = (float)(1.0 / b.mass);
  h.wave_len = (float)(CLIGHT / a.freq);
  h.c1 = (float)(5721.67 * a.current * a.frac / (a.freq * 1e6 * (double)b.n * b.mass));
  h.length = (float)a.length;
  return h;
}

void sc32_stats(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
                cudaStream_t st) {
  ScTables u = tables32(t);
  const Sc32Host h = sc32_host(b, a);
  if (a.stats_ok) {
    launch_pass_f(Op32GoodPhi{b}, b.n, s, st);
    launch_pass_f(Op32LlossGoodPhi{b}, b.n, s, st);
    launch_pass_f(Op32ScStats{b, sc, u, a.freq, a.frac, h, 0}, b.n, s, st);
    note_launch(3);
  } else {
    launch_k(k32_decide_only, dim3(1), dim3(kBlock), 0, st, b, sc, u, a.freq, a.frac, h);
    note_launch();
  }
}

// one launch of one block per SM: it returns at once when the element map
// before the kick certified its statistics (every kick of the bench
// workloads), so its cost there is the launch alone
void sc32_stats_after_push(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a,
                           PassScratch s, cudaStream_t st) {
  ScTables u = tables32(t);
  const Sc32Host h = sc32_host(b, a);
  launch_pass_f_grid(Op32LlossScStats{b, sc, u, a.freq, a.frac, h}, b.n, s, st, (uint32_t)pass_blocks_f(b.n, 1),
                     "stats_fallback");
  if (!recorder()) note_launch();
}

void sc32_mesh(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
               cudaStream_t st, const SurNet *sur, const Fork *fork) {
  ScTables u = tables32(t);
  if (a.adj_possible) {  // the mesh is sized from r_max only with adjacent bunches
    launch_pass_f(Op32AdjMesh{b, sc, u.c32, sc32_host(b, a)}, b.n, s, st);
    note_launch();
  }
  uint32_t ndep = 0;
  size_t hb = 0;
  DepQ q{};
  const uint32_t dthreads = a.dep_threads ? a.dep_threads : 256u;  // deposit block size
  if (a.deposit_ok) {
    // dep_per_sm blocks per SM at most (three unless tuned), in whole clusters
    ndep = std::min<uint32_t>((b.n + dthreads - 1) / dthreads, (a.dep_per_sm ? a.dep_per_sm : 3u) * 152u);
    ndep = (ndep + kDepCluster - 1) / kDepCluster * kDepCluster;
    hb = (size_t)a.nx_max * a.nz_max * sizeof(int);
    if (hb > kMaxHistSmem) hb = 0;
    q = dep_quant(b.n, (int)ndep, dthreads, hb);
    q.agg = a.dep_agg ? 1 : 0;
  }
  // Green's table entries of the largest mesh, a few per thread on one block
  // per SM, so that the whole launch is resident at once
  uint32_t ngreen = std::min<uint32_t>(
      (uint32_t)(((size_t)(a.nx_max + 1) * a.nx_max * a.nz_max + kBlock - 1) / kBlock), 152u);
  ngreen = (ngreen + kDepCluster - 1) / kDepCluster * kDepCluster;
  if (recorder()) {  // a lockstep range: the forked Green's tables and the deposit
    if (sur || a.adj_possible || !fork || !ndep) {
      recorder()->unsupported = "space-charge mesh with a surrogate, adjacent bunches or no deposit";
      return;
    }
    record("green", &green_merge, 4u * ngreen, MeshSeg{sc, u});
    record("deposit", &deposit_merge, ndep, DepSeg{b, sc, u, q, hb, dthreads}, dthreads);
    contract32(sc, u, a.nx_max, a.nz_max, a.mesh_fixed, st);
    return;
  }
  if (sur) {
    // field surrogate: the deposit alone, the network and its check, then
    // the Green's table and the contraction, which return at once when the
    // network's field was accepted
    if (ndep) {
      launch_k(k32_green_deposit, dim3(ndep), dim3(dthreads), q.smem ? hb : 0, st, b, sc, u, q, ndep, 0u);
      note_launch();
    }
    sur_solve(b, sc, u, a, *sur, st, 1);
    k32_green<<<ngreen, kBlock, 0, st>>>(sc, u);
    note_launch();
  } else if (fork && ndep) {
    // the Green's table on the side stream, beside the deposit: it needs no
    // shared memory, so its blocks take the warp slots the deposit's
    // shared-memory histograms leave free (in one launch they would queue
    // behind the deposit blocks, which size every block's shared memory)
    const uint32_t ng = 4u * ngreen;
    cudaEventRecord(fork->ev_fork, st);
    cudaStreamWaitEvent(fork->side, fork->ev_fork, 0);
    k32_green<<<ng, kBlock, 0, fork->side>>>(sc, u);
    cudaEventRecord(fork->ev_join, fork->side);
    launch_k(k32_green_deposit, dim3(ndep), dim3(dthreads), q.smem ? hb : 0, st, b, sc, u, q, ndep, 0u);
    cudaStreamWaitEvent(st, fork->ev_join, 0);
    note_launch(2);
  } else {
    launch_k(k32_green_deposit, dim3(ndep + ngreen), dim3(dthreads), q.smem ? hb : 0, st, b, sc, u, q, ndep, ngreen);
    note_launch();
  }
  contract32(sc, u, a.nx_max, a.nz_max, a.mesh_fixed, st);
}

void sc32_kick(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, cudaStream_t st) {
  if (!a.skip_stride) return;
  if (a.skip_stride & (a.skip_stride - 1)) {
    set_error(HPS_ERR_STATE, "SCHEFF kick: launch stride is not a power of two");
    return;
  }
  launch_k(k32_kick, dim3(grid_for(b.n)), dim3(kBlock), 0, st, b, (const ScState *)sc, tables32(t),
             make_refk(b.w_ref, b.mass), (uint64_t)(a.skip_stride - 1));
  note_launch();
}

void sc32_configure() {
  static PerDevice configured;
  configured.once([] {
    cudaFuncSetAttribute(k32_green_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxHistSmem);
    cudaFuncSetAttribute(k32_deposit_seg<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxHistSmem);
    cudaFuncSetAttribute(k32_deposit_seg<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxHistSmem);
    cudaFuncSetAttribute(k32_deposit_seg<SegCap<DepSeg>::value>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kMaxHistSmem);
    contract_configure<float>();
    const cudaError_t e = contract_tc_configure();
    if (e != cudaSuccess) set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
  });
}

bool sc32_tc_mesh(uint32_t nr, uint32_t nz) { return tc_mesh_ok(nr, nz); }
size_t sc32_tc_bytes(uint32_t nr, uint32_t nz, size_t *partial_bytes) {
  *partial_bytes = tc_partial_bytes(nr, nz);
  return tc_table_bytes(nr, nz);
}

// UpdateFldTbl2KernelDouble for FP32 tables: the tensor-core kernels when
// the solver holds their buffers for the largest mesh it takes, the FP32
// ring convolution otherwise.  Each returns at once when the other one is
// the one for the kick's mesh; mesh_fixed (the kick's mesh is the largest
// one, decided on the host) leaves out the one that cannot run.
void contract32(const ScState *sc, const ScTables &t, uint32_t nx_max, uint32_t nz_max, bool mesh_fixed,
                cudaStream_t st) {
  const bool tc = t.tcg != nullptr && t.tc_nr == nx_max && t.tc_nz == nz_max;
  const bool rec = recorder() != nullptr;
  if (tc) {
    contract_tc_launch(sc, t, nx_max, nz_max, st);
    if (!rec) note_launch(2);
  }
  if (!tc || !mesh_fixed) {
    contract_launch<float>(sc, t, nx_max, nz_max, st);
    if (!rec) note_launch();
  }
}

namespace {

// mesh of a standalone FP32 solve: mesh = {dr, dz, beta, freq, num_particle,
// current*fraction/mass, adj_bunch}
__global__ void k32_field_setup(ScState *sc, Sc32Consts *c, uint32_t nr, uint32_t nz, double dr, double dz,
                                double beta, double freq, double num_part, double cur_ov_mc2, uint32_t adj) {
  sc->nx = nr; sc->nz = nz; sc->nx_init = nr; sc->nz_init = nz; sc->nx_max = nr; sc->nz_max = nz;
  sc->dr = dr; sc->dz = dz; sc->beta = beta; sc->freq = freq; sc->adj = adj;
  sc->remesh = 1;
  const double gm = rsqrt(1.0 - beta * beta);
  c->dr0 = (float)dr;
  c->dzg0 = (float)(dz * gm);
  c->pl = (float)(beta * gm * CLIGHT / freq);
  c->green_c1 = (float)(5721.67 * cur_ov_mc2 / (freq * 1e6 * num_part));
}

__global__ void k32_bins_to_fixed(const double *bins, unsigned long long *fx, uint32_t nb) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x)
    fx[k] = (unsigned long long)__double2ll_rn(bins[k] * kBinScale);
}

}  // namespace
}  // namespace hps

extern "C" {

// UpdateTblsKernelCall (Green's table) + UpdateFinalFldTblKernelCall with the
// FP32 kernels, on a caller-given charge table; kernel: 0 the one FP32 beams
// use for the mesh, 1 the FP32 ring convolution, 2 the tensor cores
hps_status hps_scheff_field_f32_kernel(uint32_t nr, uint32_t nz, const double *bins, const double *mesh,
                                       double *field, int kernel) {
  using namespace hps;
  if (!bins || !mesh || !field) return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field_f32: null pointer");
  if (!nr || !nz || (nr & (nr - 1)) || (nz & (nz - 1)) || nz > 512 || nr > 256)
    return (hps_status)set_error(HPS_ERR_INVALID,
                                 "scheff_field_f32: nr and nz must be powers of two, nz <= 512, nr <= 256");
  if (kernel < 0 || kernel > 2) return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field_f32: unknown kernel");
  if (kernel == 2 && !tc_mesh_ok(nr, nz))
    return (hps_status)set_error(HPS_ERR_UNSUPPORTED,
                                 "scheff_field_f32: the tensor-core contraction takes nz in 128..512 and nr in "
                                 "16..64 (powers of two)");
  const bool tc = kernel == 2 || (kernel == 0 && tc_mesh_ok(nr, nz));
  sc32_configure();
  size_t nb = (size_t)nr * nz, n1 = (size_t)(nr + 1) * nr * nz * 2, n2 = (size_t)(nz + 1) * (nr + 1) * 2;
  ScState *sc = nullptr;
  Sc32Consts *c32 = nullptr;
  unsigned long long *fx = nullptr;
  double *b = nullptr;
  float *f1 = nullptr, *f2 = nullptr, *tcp = nullptr;
  void *tcg = nullptr;
  std::vector<float> host(n2);
  cudaError_t e = cudaMalloc((void **)&sc, sizeof(ScState));
  if (e == cudaSuccess) e = cudaMalloc((void **)&c32, sizeof(Sc32Consts));
  if (e == cudaSuccess) e = cudaMalloc((void **)&fx, nb * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b, nb * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void **)&f1, n1 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void **)&f2, n2 * sizeof(float));
  if (e == cudaSuccess && tc) e = cudaMalloc(&tcg, tc_table_bytes(nr, nz));
  // the padding rows of the MMA tiles (beyond the field's 2 (nr + 1) values) stay zero
  if (e == cudaSuccess && tc) e = cudaMemset(tcg, 0, tc_table_bytes(nr, nz));
  if (e == cudaSuccess && tc) e = cudaMalloc((void **)&tcp, tc_partial_bytes(nr, nz));
  if (e == cudaSuccess) e = cudaMemset(sc, 0, sizeof(ScState));
  if (e == cudaSuccess) e = cudaMemset(c32, 0, sizeof(Sc32Consts));
  if (e == cudaSuccess) e = cudaMemset(f2, 0, n2 * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(b, bins, nb * sizeof(double), cudaMemcpyHostToDevice);
  uint32_t tc_error = 0;
  if (e == cudaSuccess) {
    k32_field_setup<<<1, 1>>>(sc, c32, nr, nz, mesh[0], mesh[1], mesh[2], mesh[3], mesh[4], mesh[5],
                              (uint32_t)mesh[6]);
    k32_bins_to_fixed<<<64, kBlock>>>(b, fx, (uint32_t)nb);
    ScTables t{};
    t.bin_fx = fx;
    t.ffld1 = f1;
    t.ffld2 = f2;
    t.c32 = c32;
    if (tc) {
      t.tcg = tcg;
      t.tcp = tcp;
      t.tc_nr = nr;
      t.tc_nz = nz;
    }
    k32_green<<<4 * 152, kBlock>>>(sc, t);
    note_launch(3);
    contract32(sc, t, nr, nz, true, 0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&tc_error, &sc->tc_error, 4, cudaMemcpyDeviceToHost);
  }
  if (e == cudaSuccess) e = cudaMemcpy(host.data(), f2, n2 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(sc); cudaFree(c32); cudaFree(fx); cudaFree(b); cudaFree(f1); cudaFree(f2);
  if (tcg) cudaFree(tcg);
  if (tcp) cudaFree(tcp);
  if (e != cudaSuccess) return (hps_status)set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
  if (tc_error) return (hps_status)set_error(HPS_ERR_TIMEOUT, "scheff_field_f32: a tensor-core wait gave up");
  for (size_t k = 0; k < n2; ++k) field[k] = host[k];
  return HPS_OK;
}

hps_status hps_scheff_field_f32(uint32_t nr, uint32_t nz, const double *bins, const double *mesh, double *field) {
  return hps_scheff_field_f32_kernel(nr, nz, bins, mesh, field, 0);
}

}  // extern "C"
