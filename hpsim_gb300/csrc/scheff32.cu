// scheff32.cu -- the SCHEFF 2D r-z space-charge kick on FP32 particle state.
//
// Same launch sequence and device-side decision as scheff.cu (Scheff::Start,
// src/simulation/src/space_charge.cpp:82-139; kernels of
// src/simulation/inc/space_charge_kernel.cu).  Differences:
//  * statistics sweeps accumulate offsets in FP32 per thread and warp, FP64
//    across warps and blocks (reduce.cuh: pass_kernel_f);
//  * the thread that takes the space-charge decision also forms, in FP64,
//    every constant the FP32 kernels of the kick need (Sc32Consts), so no
//    particle kernel does FP64 arithmetic (GB300 runs FP64 at 1/64 rate);
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
#include <algorithm>
#include <vector>

#include "../../include/hpsim_gb300.h"
#include "internal.h"
#include "reduce.cuh"
#include "scheff_common.cuh"

namespace hps {

namespace {

struct NoCtx {};

__device__ inline double surv(const DevBeam &b) { return (double)(uint32_t)(b.n - b.st->num_loss); }

// Constants of the kick about to run, from the statistics and the decision
// (ApplySpchKickKernel, space_charge_kernel.cu:573-620; UpdateFldTbl1Kernel,
// :39-60; DistributeParticleKernel, :123-150), in FP64, once.
__device__ void sc32_consts(const DevBeam &b, const ScState *s, Sc32Consts *c, double length, double current) {
  const BeamStats &st = *b.st;
  const double r_beta = s->beta, r_freq = s->freq, mass = b.mass;
  const double epsq = st.st[X_SIG_GOOD] / st.st[Y_SIG_GOOD];
  const double gmg = rsqrt(1.0 - r_beta * r_beta);
  const double wave_len = CLIGHT / r_freq;
  const double dr = s->dr * s->ratio_r, dzg = s->dz * gmg * s->ratio_z;
  const double dr0 = s->dr, dzg0 = s->dz * gmg;
  const double r_current = current * s->frac;
  const double c1 = 5721.67 * r_current / (r_freq * 1e6 * (double)b.n * mass);
  const double c3 = length / (r_beta * gmg);
  c->phimc = (float)st.st[PHI_AVG_R];
  c->xbar = (float)st.st[X_AVG_GOOD];
  c->ybar = (float)st.st[Y_AVG_GOOD];
  c->epsq = (float)epsq;
  c->inv_epsq = (float)(1.0 / epsq);
  c->xfac = (float)(2.0 / (epsq + 1.0));
  c->yfac = (float)(epsq * 2.0 / (epsq + 1.0));
  c->beta = (float)r_beta;
  c->gmg = (float)gmg;
  c->c2 = (float)(r_beta * gmg * wave_len / TWOPI);
  c->pl = (float)(r_beta * gmg * wave_len);
  c->dr = (float)dr;
  c->dzg = (float)dzg;
  c->inv_dr = (float)(1.0 / dr);
  c->inv_dzg = (float)(1.0 / dzg);
  c->hl = (float)(s->nz * 0.5 * dzg);
  c->rmesh = (float)(s->nx * dr);
  c->dr0 = (float)dr0;
  c->dzg0 = (float)dzg0;
  c->inv_dr0 = (float)(1.0 / dr0);
  c->inv_dzg0 = (float)(1.0 / dzg0);
  c->hl0 = (float)(s->nz * 0.5 * dzg0);
  c->cbg_per_onm = (float)(c1 * c3 * PI * 0.5);
  c->er_c3 = (float)(s->ratio_q / (s->ratio_r * s->ratio_z * s->ratio_g * s->ratio_g) * c3);
  c->ez_c3 = (float)(s->ratio_q / (s->ratio_z * s->ratio_z) * c3);
  c->dwc = (float)(b.w_ref - (gmg - 1.0) * mass);
  c->green_c1 = (float)(5721.67 * (r_current / mass) / (r_freq * 1e6 * (double)b.n));
}

// UpdateGoodParticleCount + UpdateAvgPhi(true)
struct Op32GoodPhi {
  static constexpr int K = 2;
  using Comb = SumComb;
  using Ctx = NoCtx;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {}; }
  __device__ void particle(uint32_t i, float (&a)[K], const Ctx &) const {
    uint32_t lo = b.loss[i], ll = b.lloss[i];
    float ph = b.fphi[i];
    bool g = (uint32_t)(lo + ll) == 0u;
    a[0] += g ? 1.0f : 0.0f;
    a[1] += g ? ph : 0.0f;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t ng = (uint32_t)t[0];
    b.st->num_good = ng;
    b.st->st[PHI_AVG_GOOD] = ng > 0 ? t[1] / ng + b.phi_ref : -99999;
  }
};

// longitudinal-loss test + lloss count + good count + <phi>_good
struct Op32LlossGoodPhi {
  static constexpr int K = 3;
  using Comb = SumComb;
  struct Ctx { float lim; };
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {(float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref + TWOPI + PI)}; }
  __device__ void particle(uint32_t i, float (&a)[K], const Ctx &c) const {
    uint32_t lo = b.loss[i], ll = b.lloss[i];
    float ph = b.fphi[i];
    if (ph > c.lim && ll != 1u) {
      ll = 1u;
      b.lloss[i] = 1u;
    }
    bool g = (uint32_t)(lo + ll) == 0u;
    a[0] += ll != 0u ? 1.0f : 0.0f;
    a[1] += g ? 1.0f : 0.0f;
    a[2] += g ? ph : 0.0f;
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t ng = (uint32_t)t[1];
    b.st->num_lloss = (uint32_t)t[0];
    b.st->num_good = ng;
    b.st->st[PHI_AVG_GOOD] = ng > 0 ? t[2] / ng + b.phi_ref : -99999;
  }
};

// relative phase about <phi>_good, the SCHEFF moments, the decision and the
// kick's constants (as OpScStats in scheff.cu)
struct Op32ScStats {
  static constexpr int K = 8;
  using Comb = SumComb;
  struct Ctx { float pag; };
  DevBeam b;
  ScState *sc;
  ScTables t;
  double freq, frac, length, current;
  __device__ bool enabled() const { return true; }
  __device__ Ctx setup() const { return {(float)(b.st->st[PHI_AVG_GOOD] - b.phi_ref)}; }
  __device__ void particle(uint32_t i, float (&a)[K], const Ctx &c) const {
    uint32_t lo = b.loss[i], ll = b.lloss[i];
    float ph = b.fphi[i], x = b.fx[i], y = b.fy[i], w = b.fw[i];
    float pr = rel_phase_f(ph - c.pag);
    b.fphi_r[i] = pr;
    float alive = lo == 0u ? 1.0f : 0.0f;
    float gd = (lo == 0u && ll == 0u) ? 1.0f : 0.0f;
    a[0] += alive * pr;
    a[1] += gd * pr; a[2] += gd * pr * pr;
    a[3] += gd * x; a[4] += gd * x * x; a[5] += gd * y; a[6] += gd * y * y;
    a[7] += gd * w;
  }
  __device__ void finalize(const double *s, int tid, int nth) const {
    if (tid == 0) {
      BeamStats &st = *b.st;
      double sv = surv(b);
      double ng = st.num_good;
      st.st[PHI_AVG_R] = s[0] / sv;
      double pa = s[1] / ng, pa2 = s[2] / ng;
      st.st[PHI_SIG_GOOD] = sqrt(pa2 - pa * pa);
      double xa = s[3] / sv, x2 = s[4] / sv, ya = s[5] / sv, y2 = s[6] / sv;
      st.st[X_AVG_GOOD] = xa;
      st.st[X_SIG_GOOD] = sqrt(x2 - xa * xa);
      st.st[Y_AVG_GOOD] = ya;
      st.st[Y_SIG_GOOD] = sqrt(y2 - ya * ya);
      st.st[W_AVG_GOOD] = st.num_good > 0 ? s[7] / st.num_good + b.w_ref : -99999;
      if (sc) {
        scheff_decide(b, sc, freq, frac);
        sc32_consts(b, sc, t.c32, length, current);
      }
    }
    if (!sc) return;
    __syncthreads();
    zero_mesh_tables(sc, t, tid, nth);
  }
};

struct Op32AdjMesh {
  static constexpr int K = 2;
  using Comb = MaxComb;
  struct Ctx { float xa, ya, pa; };
  DevBeam b;
  ScState *sc;
  Sc32Consts *c32;
  double length, current;
  __device__ bool enabled() const { return sc->remesh && sc->adj != 0u; }
  __device__ Ctx setup() const {
    return {(float)b.st->st[X_AVG], (float)b.st->st[Y_AVG], (float)b.st->st[PHI_AVG_R]};
  }
  __device__ void particle(uint32_t i, float (&a)[K], const Ctx &c) const {
    uint32_t lo = b.loss[i];
    float tx = b.fx[i] - c.xa, ty = b.fy[i] - c.ya, tp = fabsf(b.fphi_r[i] - c.pa);
    if (lo != 0u) return;
    a[0] = fmaxf(a[0], tx * tx + ty * ty);
    a[1] = fmaxf(a[1], tp);
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    b.st->st[R_MAX] = sqrt(t[0]);
    b.st->st[ABS_PHI_MAX] = t[1];
    mesh_size(sc, b.st->st[R_MAX], 0.0, 1.0);
    sc32_consts(b, sc, c32, length, current);
  }
};

__global__ void k32_decide_only(DevBeam b, ScState *sc, ScTables t, double freq, double frac, double length,
                                double current) {
  if (threadIdx.x == 0) {
    scheff_decide(b, sc, freq, frac);
    sc32_consts(b, sc, t.c32, length, current);
  }
  __syncthreads();
  zero_mesh_tables(sc, t, threadIdx.x, blockDim.x);
}

// wrap into [-pi, pi] by whole turns (space_charge_kernel.cu:160-166); the
// relative phases are already wrapped, so one turn at most is removed
__device__ inline float wrap_turns(float d) {
  const float pi = 3.14159265358979323846f, twopi = 6.28318530717958647692f;
  for (int guard = 0; (d > pi || d < -pi) && guard < 64; ++guard) d += d > 0.0f ? -twopi : twopi;
  return d;
}

// ---- Green's table ---------------------------------------------------------
// UpdateFldTbl1Kernel (space_charge_kernel.cu:39-100) in FP32.  With
// b = (rp + rs)^2, c = (rp - rs)^2 and the complementary parameter
// g = 1 - 4 rs rp / (b + d^2) = (c + d^2) / (b + d^2) (no cancellation), the
// reference's radial term  ek - (rs^2 - rp^2 + d^2) ee / (c + d^2)  equals
// (ek - ee) - ee 2 rp (rs - rp) / (c + d^2).  ek - ee is the difference of
// the two fits re-expanded in m = 1 - g = 4 rs rp / (b + d^2) and
// h = log(g) = log1p(-m):
//   ek - ee = C0 + m (Cm + Cmm m) + h (Ch + m (Chm + Chmm m)),
// with the coefficients formed exactly from the fits' (C0 = 6e-8 is the fits'
// own residual at m = 0), so the far field (ek - ee = O(m)) is not a
// difference of two O(1) values.  Rows rs >= (nr/by)*by are not written, as
// in the reference's grid.
struct GreenTerm { float er, ez; };
__device__ inline GreenTerm green_term(float rs, float rp, float d) {
  const float d2 = d * d;
  const float c = (rp - rs) * (rp - rs), b = (rp + rs) * (rp + rs);
  const float inv = 1.0f / (b + d2);
  const float g = (c + d2) * inv, m = 4.0f * rs * rp * inv;
  const float h = m < 0.5f ? log1pf(-m) : logf(g);
  const float ee = 1.0f + g * (0.4630106f - 0.2452740f * h + g * (0.1077857f - 0.04125321f * h));
  // D0..D5 = ek - ee coefficients of 1, h, g, g h, g^2, g^2 h:
  //   0.38629436, -0.5, -0.3510409, 0.1239254, -0.0352534, 0.01237849
  // C0 = D0+D2+D4, Ch = D1+D3+D5, Cm = -D2-2D4, Chm = -D3-2D5, Cmm = D4, Chmm = D5
  const float dke = 6.0e-8f + m * (0.4215477f - 0.0352534f * m) +
                    h * (-0.36369611f + m * (-0.14868238f + 0.01237849f * m));
  const float a = sqrtf(b + d2);
  GreenTerm t;
  t.er = rp != 0.0f ? (dke - ee * 2.0f * rp * (rs - rp) / (c + d2)) / (2.0f * rp * a) : 0.0f;
  t.ez = d * ee / (a * (c + d2));
  return t;
}

__global__ void k32_green(const ScState *sc, ScTables t) {
  if (!sc->remesh) return;
  const uint32_t nr = sc->nx, nz = sc->nz;
  const uint32_t by = (512 / nz < nr) ? 512 / nz : nr;
  const uint32_t nrs = by ? (nr / by) * by : 0;
  const uint32_t total = (nr + 1) * nrs * nz;
  const Sc32Consts &k = *t.c32;
  const float dr = k.dr0, dzg = k.dzg0, pl = k.pl, c1 = k.green_c1;
  const uint32_t adj = sc->adj;
  float2 *out = (float2 *)t.ffld1;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
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
    out[(size_t)rpi * nr * nz + (size_t)kk * nz + tz] = make_float2(c1 * g.er, c1 * g.ez);
  }
}

// ---- deposit -----------------------------------------------------------------
struct DepQ {
  float scale;   // 2^s: fixed-point scale of the per-block histogram
  int shift;     // 36 - s: to the global table's 2^36 scale
  int smem;      // per-block histogram in shared memory (else global atomics)
};

// DistributeParticleKernel (space_charge_kernel.cu:123-224) in FP32
__global__ void __launch_bounds__(kBlock) k32_deposit(DevBeam bm, ScState *sc, ScTables t, DepQ q) {
  if (!sc->remesh) return;
  extern __shared__ int hist32[];
  const uint32_t nx = sc->nx, nz = sc->nz, nb = nx * nz;
  if (q.smem) {
    for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) hist32[k] = 0;
    __syncthreads();
  }
  const Sc32Consts &kc = *t.c32;
  const float phimc = kc.phimc, xbar = kc.xbar, ybar = kc.ybar, epsq = kc.epsq, inv_epsq = kc.inv_epsq;
  const float dr = kc.dr0, dzg = kc.dzg0, inv_dr = kc.inv_dr0, inv_dzg = kc.inv_dzg0, hl = kc.hl0, c2 = kc.c2;
  const float drdr = dr * dr;
  const long long m = 1ll << q.shift;
  uint32_t cnt = 0;
  for (uint32_t np = blockIdx.x * blockDim.x + threadIdx.x; np < bm.n; np += gridDim.x * blockDim.x) {
    const uint32_t lo = bm.loss[np], ll = bm.lloss[np];
    const float px = bm.fx[np], py = bm.fy[np], pz = bm.fphi_r[np];
    float dx = px - xbar, dy = py - ybar;
    float rsq_sh = dx * dx * inv_epsq + dy * dy * epsq;
    int i = (int)(sqrtf(rsq_sh) * inv_dr + 1.0f);
    float z = -c2 * wrap_turns(pz - phimc);
    if (lo != 0u || ll != 0u) continue;
    if (!(i >= 1 && (uint32_t)i <= nx)) continue;
    if (!(fabsf(z) < hl)) continue;
    float zz = z + hl;
    int jm1 = (int)(zz * inv_dzg + 1.0f);
    if (jm1 < 1 || jm1 > (int)nz) continue;
    int i1 = i + 1;
    if (rsq_sh < 0.5f * drdr * (float)(i * i + (i - 1) * (i - 1))) i1 = i - 1;
    i1 = min(max(i1, 1), (int)nx);
    int j1 = jm1 + 1;
    if (zz < ((float)jm1 - 0.5f) * dzg) j1 = jm1 - 1;
    j1 = min(max(j1, 1), (int)nz);
    float a = 1.0f;
    if (i1 != i) {
      float sqrtmp = sqrtf(4.0f * rsq_sh / drdr - 1.0f);
      float rminsq = 0.25f * drdr * (sqrtmp - 1.0f) * (sqrtmp - 1.0f);
      float rmaxsq = rminsq + sqrtmp * drdr;
      if (i1 < i) a = (rmaxsq - (float)((i - 1) * (i - 1)) * drdr) / (rmaxsq - rminsq);
      else a = ((float)((i1 - 1) * (i1 - 1)) * drdr - rminsq) / (rmaxsq - rminsq);
    }
    float cc = 1.0f;
    if (j1 != jm1) cc = (zz - ((float)j1 - 0.5f) * dzg) / ((float)(jm1 - j1) * dzg);
    float bb = 1.0f - a, d = 1.0f - cc;
    int k00 = (jm1 - 1) * (int)nx + i - 1, k01 = k00 + (i1 - i);
    int k10 = (j1 - 1) * (int)nx + i - 1, k11 = k10 + (i1 - i);
    int w00 = __float2int_rn(a * cc * q.scale), w01 = __float2int_rn(bb * cc * q.scale);
    int w10 = __float2int_rn(a * d * q.scale), w11 = __float2int_rn(bb * d * q.scale);
    if (q.smem) {
      if (w00) atomicAdd(hist32 + k00, w00);
      if (w01) atomicAdd(hist32 + k01, w01);
      if (w10) atomicAdd(hist32 + k10, w10);
      if (w11) atomicAdd(hist32 + k11, w11);
    } else {
      if (w00) atomicAdd(t.bin_fx + k00, (unsigned long long)((long long)w00 * m));
      if (w01) atomicAdd(t.bin_fx + k01, (unsigned long long)((long long)w01 * m));
      if (w10) atomicAdd(t.bin_fx + k10, (unsigned long long)((long long)w10 * m));
      if (w11) atomicAdd(t.bin_fx + k11, (unsigned long long)((long long)w11 * m));
    }
    ++cnt;
  }
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&sc->num_on_mesh, cnt);
  if (!q.smem) return;
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) {
    int v = hist32[k];
    if (v) atomicAdd(t.bin_fx + k, (unsigned long long)((long long)v * m));
  }
}

// ---- contraction -------------------------------------------------------------
// Ring-to-mesh field sum (UpdateFldTbl2KernelDouble, space_charge_kernel.cu:
// 472-568) in FP32:  E[zp][rp] = sum over bins (zs, rs) of q(zs, rs) *
// G[rp][rs][dz(zp, zs)], Ez negated for source bins at or above zp.  For one
// beam this is a matrix-vector product (one charge vector against the
// Toeplitz-in-z Green's matrix), so it runs on the FP32 pipes: one block per
// (rp, 32 consecutive zp), warp w sums source rows rs = w (mod 32) for its
// lane's zp, rows staged through shared memory in tiles of the Green's table,
// warp partial sums added in a fixed order.  The set of bins each point sums
// is the reference's (its integer partition of the table; see scheff.cu).
constexpr int kCZ = 32;                 // field points (zp) per block
constexpr int kContractThreads = 1024;  // 32 warps
constexpr int kContractSmem = 96 * 1024;

__global__ void __launch_bounds__(kContractThreads) k32_contract(const ScState *sc, ScTables t) {
  if (!sc->remesh) return;
  const uint32_t nx = sc->nx, nz = sc->nz, fld_sz = nx * nz, nrow = nx + 1;
  const uint32_t rp = blockIdx.x, zp0 = blockIdx.y * kCZ;
  if (rp > nx || zp0 > nz) return;
  extern __shared__ float sm[];
  const uint32_t tile_rs = min((uint32_t)(kContractSmem / (12 * nz)), nx);  // 8 B Green's + 4 B charge per (rs, z)
  float2 *gt = (float2 *)sm;                   // [tile_rs][nz]
  float *bt = sm + 2 * tile_rs * nz;           // [nz][tile_rs]
  __shared__ float red[kContractThreads / 32][kCZ][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nwarp = kContractThreads / 32;
  const uint32_t zp = zp0 + lane;
  uint32_t lim;
  if (zp < nz) {
    uint32_t gnum = 1024 / nz;
    lim = gnum ? gnum * (fld_sz / gnum) : 0;
  } else if (rp < nx) {
    uint32_t gnum = 1024 / nx;
    lim = gnum ? gnum * (fld_sz / gnum) : 0;
  } else {
    lim = (fld_sz / 1024) * 1024;
  }
  const float2 *g1 = (const float2 *)t.ffld1;
  float ax0 = 0.0f, az0 = 0.0f, ax1 = 0.0f, az1 = 0.0f;
  for (uint32_t rs0 = 0; rs0 < nx; rs0 += tile_rs) {
    const uint32_t nrs = min(tile_rs, nx - rs0);
    __syncthreads();
    const float2 *g = g1 + (size_t)rp * fld_sz + (size_t)rs0 * nz;
    for (uint32_t e = threadIdx.x; e < nrs * nz; e += blockDim.x) gt[e] = g[e];
    for (uint32_t e = threadIdx.x; e < nrs * nz; e += blockDim.x) {
      uint32_t zs = e / nrs, r = e % nrs;
      bt[zs * tile_rs + r] = (float)(long long)t.bin_fx[zs * nx + rs0 + r] * (float)kBinInvScale;
    }
    __syncthreads();
    if (zp <= nz) {
      for (uint32_t r = warp; r < nrs; r += nwarp) {
        const float2 *gr = gt + r * nz;
        const uint32_t rs = rs0 + r;
        uint32_t zend = nz;
        if (lim < nz * nx) {  // bins zs * nx + rs >= lim are not summed
          uint32_t zl = lim > rs ? (lim - rs + nx - 1) / nx : 0;
          zend = min(zend, zl);
        }
        uint32_t zs = 0;
        for (; zs + 1 < zend; zs += 2) {
          float bv0 = bt[zs * tile_rs + r], bv1 = bt[(zs + 1) * tile_rs + r];
          bool up0 = zp < nz && zs >= zp, up1 = zp < nz && zs + 1 >= zp;
          float2 gv0 = gr[up0 ? zs - zp : zp - zs - 1];
          float2 gv1 = gr[up1 ? zs + 1 - zp : zp - zs - 2];
          ax0 = fmaf(bv0, gv0.x, ax0);
          az0 = fmaf(up0 ? -bv0 : bv0, gv0.y, az0);
          ax1 = fmaf(bv1, gv1.x, ax1);
          az1 = fmaf(up1 ? -bv1 : bv1, gv1.y, az1);
        }
        if (zs < zend) {
          float bv0 = bt[zs * tile_rs + r];
          bool up0 = zp < nz && zs >= zp;
          float2 gv0 = gr[up0 ? zs - zp : zp - zs - 1];
          ax0 = fmaf(bv0, gv0.x, ax0);
          az0 = fmaf(up0 ? -bv0 : bv0, gv0.y, az0);
        }
      }
    }
  }
  red[warp][lane][0] = ax0 + ax1;
  red[warp][lane][1] = az0 + az1;
  __syncthreads();
  if (warp == 0 && zp <= nz) {
    float sx = 0.0f, sz = 0.0f;
    for (int w = 0; w < nwarp; ++w) { sx += red[w][lane][0]; sz += red[w][lane][1]; }
    size_t pt = (size_t)zp * nrow + rp;
    t.ffld2[2 * pt] = sx;
    t.ffld2[2 * pt + 1] = sz;
  }
}

// ---- kick ----------------------------------------------------------------------
// ApplySpchKickKernel (space_charge_kernel.cu:573-706) in FP32
__global__ void __launch_bounds__(kBlock) k32_kick(DevBeam bm, const ScState *sc, ScTables t, RefK r,
                                                  uint32_t skip_stride) {
  const Sc32Consts &kc = *t.c32;
  const uint32_t nx = sc->nx, nz = sc->nz, adj = sc->adj;
  const float cbgcoef = kc.cbg_per_onm * (float)sc->num_on_mesh;
  const float phimc = kc.phimc, xbar = kc.xbar, ybar = kc.ybar, epsq = kc.epsq, inv_epsq = kc.inv_epsq;
  const float beta = kc.beta, gmg = kc.gmg, inv_dr = kc.inv_dr, inv_dzg = kc.inv_dzg, hl = kc.hl;
  const float rmesh = kc.rmesh, c2 = kc.c2, xfac = kc.xfac, yfac = kc.yfac, pl = kc.pl;
  const float er_c3 = kc.er_c3, ez_c3 = kc.ez_c3, dwc = kc.dwc;
  const uint32_t tbl_sz = (nx + 1) * (nz + 1);
  const float2 *fld = (const float2 *)t.ffld2;
  for (uint32_t indx = blockIdx.x * blockDim.x + threadIdx.x; indx < bm.n; indx += gridDim.x * blockDim.x) {
    const uint32_t lo = bm.loss[indx], ll = bm.lloss[indx];
    const float x = bm.fx[indx], y = bm.fy[indx], xp = bm.fxp[indx], yp = bm.fyp[indx];
    const float phi = bm.fphi_r[indx], dw = bm.fw[indx];
    if (indx % skip_stride == 0 || lo != 0u || ll != 0u) continue;
    float g = fmaf(dw, r.minv, r.g);
    float gm = g + 1.0f;
    float bgz = sqrtf(g * (g + 2.0f));
    float bgx = bgz * xp, bgy = bgz * yp;
    // p* = gamma_c (bgz - beta gm) without cancellation
    float dgc = (dw + dwc) * r.minv;  // gm - gamma_c
    float s0 = dgc * (gm + gmg) / (gmg * (bgz + beta * gm));
    float xxbar = x - xbar, yybar = y - ybar;
    float rr = sqrtf(xxbar * xxbar * inv_epsq + yybar * yybar * epsq);
    if (rr == 0.0f) rr = 1.0e-8f;
    float inv_rr = 1.0f / rr;
    float xovr = xxbar * xfac * inv_rr, yovr = yybar * yfac * inv_rr;
    float z = -c2 * wrap_turns(phi - phimc);
    float cbgr, cbgzs;
    if (rr > rmesh || fabsf(z) > hl) {
      z = -c2 * (phi - phimc);
      float d = sqrtf(z * z + rr * rr);
      float invd3 = 1.0f / (d * d * d);
      float rod3 = rr * invd3, zod3 = z * invd3;
      for (uint32_t nb = 1; nb <= adj; ++nb) {
        float xi = (float)nb;
        for (int lr = 0; lr < 2; ++lr) {
          float sft = z + xi * pl;
          d = sqrtf(sft * sft + rr * rr);
          invd3 = 1.0f / (d * d * d);
          rod3 += rr * invd3;
          zod3 += sft * invd3;
          xi = -xi;
        }
      }
      cbgr = cbgcoef * rod3;
      cbgzs = cbgcoef * zod3;
    } else {
      float ri = rr * inv_dr;
      uint32_t i = 1 + (int)ri;
      float a = ri - (float)(i - 1);
      float bb = 1.0f - a;
      float zi = (z + hl) * inv_dzg;
      uint32_t j = 1 + (int)zi;
      float c = zi - (float)(j - 1);
      float d = 1.0f - c;
      uint32_t l = (j - 1) * (nx + 1) + i;
      uint32_t m = l + (nx + 1);
      if (m >= tbl_sz) m = tbl_sz - 1;
      if (l >= tbl_sz || l < 1) l = tbl_sz - 1;
      if (m < 1) m = 1;
      float2 fl = fld[l], fl1 = fld[l - 1], fm = fld[m], fm1 = fld[m - 1];
      cbgr = er_c3 * (d * (a * fl.x + bb * fl1.x) + c * (a * fm.x + bb * fm1.x));
      cbgzs = ez_c3 * (d * (a * fl.y + bb * fl1.y) + c * (a * fm.y + bb * fm1.y));
    }
    bgx += cbgr * xovr;
    bgy += cbgr * yovr;
    float s = s0 + cbgzs;
    float bgzf = gmg * (s + beta * (1.0f + 0.5f * s * s));
    if (bgzf <= 0.0f) {
      bm.loss[indx] = 9999u;
    } else {
      float s2 = s0 * s0;
      float dbgz = gmg * (cbgzs + beta * (0.5f * cbgzs * (2.0f * s0 + cbgzs) +
                                          s2 * s2 / (4.0f * (1.0f + 0.5f * s2 + sqrtf(1.0f + s2)))));
      float inv_f = 1.0f / bgzf;
      bm.fxp[indx] = bgx * inv_f;
      bm.fyp[indx] = bgy * inv_f;
      float w = r.w + dw;
      bm.fw[indx] = dw + w * (gm + 1.0f) * dbgz / (gm * bgz);
    }
  }
}

DepQ dep_quant(uint32_t n, int grid, size_t hist_bytes) {
  DepQ q;
  uint32_t per = (uint32_t)grid * kBlock;
  uint32_t iters = (n + per - 1) / per;
  uint64_t p = (uint64_t)iters * kBlock;  // particles one block can deposit
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
  launch_pass_f(Op32ScStats{b, nullptr, ScTables{}, 0.0, 0.0, 0.0, 0.0}, b.n, s, st);
  note_launch(3);
}

static ScTables tables32(const ScTables &t) {
  ScTables u = t;
  u.fld2 = nullptr;  // FP32 beams use ffld1 / ffld2
  return u;
}

void sc32_stats(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
                cudaStream_t st) {
  ScTables u = tables32(t);
  if (a.stats_ok) {
    launch_pass_f(Op32GoodPhi{b}, b.n, s, st);
    launch_pass_f(Op32LlossGoodPhi{b}, b.n, s, st);
    launch_pass_f(Op32ScStats{b, sc, u, a.freq, a.frac, a.length, a.current}, b.n, s, st);
    note_launch(3);
  } else {
    k32_decide_only<<<1, kBlock, 0, st>>>(b, sc, u, a.freq, a.frac, a.length, a.current);
    note_launch();
  }
}

void sc32_mesh(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
               cudaStream_t st) {
  ScTables u = tables32(t);
  launch_pass_f(Op32AdjMesh{b, sc, u.c32, a.length, a.current}, b.n, s, st);
  note_launch();
  k32_green<<<4 * 152, kBlock, 0, st>>>(sc, u);
  note_launch();
  if (a.deposit_ok) {
    int grid = (int)std::min<uint32_t>((b.n + kBlock - 1) / kBlock, (uint32_t)kMaxPassBlocks);
    if (grid < 1) grid = 1;
    size_t hb = (size_t)a.nx_max * a.nz_max * sizeof(int);
    if (hb > kMaxHistSmem) hb = 0;
    DepQ q = dep_quant(b.n, grid, hb);
    k32_deposit<<<grid, kBlock, q.smem ? hb : 0, st>>>(b, sc, u, q);
    note_launch();
  }
  dim3 cg(a.nx_max + 1, (a.nz_max + 1 + kCZ - 1) / kCZ);
  k32_contract<<<cg, kContractThreads, kContractSmem, st>>>(sc, u);
  note_launch();
}

void sc32_kick(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, cudaStream_t st) {
  if (!a.skip_stride) return;
  uint32_t stride = a.skip_stride > 0xffffffffull ? 0xffffffffu : (uint32_t)a.skip_stride;
  k32_kick<<<grid_for(b.n), kBlock, 0, st>>>(b, sc, tables32(t), make_refk(b.w_ref, b.mass), stride);
  note_launch();
}

void sc32_configure() {
  static bool done = false;
  if (done) return;
  done = true;
  cudaFuncSetAttribute(k32_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxHistSmem);
  cudaFuncSetAttribute(k32_contract, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
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
// FP32 kernels, on a caller-given charge table
hps_status hps_scheff_field_f32(uint32_t nr, uint32_t nz, const double *bins, const double *mesh, double *field) {
  using namespace hps;
  if (!bins || !mesh || !field) return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field_f32: null pointer");
  if (!nr || !nz || (nr & (nr - 1)) || (nz & (nz - 1)) || nz > 512 || nr > 256)
    return (hps_status)set_error(HPS_ERR_INVALID,
                                 "scheff_field_f32: nr and nz must be powers of two, nz <= 512, nr <= 256");
  sc32_configure();
  size_t nb = (size_t)nr * nz, n1 = (size_t)(nr + 1) * nr * nz * 2, n2 = (size_t)(nz + 1) * (nr + 1) * 2;
  ScState *sc = nullptr;
  Sc32Consts *c32 = nullptr;
  unsigned long long *fx = nullptr;
  double *b = nullptr;
  float *f1 = nullptr, *f2 = nullptr;
  std::vector<float> host(n2);
  cudaError_t e = cudaMalloc((void **)&sc, sizeof(ScState));
  if (e == cudaSuccess) e = cudaMalloc((void **)&c32, sizeof(Sc32Consts));
  if (e == cudaSuccess) e = cudaMalloc((void **)&fx, nb * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b, nb * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void **)&f1, n1 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void **)&f2, n2 * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(sc, 0, sizeof(ScState));
  if (e == cudaSuccess) e = cudaMemset(c32, 0, sizeof(Sc32Consts));
  if (e == cudaSuccess) e = cudaMemset(f2, 0, n2 * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(b, bins, nb * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k32_field_setup<<<1, 1>>>(sc, c32, nr, nz, mesh[0], mesh[1], mesh[2], mesh[3], mesh[4], mesh[5],
                              (uint32_t)mesh[6]);
    k32_bins_to_fixed<<<64, kBlock>>>(b, fx, (uint32_t)nb);
    ScTables t{};
    t.bin_fx = fx;
    t.ffld1 = f1;
    t.ffld2 = f2;
    t.c32 = c32;
    k32_green<<<4 * 152, kBlock>>>(sc, t);
    dim3 cg(nr + 1, (nz + 1 + kCZ - 1) / kCZ);
    k32_contract<<<cg, kContractThreads, kContractSmem>>>(sc, t);
    note_launch(4);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host.data(), f2, n2 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(sc); cudaFree(c32); cudaFree(fx); cudaFree(b); cudaFree(f1); cudaFree(f2);
  if (e != cudaSuccess) return (hps_status)set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
  for (size_t k = 0; k < n2; ++k) field[k] = host[k];
  return HPS_OK;
}

}  // extern "C"
