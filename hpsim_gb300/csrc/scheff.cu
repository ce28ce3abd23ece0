// scheff.cu -- the SCHEFF 2D r-z space-charge kick on FP64 particle state.
//
// Reference: Scheff::Start (src/simulation/src/space_charge.cpp:82-139), the
// launcher glue of src/simulation/src/space_charge.cu and the kernels of
// src/simulation/inc/space_charge_kernel.cu.  The reference reads five
// moments back to the host per kick and decides there whether to rebuild the
// mesh; here the statistics, the decision and the mesh sizing all stay on
// the device, so a whole lattice pass is a fixed launch sequence that can be
// captured in a CUDA graph.  Launch sequence per kick:
//   3 statistics sweeps (the last one also decides) -> [max-r sweep when
//   adjacent bunches are on] -> Green's table -> deposit -> contraction ->
//   kick, where the mesh kernels return at once unless the decision was
//   "remesh".
#include <mutex>

#include "../../include/hpsim_gb300.h"
#include "internal.h"
#include "contract.cuh"
#include "reduce.cuh"
#include "scheff_common.cuh"

namespace hps {

namespace {

__device__ inline bool good(const DevBeam &b, uint32_t i) { return (uint32_t)(b.loss[i] + b.lloss[i]) == 0u; }
__device__ inline double surv(const DevBeam &b) { return (double)(uint32_t)(b.n - b.st->num_loss); }


// Beam::UpdateLongitudinalLoss first half: UpdateGoodParticleCount,
// UpdateAvgPhi(true)  (beam.cpp:776-782, 788-791, 846-852)
struct OpGoodPhi {
  static constexpr int K = 2;
  using Comb = SumComb;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    if (!good(b, i)) return;
    a[0] += 1.0;
    a[1] += b.phi[i];
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t ng = (uint32_t)t[0];
    b.st->num_good = ng;
    b.st->st[PHI_AVG_GOOD] = ng > 0 ? t[1] / ng : -99999;
  }
};

// UpdateLongitudinalLossCoordinateKernel + UpdateLossCountKernelCall(lloss)
// + UpdateGoodParticleCount + UpdateAvgPhi(true)  (beam.cpp:780-781, 1008-1009)
struct OpLlossGoodPhi {
  static constexpr int K = 3;
  using Comb = SumComb;
  DevBeam b;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    double lim = b.st->st[PHI_AVG_GOOD];
    uint32_t ll = b.lloss[i];
    if (b.phi[i] > lim + TWOPI + PI) {
      ll = 1u;
      b.lloss[i] = 1u;
    }
    a[0] += ll != 0u;
    if ((uint32_t)(b.loss[i] + ll) == 0u) {
      a[1] += 1.0;
      a[2] += b.phi[i];
    }
  }
  __device__ void finalize(const double *t, int tid, int) const {
    if (tid) return;
    uint32_t ng = (uint32_t)t[1];
    b.st->num_lloss = (uint32_t)t[0];
    b.st->num_good = ng;
    b.st->st[PHI_AVG_GOOD] = ng > 0 ? t[2] / ng : -99999;
  }
};

// The rest of UpdateStatForSpaceCharge (beam.cpp:1010-1014): relative phase
// about <phi>_good for every particle, <phi_r> over loss == 0 divided by
// num - num_loss, sigma(phi_r) over good particles, <x>, sigma_x, <y>,
// sigma_y over good particles divided by num - num_loss
// (UpdateHorizontalAvgSigKernel), <w> over good particles; then, when a
// solver is attached, the Scheff::Start decision.
struct OpScStats {
  static constexpr int K = 8;
  using Comb = SumComb;
  DevBeam b;
  ScState *sc;
  ScTables t;
  double freq, frac;
  __device__ bool enabled() const { return true; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    double pr = rel_phase(b.phi[i], b.st->st[PHI_AVG_GOOD]);
    b.phi_r[i] = pr;
    if (b.loss[i] != 0u) return;
    a[0] += pr;
    if (b.lloss[i] != 0u) return;
    double x = b.x[i], y = b.y[i];
    a[1] += pr; a[2] += pr * pr;
    a[3] += x; a[4] += x * x; a[5] += y; a[6] += y * y;
    a[7] += b.w[i];
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
      st.st[W_AVG_GOOD] = st.num_good > 0 ? s[7] / st.num_good : -99999;
      if (sc) scheff_decide(b, sc, freq, frac);
    }
    if (!sc) return;
    __syncthreads();
    zero_mesh_tables(sc, t, tid, nth);
  }
};

// UpdateMaxRPhi + UpdateScheffMeshSizeKernel(r_max, coef = 1) when adjacent
// bunches are on (space_charge.cu:124-128)
struct OpAdjMesh {
  static constexpr int K = 2;
  using Comb = MaxComb;
  DevBeam b;
  ScState *sc;
  __device__ bool enabled() const { return sc->remesh && sc->adj != 0u; }
  __device__ void particle(uint32_t i, double (&a)[K]) const {
    if (b.loss[i] != 0u) return;
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
    mesh_size(sc, b.st->st[R_MAX], 0.0, 1.0);
  }
};

// Scheff::Start with num_particle <= 2: statistics are not refreshed, the
// decision still runs on whatever they hold.
__global__ void k_decide_only(DevBeam b, ScState *sc, ScTables t, double freq, double frac) {
  if (threadIdx.x == 0) scheff_decide(b, sc, freq, frac);
  __syncthreads();
  zero_mesh_tables(sc, t, threadIdx.x, blockDim.x);
}

// UpdateFldTbl1Kernel, space_charge_kernel.cu:39-100 (one thread per table
// entry; rows rs >= (nr/by)*by are not written, as in the reference's grid);
// not needed when a field surrogate's field was accepted
__global__ void k_green(const ScState *sc, ScTables t, uint32_t num_part, double cur_ov_mc2) {
  if (!sc->remesh || sc->sur_accepted) return;
  const uint32_t nr = sc->nx, nz = sc->nz;
  const uint32_t by = (512 / nz < nr) ? 512 / nz : nr;
  const uint32_t nrs = by ? (nr / by) * by : 0;
  const uint32_t total = (nr + 1) * nrs * nz;
  const double r_beta = sc->beta, r_freq = sc->freq;
  const uint32_t adj = sc->adj;
  const double gm = rsqrt(1.0 - r_beta * r_beta);
  const double dr = sc->dr, dzg = sc->dz * gm;
  const double wave_len = CLIGHT / r_freq;
  const double pl = r_beta * gm * wave_len;
  const double c1 = 5721.67 * cur_ov_mc2 / (r_freq * 1e6 * (double)num_part);
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    uint32_t tz = e % nz;
    uint32_t k = (e / nz) % nrs;
    uint32_t rpi = e / (nz * nrs);
    double rs = sqrt(0.5 * (k * k + (k + 1) * (k + 1))) * dr;
    double zs = 0.5 * dzg;
    double zp = (tz + 1) * dzg;
    double rp = rpi * dr;
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
    for (uint32_t i = 1; i <= adj; ++i) {
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
    size_t cnt = (size_t)rpi * nr * nz + (size_t)k * nz + tz;
    t.fld1[2 * cnt] = c1 * er1;
    t.fld1[2 * cnt + 1] = c1 * ez1;
  }
}

__device__ inline void dep_add(unsigned long long *h, int k, double v) {
  long long q = __double2ll_rn(v * kBinScale);
  if (q) atomicAdd(h + k, (unsigned long long)q);
}

// DistributeParticleKernel, space_charge_kernel.cu:123-224: each block
// deposits into its own histogram in shared memory (integer weights), then
// adds it to the global table; integer sums make the table independent of
// the order in which particles arrive.
__global__ void k_deposit(DevBeam bm, ScState *sc, ScTables t) {
  if (!sc->remesh) return;
  extern __shared__ unsigned long long hist[];
  const uint32_t nx = sc->nx, nz = sc->nz, nb = nx * nz;
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) hist[k] = 0ull;
  __syncthreads();
  const BeamStats &st = *bm.st;
  const double phimc = st.st[PHI_AVG_R], xbar = st.st[X_AVG_GOOD], ybar = st.st[Y_AVG_GOOD];
  const double epsq = st.st[X_SIG_GOOD] / st.st[Y_SIG_GOOD];
  const double r_beta = sc->beta, r_freq = sc->freq;
  const double gm = rsqrt(1.0 - r_beta * r_beta);
  const double dr = sc->dr, dzg = sc->dz * gm;
  const double wave_len = CLIGHT / r_freq;
  const double hl = nz * 0.5 * dzg;
  const double c2 = r_beta * gm * wave_len / TWOPI;
  uint32_t cnt = 0;
  for (uint32_t np = blockIdx.x * blockDim.x + threadIdx.x; np < bm.n; np += gridDim.x * blockDim.x) {
    if (!(bm.loss[np] == 0u && bm.lloss[np] == 0u)) continue;
    double x = bm.x[np], y = bm.y[np], z = bm.phi_r[np];
    double rsq_sh = (x - xbar) * (x - xbar) / epsq + (y - ybar) * (y - ybar) * epsq;
    int i = (int)(sqrt(rsq_sh) / dr + 1);
    if (!(i >= 1 && (uint32_t)i <= nx)) continue;
    double ddz = z - phimc;
    for (int guard = 0; (ddz > PI || ddz < -PI) && guard < 1000000; ++guard) {
      if (ddz > 0.0) ddz -= TWOPI;
      else ddz += TWOPI;
    }
    z = -c2 * ddz;
    if (!(fabs(z) < hl)) continue;
    double zz = z + hl;
    int jm1 = (int)(zz / dzg + 1);
    int i1 = i + 1;
    double drdr = dr * dr;
    if (rsq_sh < 0.5 * drdr * (double)(i * i + (i - 1) * (i - 1))) i1 = i - 1;
    if (i1 < 1) i1 = 1;
    if (i1 > (int)nx) i1 = nx;
    int j1 = jm1 + 1;
    if (zz < (jm1 - 1 + 0.5) * dzg) j1 = jm1 - 1;
    if (j1 < 1) j1 = 1;
    if (j1 > (int)nz) j1 = nz;
    if (jm1 < 1 || jm1 > (int)nz) continue;  // cannot happen for |z| < hl
    double a;
    if (i1 == i) a = 1.0;
    else {
      double sqrtmp = sqrt(4.0 * rsq_sh / drdr - 1.0);
      double rminsq = 0.25 * drdr * (sqrtmp - 1.0) * (sqrtmp - 1.0);
      double rmaxsq = rminsq + sqrtmp * drdr;
      if (i1 < i) a = (rmaxsq - (i - 1) * (i - 1) * drdr) / (rmaxsq - rminsq);
      else a = ((i1 - 1) * (i1 - 1) * drdr - rminsq) / (rmaxsq - rminsq);
    }
    double cc = 1.0;
    if (j1 != jm1) cc = (zz - (j1 - 1 + 0.5) * dzg) / ((jm1 - j1) * dzg);
    double bb = 1.0 - a, d = 1.0 - cc;
    int k = (jm1 - 1) * nx + i;
    dep_add(hist, k - 1, a * cc);
    k += i1 - i;
    dep_add(hist, k - 1, bb * cc);
    k = (j1 - 1) * nx + i;
    dep_add(hist, k - 1, a * d);
    k += i1 - i;
    dep_add(hist, k - 1, bb * d);
    ++cnt;
  }
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&sc->num_on_mesh, cnt);
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) {
    unsigned long long v = hist[k];
    if (v) atomicAdd(t.bin_fx + k, v);
  }
}


// ApplySpchKickKernel, space_charge_kernel.cu:573-706.  The reference's
// grid-stride loop `while (indx > 0 && ...)` ends thread 0 before its first
// particle, so particles whose index is a multiple of its launch's thread
// count (skip_stride) are never kicked; the same set is skipped here.
__global__ void k_kick(DevBeam bm, const ScState *sc, ScTables t, double length, double current,
                       uint64_t skip_stride) {
  const uint32_t nx = sc->nx, nz = sc->nz;
  const double r_beta = sc->beta, r_freq = sc->freq, r_mass = bm.mass;
  const double r_current = current * sc->frac;
  const double rr = sc->ratio_r, rz = sc->ratio_z, rq = sc->ratio_q, rg = sc->ratio_g;
  const BeamStats &st = *bm.st;
  const double phimc = st.st[PHI_AVG_R], xbar = st.st[X_AVG_GOOD], ybar = st.st[Y_AVG_GOOD];
  const double epsq = st.st[X_SIG_GOOD] / st.st[Y_SIG_GOOD];
  const double gmg = rsqrt(1.0 - r_beta * r_beta);
  const double dr = sc->dr * rr;
  const double dzg = sc->dz * gmg * rz;
  const double wave_len = CLIGHT / r_freq;
  const double hl = nz * 0.5 * dzg;
  const double c1 = 5721.67 * r_current / (r_freq * 1e6 * (double)bm.n * r_mass);
  const double c2 = r_beta * gmg * wave_len / TWOPI;
  const double c3 = length / (r_beta * gmg);
  const double xfac = 2.0 / (epsq + 1.0);
  const double yfac = epsq * xfac;
  const uint32_t adj = sc->adj, onm = sc->num_on_mesh;
  const uint32_t tbl_sz = (nx + 1) * (nz + 1);
  const double *fld = t.fld2;
  for (uint32_t indx = blockIdx.x * blockDim.x + threadIdx.x; indx < bm.n; indx += gridDim.x * blockDim.x) {
    if (indx % skip_stride == 0) continue;
    if (!(bm.loss[indx] == 0u && bm.lloss[indx] == 0u)) continue;
    double x = bm.x[indx], y = bm.y[indx], xp = bm.xp[indx], yp = bm.yp[indx];
    double phi = bm.phi_r[indx], w = bm.w[indx];
    double cbgr, cbgzs;
    double gm = w / r_mass + 1.0;
    double bgz = sqrt((gm - 1.0) * (gm + 1.0));
    double bgx = bgz * xp;
    double bgy = bgz * yp;
    double bgzstar = gmg * (bgz - r_beta * gm);
    double xxbar = x - xbar, yybar = y - ybar;
    double r = sqrt(xxbar * xxbar / epsq + yybar * yybar * epsq);
    if (r == 0.0) r = 1.0e-8;
    double xovr = xxbar * xfac / r;
    double yovr = yybar * yfac / r;
    double ddz = phi - phimc;
    for (int guard = 0; (ddz > PI || ddz < -PI) && guard < 1000000; ++guard) {
      if (ddz > 0.0) ddz -= TWOPI;
      else ddz += TWOPI;
    }
    double z = -c2 * ddz;
    if (r > nx * dr || fabs(z) > hl) {
      z = -c2 * (phi - phimc);
      double d = sqrt(z * z + r * r);
      double invd3 = 1.0 / (d * d * d);
      double rod3 = r * invd3;
      double zod3 = z * invd3;
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
      uint32_t i = 1 + (int)(r / dr);
      double a = r / dr - (i - 1.0);
      double bb = 1.0 - a;
      uint32_t j = 1 + (int)((z + hl) / dzg);
      double c = (z + hl) / dzg - (j - 1.0);
      double d = 1.0 - c;
      uint32_t l = (j - 1) * (nx + 1) + i;
      uint32_t m = l + (nx + 1);
      if (m >= tbl_sz) m = tbl_sz - 1;
      // l leaves the table only for r == nx*dr with z == hl, or NaN input
      if (l >= tbl_sz || l < 1) l = tbl_sz - 1;
      if (m < 1) m = 1;
      double er_ratio = rq / (rr * rz * rg * rg);
      double ez_ratio = rq / (rz * rz);
      cbgr = er_ratio * c3 * (d * (a * fld[2 * l] + bb * fld[2 * (l - 1)]) + c * (a * fld[2 * m] + bb * fld[2 * (m - 1)]));
      cbgzs = ez_ratio * c3 * (d * (a * fld[2 * l + 1] + bb * fld[2 * (l - 1) + 1]) +
                               c * (a * fld[2 * m + 1] + bb * fld[2 * (m - 1) + 1]));
    }
    bgx += cbgr * xovr;
    bgy += cbgr * yovr;
    bgzstar += cbgzs;
    double gstar = 1.0 + 0.5 * bgzstar * bgzstar;
    double bgzf = gmg * (bgzstar + r_beta * gstar);
    if (bgzf <= 0.0) bm.loss[indx] = 9999u;
    else {
      bm.xp[indx] = bgx / bgzf;
      bm.yp[indx] = bgy / bgzf;
      bm.w[indx] *= 1.0 + (gm + 1.0) * (bgzf - bgz) / (gm * bgz);
    }
  }
}

}  // namespace

void beam_update_stat_for_sc(const DevBeam &b, PassScratch s, cudaStream_t st) {
  if (b.n <= 2) return;
  launch_pass(OpGoodPhi{b}, b.n, s, st);
  launch_pass(OpLlossGoodPhi{b}, b.n, s, st);
  launch_pass(OpScStats{b, nullptr, ScTables{}, 0.0, 0.0}, b.n, s, st);
  note_launch(3);
}

void sc_stats(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
              cudaStream_t st) {
  if (a.stats_ok) {
    launch_pass(OpGoodPhi{b}, b.n, s, st);
    launch_pass(OpLlossGoodPhi{b}, b.n, s, st);
    launch_pass(OpScStats{b, sc, t, a.freq, a.frac}, b.n, s, st);
    note_launch(3);
  } else {
    k_decide_only<<<1, kBlock, 0, st>>>(b, sc, t, a.freq, a.frac);
    note_launch();
  }
}

// UpdateFldTbl2KernelDouble (space_charge_kernel.cu:472-568) on the FP64
// tables: contract.cuh's ring-convolution kernel, grid and shared memory
// sized for the largest mesh the solver takes
void contract64(const ScState *sc, const ScTables &t, uint32_t nx_max, uint32_t nz_max, cudaStream_t st) {
  static PerDevice configured;
  configured.once([] { contract_configure<double>(); });
  contract_launch<double>(sc, t, nx_max, nz_max, st);
}

void sc_mesh(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
             cudaStream_t st, const SurNet *sur) {
  launch_pass(OpAdjMesh{b, sc}, b.n, s, st);
  note_launch();
  // mesh kernels are sized for the largest mesh this solver can take; with a
  // field surrogate the deposit comes first, and an accepted surrogate field
  // makes the Green's table and the contraction return at once
  if (!sur) {
    k_green<<<2 * 152, kBlock, 0, st>>>(sc, t, b.n, a.current * a.frac / b.mass);
    note_launch();
  }
  if (a.deposit_ok) {
    k_deposit<<<grid_for(b.n), kBlock, a.deposit_smem, st>>>(b, sc, t);
    note_launch();
  }
  if (sur) {
    sur_solve(b, sc, t, a, *sur, st);
    k_green<<<2 * 152, kBlock, 0, st>>>(sc, t, b.n, a.current * a.frac / b.mass);
    note_launch();
  }
  contract64(sc, t, a.nx_max, a.nz_max, st);
  note_launch();
}

void sc_kick(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, cudaStream_t st) {
  if (a.skip_stride) {
    k_kick<<<grid_for(b.n), kBlock, 0, st>>>(b, sc, t, a.length, a.current, a.skip_stride);
    note_launch();
  }
}

// Green's table in FP64 for the FP32 solver too: its elliptic-integral fits
// difference two O(1) terms into an O(r^2/d^2) far field
void sc_green(const ScState *sc, const ScTables &t, uint32_t num_part, double cur_ov_mc2, cudaStream_t st) {
  k_green<<<2 * 152, kBlock, 0, st>>>(sc, t, num_part, cur_ov_mc2);
  note_launch();
}

// the limit only grows, per device (the attribute is per device)
void sc_configure(size_t max_deposit_smem) {
  static std::mutex m;
  static size_t configured[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaFuncSetAttribute(k_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_deposit_smem);
    return;
  }
  std::lock_guard<std::mutex> lock(m);
  if (max_deposit_smem <= configured[dev]) return;
  configured[dev] = max_deposit_smem;
  cudaFuncSetAttribute(k_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_deposit_smem);
}

// ---- standalone field solve: charge table -> field table ------------------

namespace {

// Mesh description of a standalone solve (what Scheff::Start would have
// settled on before UpdateTblsKernelCall / UpdateFinalFldTblKernelCall).
__global__ void k_field_setup(ScState *sc, uint32_t nr, uint32_t nz, double dr, double dz, double beta,
                              double freq, uint32_t adj) {
  sc->nx = nr; sc->nz = nz; sc->nx_init = nr; sc->nz_init = nz; sc->nx_max = nr; sc->nz_max = nz;
  sc->dr = dr; sc->dz = dz; sc->beta = beta; sc->freq = freq; sc->adj = adj;
  sc->remesh = 1;
}

// charge table in FP64 -> the deposit's fixed-point table
__global__ void k_bins_to_fixed(const double *bins, unsigned long long *fx, uint32_t nb) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x)
    fx[k] = (unsigned long long)__double2ll_rn(bins[k] * kBinScale);
}

bool mesh_ok(uint32_t nr, uint32_t nz) {
  return nr && nz && !(nr & (nr - 1)) && !(nz & (nz - 1)) && nz <= 512 && nr <= 256;
}

}  // namespace

// Green's table + contraction for a given charge table (UpdateFldTbl1Kernel
// and UpdateFldTbl2KernelDouble).  sc, fx, fld1 and fld2 are device buffers
// sized for (nr, nz); fld2 is overwritten.
// Returns the status of the field table's clearing or of the launches.
cudaError_t sc_field_solve(ScState *sc, unsigned long long *fx, double *fld1, double *fld2, uint32_t nr, uint32_t nz,
                           const double *bins_dev, const double *mesh, cudaStream_t st) {
  k_field_setup<<<1, 1, 0, st>>>(sc, nr, nz, mesh[0], mesh[1], mesh[2], mesh[3], (uint32_t)mesh[6]);
  k_bins_to_fixed<<<64, kBlock, 0, st>>>(bins_dev, fx, nr * nz);
  const cudaError_t me = cudaMemsetAsync(fld2, 0, (size_t)(nz + 1) * (nr + 1) * 2 * sizeof(double), st);
  if (me != cudaSuccess) return me;
  ScTables t{};
  t.bin_fx = fx;
  t.fld1 = fld1;
  t.fld2 = fld2;
  k_green<<<2 * 152, kBlock, 0, st>>>(sc, t, (uint32_t)mesh[4], mesh[5]);
  contract64(sc, t, nr, nz, st);
  note_launch(4);
  return cudaGetLastError();
}

}  // namespace hps

extern "C" {

// UpdateTblsKernelCall (Green's table part) + UpdateFinalFldTblKernelCall,
// src/simulation/src/space_charge.cu:148-218, on a caller-given charge table.
hps_status hps_scheff_field(uint32_t nr, uint32_t nz, const double *bins, const double *mesh, double *field) {
  using namespace hps;
  if (!bins || !mesh || !field) return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field: null pointer");
  if (!mesh_ok(nr, nz))
    return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field: nr and nz must be powers of two, nz <= 512, nr <= 256");
  size_t nb = (size_t)nr * nz, n1 = (size_t)(nr + 1) * nr * nz * 2, n2 = (size_t)(nz + 1) * (nr + 1) * 2;
  ScState *sc = nullptr;
  unsigned long long *fx = nullptr;
  double *b = nullptr, *f1 = nullptr, *f2 = nullptr;
  cudaError_t e = cudaMalloc((void **)&sc, sizeof(ScState));
  if (e == cudaSuccess) e = cudaMalloc((void **)&fx, nb * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b, nb * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void **)&f1, n1 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void **)&f2, n2 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(sc, 0, sizeof(ScState));
  if (e == cudaSuccess) e = cudaMemcpy(b, bins, nb * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = sc_field_solve(sc, fx, f1, f2, nr, nz, b, mesh, 0);
  if (e == cudaSuccess) e = cudaMemcpy(field, f2, n2 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(sc); cudaFree(fx); cudaFree(b); cudaFree(f1); cudaFree(f2);
  if (e != cudaSuccess) return (hps_status)set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
  return HPS_OK;
}

}  // extern "C"

// ---- field solve without allocation --------------------------------------
//
// Some callers cannot allocate device memory while they run: an online model
// that re-solves the space-charge field inside a control-system cycle and
// must not wait on the CUDA allocator, or a host application that owns the
// whole device through its own memory pool and hands its plugins finished
// buffers.  hps_scheff_field_noalloc serves them: the caller supplies the
// charge table and the field table in device memory, and the intermediate
// tables live in one statically sized device array of this library (held
// by every GPU that loads the library until the process exits).
namespace hps {
namespace {

constexpr uint32_t kNoAllocMaxBins = 4096;                // nr * nz
constexpr uint32_t kNoAllocMaxGreen = 33u * 32u * 128u;   // (nr + 1) * nr * nz
constexpr size_t kNoAllocStateBytes = 256;
constexpr size_t kNoAllocBytes =
    kNoAllocStateBytes + kNoAllocMaxBins * sizeof(unsigned long long) + (size_t)kNoAllocMaxGreen * 2 * sizeof(double);
static_assert(sizeof(ScState) <= kNoAllocStateBytes, "ScState outgrew its slot in the static scratch");

// state block | fixed-point charge table | Green's table
static __device__ __align__(256) unsigned char g_field_scratch[kNoAllocBytes];

std::mutex g_scratch_mutex;
void *g_scratch_addr[kMaxDevices];  // device address of g_field_scratch, per device

// Device address of the scratch array on the current device.  The symbol's
// name is only a host-side handle: the address has to be asked for once per
// device, with that device current.  The cached address belongs to the
// device's current context: after cudaDeviceReset the library has to be
// reloaded before this entry point is used on that device again.
int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(HPS_ERR_UNSUPPORTED, "scheff_field_noalloc: device index too large");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_field_scratch);
    if (e != cudaSuccess) return set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return HPS_OK;
}

}  // namespace
}  // namespace hps

extern "C" {

// Same computation as hps_scheff_field on device buffers, allocating nothing.
// The first call on a device looks up the scratch array's device address;
// make that first call before any stream capture.  Meshes are limited to
// nr*nz <= 4096 and (nr+1)*nr*nz <= 135168 (32 x 128 at most for nr = 32);
// larger ones are rejected.  All calls share the scratch, so calls whose
// work overlaps on the GPU (different streams, or other threads) race; the
// scratch keeps the previous call's tables, and every entry this call reads
// is rewritten first.  The field table is cleared before it is summed into.
hps_status hps_scheff_field_noalloc(uint32_t nr, uint32_t nz, const double *bins_dev, const double *mesh,
                                    double *field_dev, void *stream) {
  using namespace hps;
  if (!bins_dev || !mesh || !field_dev) return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field_noalloc: null pointer");
  if (!mesh_ok(nr, nz))
    return (hps_status)set_error(HPS_ERR_INVALID, "scheff_field_noalloc: nr and nz must be powers of two");
  if ((size_t)nr * nz > kNoAllocMaxBins || (size_t)(nr + 1) * nr * nz > kNoAllocMaxGreen)
    return (hps_status)set_error(HPS_ERR_INVALID,
                                 "scheff_field_noalloc: mesh too large for the static scratch "
                                 "(limit nr*nz <= 4096 and (nr+1)*nr*nz <= 135168, e.g. 32 x 128)");
  // an error left pending by earlier work is the caller's, not this call's
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess)
    return (hps_status)set_error(HPS_ERR_CUDA, (std::string("scheff_field_noalloc: an earlier CUDA error is "
                                                            "pending: ") + cudaGetErrorString(pending)).c_str());
  void *base = nullptr;
  int st = scratch_address(&base);
  if (st != HPS_OK) return (hps_status)st;
  unsigned char *p = (unsigned char *)base;
  ScState *sc = (ScState *)p;
  unsigned long long *fx = (unsigned long long *)(p + kNoAllocStateBytes);
  double *fld1 = (double *)(p + kNoAllocStateBytes + kNoAllocMaxBins * sizeof(unsigned long long));
  const cudaError_t e = sc_field_solve(sc, fx, fld1, field_dev, nr, nz, bins_dev, mesh, (cudaStream_t)stream);
  if (e != cudaSuccess) return (hps_status)set_error(HPS_ERR_CUDA, cudaGetErrorString(e));
  return HPS_OK;
}

}  // extern "C"
