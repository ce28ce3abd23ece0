// common.cuh -- device-side types shared by the tracking kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/hps_layout.h"

namespace hps {

// src/util/inc/constant.h:7-11
constexpr double CLIGHT = 299.792458;
constexpr double PI = 3.14159265358979323846;
constexpr double TWOPI = 3.14159265358979323846 * 2.0;

constexpr int kBlock = 256;      // threads per block of the particle kernels
constexpr int kMaxPassBlocks = 1216;  // 8 x 152 SMs

// Indices of the per-beam device scalars (same order as HPS_ST_* in the ABI).
enum Stat {
  X_AVG, X_AVG_GOOD, XP_AVG, Y_AVG, Y_AVG_GOOD, YP_AVG, PHI_AVG, PHI_AVG_R, PHI_AVG_GOOD,
  W_AVG, W_AVG_GOOD, X_SIG, X_SIG_GOOD, XP_SIG, Y_SIG, Y_SIG_GOOD, YP_SIG, PHI_SIG,
  PHI_SIG_R, PHI_SIG_GOOD, W_SIG, W_SIG_GOOD, X_EMIT, Y_EMIT, Z_EMIT, R_MAX, ABS_PHI_MAX,
  NSTAT
};

// The reference's per-beam device scalars (src/beam/inc/beam.h:175-263).
struct BeamStats {
  double st[NSTAT];
  uint32_t num_loss, num_lloss, num_good;
  // FP32 beams, SCHEFF statistics fused into the element map before a kick:
  // 0 done; 2 the loss test and the moments sweep still have to run; 1 the
  // loss test changed the good set and the moments sweep runs again
  uint32_t sc_redo;
};

// Particle storage.  FP64 beams use the double arrays; FP32 beams use the
// float arrays, where fphi / fw are offsets from the synchronous particle.
struct DevBeam {
  uint32_t n;
  double mass, charge;
  double *x, *xp, *y, *yp, *phi, *phi_r, *w;
  float *fx, *fxp, *fy, *fyp, *fphi, *fw, *fphi_r;
  uint32_t *loss, *lloss;
  BeamStats *st;
  // FP32 beams: absolute phase and energy of the synchronous (reference)
  // particle the offsets fphi, fw are taken from.  Tracked on the host in
  // FP64 through the same element formulas (on axis) and passed by value.
  double phi_ref, w_ref;
  // launch shape of the FP32 particle sweeps and statistics passes: at most
  // this many blocks per SM (0: as many as the SM holds at once)
  uint32_t sweep_cap;
};

// SCHEFF solver state in device memory (configuration, the adaptive-remesh
// memory of space_charge.h:112-125 and the per-kick decision).
struct ScState {
  uint32_t nx, nz, nx_init, nz_init, nx_max, nz_max, adj_bunch;
  uint32_t good_cnt_old;
  double adj_bunch_w, mesh_w, remesh_val, interval, interval_init;
  double sigr_old, sigz_old, gm_old;
  double dr, dz;                       // scheff_sz (space_charge_kernel.cu:12)
  uint32_t num_on_mesh;                // space_charge_kernel.cu:13
  // decision of the current kick (Scheff::Start, space_charge.cpp:82-139)
  int remesh;
  uint32_t adj;
  double beta, freq, frac;
  double ratio_r, ratio_z, ratio_q, ratio_g;
  uint32_t n_solves;
  int resized;
  // FP32 beams: kicks whose statistics the element map before them could not
  // certify (the loss-test and moments sweeps ran)
  uint32_t n_stat_sweeps;
  // FP64 beams with a field surrogate: this kick's field came from it
  int sur_accepted;
  // the tensor-core contraction gave up a bounded wait (stays set)
  uint32_t tc_error;
};

// Constants of one FP32 SCHEFF kick, formed once per kick in FP32 by the
// thread that takes the space-charge decision, read by every FP32 kernel of
// the kick (FP64 arithmetic per thread or per block would cost more than the
// particle sweeps themselves on GB300).
struct Sc32Consts {
  float pag;                                            // <phi>_good - phi_sync: relative-phase origin
  float phimc, xbar, ybar, epsq, inv_epsq, xfac, yfac;  // bunch centre and aspect
  float beta, gmg, c2, pl;                              // bunch-frame kinematics
  float dr, dzg, inv_dr, inv_dzg, hl, rmesh;            // mesh as seen by the kick (ratio-scaled)
  float dr0, dzg0, inv_dr0, inv_dzg0, hl0;              // mesh of the last solve (deposit, Green's table)
  float cbg_per_onm;                                    // c1 c3 pi/2 (times num_on_mesh)
  float er_c3, ez_c3;                                   // interpolated-field scale
  float dwc;                                            // synchronous particle - bunch-frame energy
  float green_c1;                                       // Green's table scale
};

// Host-side constants of one FP32 kick.  The statistics finalisers run on
// one thread; on GB300 an FP64 divide or square root there costs about a
// microsecond, so FP32 beams take the space-charge decision and form the
// kick's constants in FP32 arithmetic from these (FP64 state fields are kept
// for the solver's memory).
struct Sc32Host {
  float inv_mass;   // 1 / m
  float wave_len;   // c / f of the beam
  float c1;         // 5721.67 I frac / (f 1e6 N m): Green's table and far-field scale
  float length;     // kick length
};

struct ScTables {
  unsigned long long *bin_fx;  // fixed-point deposit, nz_max*nx_max
  double *fld1;                // (nx+1)*nx*nz (x,y interleaved)
  double *fld2;                // (nz+1)*(nx+1) (x,y interleaved)
  float *ffld1, *ffld2;        // FP32 variants (FP32 beams)
  Sc32Consts *c32;             // FP32 beams: constants of the current kick
  // FP32 beams on a tensor-core mesh (contract_tc.cuh): the folded Green's
  // table as split-BF16 MMA tiles, the per-(tile, source radius) partial
  // fields, and the mesh they are sized for (tcg null: no tensor-core path)
  void *tcg;
  float *tcp;
  uint32_t tc_nr, tc_nz;
};

// Kinematics of the reference particle in FP32, for offset arithmetic.
struct RefK {
  float w, g, gam, beta, minv;
};
__host__ __device__ inline RefK make_refk(double w, double mass) {
  double g = w / mass;
  RefK r;
  r.w = (float)w;
  r.g = (float)g;
  r.gam = (float)(g + 1.0);
  r.beta = (float)(sqrt(g * (g + 2.0)) / (g + 1.0));
  r.minv = (float)(1.0 / mass);
  return r;
}

// 1/beta_i - 1/beta_ref for a particle dw above the reference, computed from
// beta_i^2 - beta_r^2 = (gamma_i^2 - gamma_r^2)/(gamma_i^2 gamma_r^2) so the
// difference keeps FP32 relative precision:
//   1/beta_i - 1/beta_r = -(dgamma (gamma_i + gamma_r)) /
//                          (gamma_i gamma_r^2 (beta_i + beta_r) (beta gamma)_i beta_r)
// (one division); also returns g_i = W_i/m, beta_i and (beta gamma)_i.
// square root by the hardware approximation (sqrt.approx.f32: within about
// an ulp; +0 -> +0, negative -> NaN), for the per-particle sweeps
__device__ __forceinline__ float sqrt_fast(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ inline float dinvb(float dw, const RefK &r, float &g, float &beta, float &bg) {
  g = fmaf(dw, r.minv, r.g);
  const float gam = g + 1.0f;
  bg = sqrt_fast(g * (g + 2.0f));
  // both quotients by the two-ulp reciprocal-multiply: the denominators are
  // products of gamma, beta and beta gamma of live particles, far from zero
  // and from overflow
  beta = __fdividef(bg, gam);
  const float dg = dw * r.minv;
  return -__fdividef(dg * (gam + r.gam), gam * r.gam * r.gam * (beta + r.beta) * bg * r.beta);
}
__device__ inline float dinvb(float dw, const RefK &r, float &g, float &beta) {
  float bg;
  return dinvb(dw, r, g, beta, bg);
}

// deposit weights are accumulated as integers: deterministic in any order
constexpr double kBinScale = 68719476736.0;        // 2^36
constexpr double kBinInvScale = 1.0 / 68719476736.0;

// reduction scratch of one beam
struct PassScratch {
  double *part;          // kMaxPassBlocks * 32
  unsigned int *counter; // 1
};

__host__ __device__ inline uint32_t next_pow2(uint32_t x) {
  --x;
  x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
  return ++x;
}

// particles a beam may hold: next_pow2 of the count and the sweeps'
// 32-bit particle indices (index + grid stride) stay in range
constexpr uint32_t kMaxParticles = 1u << 31;

// Beam::SetNumThreadsPerBlock, src/beam/src/beam.cpp:148-168
__host__ __device__ inline void ref_launch(uint32_t n, uint32_t *grid, uint32_t *blck) {
  uint32_t nt = next_pow2(n);
  if (nt > 256) { *grid = nt / 256; *blck = 256; }
  else { *grid = 1; *blck = nt; }
}

inline int pass_blocks(uint32_t n) {
  uint32_t b = (n + 4 * kBlock - 1) / (4 * kBlock);
  if (b < 1) b = 1;
  if (b > (uint32_t)kMaxPassBlocks) b = kMaxPassBlocks;
  return (int)b;
}

// kernel<<<grid, block, smem, st>>>(args...) for kernels named through a
// template parameter
template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args &&...args) {
  kernel<<<grid, block, smem, st>>>(std::forward<Args>(args)...);
}

inline int grid_for(uint32_t n) {
  uint32_t b = (n + kBlock - 1) / kBlock;
  if (b < 1) b = 1;
  if (b > 152u * 16u) b = 152u * 16u;
  return (int)b;
}

}  // namespace hps
