// internal.h -- launchers shared between the translation units of the
// library (host-side declarations; no device code).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace hps {

// count of kernel launches issued by this library (hps_kernel_launch_count)
void note_launch(int n = 1);
// record the message returned by hps_last_error() and pass the status through
int set_error(int status, const char *msg);

// Kernel attributes (the dynamic shared-memory limit above 48 KB) belong to
// the device that was current when they were set.  PerDevice runs a set-up
// once on every device the process uses, with that device current; a
// device index beyond the table runs it at every call.
constexpr int kMaxDevices = 64;
struct PerDevice {
  std::mutex m;
  bool done[kMaxDevices] = {};
  template <class F>
  void once(F &&f) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
      f();
      return;
    }
    std::lock_guard<std::mutex> lock(m);
    if (!done[dev]) {
      f();
      done[dev] = true;
    }
  }
};

// ---- beam reductions and small beam kernels (beam_ops.cu) -------------
void beam_update_loss(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_update_lloss_count(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_update_good_count(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_update_avg(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st);
void beam_update_sig(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st);
void beam_update_emittance(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_update_relative_phi(const DevBeam &b, int use_good, cudaStream_t st);
void beam_update_longitudinal_loss(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_update_avg_xy(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_update_max_r_phi(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam_change_frequency(const DevBeam &b, double ratio, PassScratch s, cudaStream_t st);
void beam_apply_cut(const DevBeam &b, int coord, double lo, double hi, cudaStream_t st);
void beam_shift(const DevBeam &b, int coord, double val, cudaStream_t st);
void beam_set_ref(const DevBeam &b, int coord, double val, cudaStream_t st);
void beam_monitor(const DevBeam &b, const ScState *sc, double *mon_dev, uint32_t elem,
                  PassScratch s, cudaStream_t st);

// ---- element transfer maps (push.cu) ------------------------------------
struct GapArgs {
  double length, frequency, clbl, amplitude, phase_ref, phase_shift, energy_out, beta_center,
      dg, t, tp, sp, fbc, fbm, ta[6], sa[5];
  double design_w_in, phi_in, q1, q2, wl;
  uint32_t ccl_cell_num;
  int ccl;
};
void load_gap_args(const double *p, GapArgs *g);

void push_partial_drift(const DevBeam &b, double wl, double hf, double aper, uint32_t eid, cudaStream_t st);
void push_half_quad(const DevBeam &b, double wl, double len, double aper, double grad, uint32_t eid,
                    cudaStream_t st);
void push_steerer(const DevBeam &b, double blh, double blv, cudaStream_t st);
void push_gap_first(const DevBeam &b, const GapArgs &g, cudaStream_t st);
void push_gap_second(const DevBeam &b, const GapArgs &g, cudaStream_t st);
void push_buncher(const DevBeam &b, double wl, double w_ref, double freq, double voltage, double phase,
                  double aper, double freq_ratio, uint32_t eid, cudaStream_t st);
void push_rotation(const DevBeam &b, double angle, cudaStream_t st);
void push_aperture(const DevBeam &b, int rect, const double *p, uint32_t eid, cudaStream_t st);
void push_dipole(const DevBeam &b, const double *p, double wl, int second, cudaStream_t st);

// ---- SCHEFF (scheff.cu) -------------------------------------------------
struct ScKickArgs {
  double freq;          // beam frequency (Beam::freq) at the kick
  double current;       // beam current (Beam::current) at the kick
  double frac;          // space-charge fraction (SpaceCharge::fraction_)
  double length;        // kick length
  uint64_t skip_stride; // particles i % skip_stride == 0 are not kicked (0: no kick launch)
  int deposit_ok;       // DistributeParticleKernel launch is valid (blck_size/4 > 0)
  int stats_ok;         // num_particle > 2 (UpdateStatForSpaceCharge runs)
  size_t deposit_smem;  // bytes of the per-block histogram (largest mesh)
  uint32_t nx_max, nz_max;  // largest mesh the solver's tables hold
  int adj_possible;         // adjacent bunches configured (else r_max never sizes the mesh)
  bool mesh_fixed;          // the kick's mesh is the largest one (no mesh-size cut-off energy)
  uint32_t dep_per_sm;      // FP32 deposit: blocks per SM (launch shape)
  uint32_t dep_agg;         // FP32 deposit: warp-aggregated histogram adds (launch shape)
  uint32_t dep_threads;     // FP32 deposit: threads per block, 256 | 512 | 1024 (launch shape)
};
// allow the deposit kernel the shared memory of the largest mesh
void sc_configure(size_t max_deposit_smem);
// Scheff::Start split in three phases: statistics + decision, mesh (Green's
// table, deposit, contraction; no-ops unless remeshing), kick
void sc_stats(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
              cudaStream_t st);
struct SurNet;
void sc_mesh(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
             cudaStream_t st, const SurNet *sur = nullptr);
void sc_kick(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, cudaStream_t st);
void beam_update_stat_for_sc(const DevBeam &b, PassScratch s, cudaStream_t st);
// Green's table (k_green) for a solver whose state says "remesh"
void sc_green(const ScState *sc, const ScTables &t, uint32_t num_part, double cur_ov_mc2, cudaStream_t st);

// ---- SCHEFF field surrogate (nn.cu, surrogate.cu) ------------------------
// dims = {batch, c_in, c_out, h_in, w_in, stride, up}; skip may be null
void nn_conv_forward(const int32_t *dims, const void *x, const void *w, const float *bias, int relu,
                     const void *skip, void *y, cudaStream_t st);
void nn_gmean_forward(void *y, int planes, int hw, cudaStream_t st);
// the tensor-core forward (inference): bytes of a layer's weight tiles (0:
// the kernel does not take the shape), their layout from BF16 weights, and
// the layer; *err is set when a pipeline wait gave up
size_t conv_tc_tile_bytes(const int32_t *dims);
void conv_tc_prepare(const int32_t *dims, const void *w, void *tiles, cudaStream_t st);
void nn_conv_forward_tc(const int32_t *dims, const void *x, const void *tiles, const float *bias, int relu,
                        const void *skip, void *y, unsigned int *err, cudaStream_t st);

// A trained network attached to a solver, its device buffers (batch of one)
// and its acceptance test
struct SurNet {
  std::vector<std::array<int, 5>> arch;  // c_in, c_out, stride, up, relu
  std::vector<int32_t> dims;             // 7 per layer
  std::vector<int> hw, skip;             // output plane size; layer whose output is added (-1: none)
  int gmean_after = -1;
  std::vector<void *> w, act;            // BF16 weights and outputs
  std::vector<void *> wt;                // per layer: weight tiles of the tensor-core kernel (null: not taken)
  bool use_tc = true;                    // layers with tiles run on the tensor cores
  std::vector<float *> b;
  void *x = nullptr, *spot = nullptr, *d = nullptr;
  uint32_t nr = 0, nz = 0, n_samples = 0;
  double out_scale = 1.0, tol = 0.0;
  SurNet() = default;
  SurNet(const SurNet &) = delete;
  SurNet &operator=(const SurNet &) = delete;
  ~SurNet();
};
// 0 ok, 1 invalid (err says why), 2 device error
int sur_build(SurNet &n, int n_layers, const int32_t *arch, int gmean_after, const int32_t *skip,
              const uint16_t *const *weights, const float *const *biases, uint32_t nr, uint32_t nz, double out_scale,
              double tol, uint32_t n_samples, std::string &err);
// after the deposit of a kick: the network's field, checked at spot points,
// accepted into the field table (the FP32 one with fp32 != 0) or left to the
// contraction
void sur_solve(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, const SurNet &n,
               cudaStream_t st, int fp32 = 0);
int sur_read(const SurNet &n, double *accepted, double *rejected, double *residual);
// layers on the tensor cores; whether a tensor-core layer's wait gave up
int sur_conv_state(const SurNet &n, int *tc_layers, unsigned int *err);

// ---- FP32 beams (push32.cu, beam32.cu, scheff32.cu) ----------------------
// the statistics after a PUSH_SCSTATS map that could not certify its own:
// the longitudinal-loss test and the SCHEFF moments in one sweep, repeated
// only when the test flagged a particle (the good set, hence <phi>_good,
// changed).  Both sweeps return at once when they are not needed.
void sc32_stats_after_push(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a,
                           PassScratch s, cudaStream_t st);
// An element map fused with the space-charge sweep next to it:
//  PUSH_SCSTATS     the map, then every statistic of the kick after it from
//                   the new state, the decision and the kick's constants,
//                   when the sweep can certify them (else sc_redo = 2 and
//                   sc32_stats_after_push completes them);
//  PUSH_AFTER_KICK  the SCHEFF kick, then the map, in one sweep.
enum { PUSH_SCSTATS = 1, PUSH_AFTER_KICK = 2 };
struct PushFuse {
  int mode;
  PassScratch scr;      // PUSH_SCSTATS: reduction scratch
  ScState *sc;          // solver state and tables
  ScTables t;
  uint64_t skip_mask;   // PUSH_AFTER_KICK: skipped set (i & mask == 0)
  Sc32Host h;           // PUSH_SCSTATS: host constants, beam frequency, fraction
  double freq, frac;
  int s_last;           // PUSH_SCSTATS: a kick of this simulation call came before
};

// Launchers that move the synchronous particle update b.phi_ref / b.w_ref.
void push32_partial_drift(DevBeam &b, double wl, double hf, double aper, uint32_t eid, cudaStream_t st,
                          const PushFuse *pf = nullptr);
void push32_half_quad(DevBeam &b, double wl, double len, double aper, double grad, uint32_t eid, cudaStream_t st,
                      const PushFuse *pf = nullptr);
void push32_steerer(DevBeam &b, double blh, double blv, cudaStream_t st);
void push32_gap_first(DevBeam &b, const GapArgs &g, cudaStream_t st, const PushFuse *pf = nullptr);
void push32_gap_second(DevBeam &b, const GapArgs &g, cudaStream_t st, const PushFuse *pf = nullptr);
void push32_buncher(DevBeam &b, double wl, double w_ref_design, double freq, double voltage, double phase,
                    double aper, double freq_ratio, uint32_t eid, cudaStream_t st);
void push32_rotation(DevBeam &b, double angle, cudaStream_t st);
void push32_aperture(DevBeam &b, int rect, const double *p, uint32_t eid, cudaStream_t st);
void push32_dipole(DevBeam &b, const double *p, double wl, int second, cudaStream_t st,
                   const PushFuse *pf = nullptr);

void beam32_update_avg(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st);
void beam32_update_sig(const DevBeam &b, int coord, int good, PassScratch s, cudaStream_t st);
void beam32_update_emittance(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam32_update_relative_phi(const DevBeam &b, int use_good, cudaStream_t st);
void beam32_update_longitudinal_loss(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam32_update_avg_xy(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam32_update_max_r_phi(const DevBeam &b, PassScratch s, cudaStream_t st);
void beam32_change_frequency(DevBeam &b, double ratio, PassScratch s, cudaStream_t st);
void beam32_apply_cut(const DevBeam &b, int coord, double lo, double hi, cudaStream_t st);
void beam32_shift(const DevBeam &b, int coord, double val, cudaStream_t st);
void beam32_set_ref(DevBeam &b, int coord, double val, cudaStream_t st);
void beam32_monitor(const DevBeam &b, const ScState *sc, double *mon_dev, uint32_t elem, PassScratch s,
                    cudaStream_t st);
void beam32_from_double(const DevBeam &b, const double *const *src, cudaStream_t st);
void beam32_to_double(const DevBeam &b, int coord, double *out, cudaStream_t st);
void beam32_update_stat_for_sc(const DevBeam &b, PassScratch s, cudaStream_t st);

void sc32_configure();
// the tensor-core contraction (contract_tc.cuh): meshes it takes, and the
// bytes of its folded split-BF16 Green's table and of its partial fields
bool sc32_tc_mesh(uint32_t nr, uint32_t nz);
size_t sc32_tc_bytes(uint32_t nr, uint32_t nz, size_t *partial_bytes);
void contract32(const ScState *sc, const ScTables &t, uint32_t nx_max, uint32_t nz_max, bool mesh_fixed,
                cudaStream_t st);
void sc32_stats(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
                cudaStream_t st);
// a fork of a beam's stream: kernels on `side` between ev_fork and ev_join
// run beside the kernels on `main` (a parallel branch of a captured graph)
struct Fork {
  cudaStream_t main, side;
  cudaEvent_t ev_fork, ev_join;
};
// fork (may be null): the Green's table runs beside the deposit
void sc32_mesh(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, PassScratch s,
               cudaStream_t st, const SurNet *sur = nullptr, const Fork *fork = nullptr);
void sc32_kick(const DevBeam &b, ScState *sc, const ScTables &t, const ScKickArgs &a, cudaStream_t st);
// constants of the FP32 kernels of a kick
Sc32Host sc32_host(const DevBeam &b, const ScKickArgs &a);

// ---- headless plot data (plot.cu) -----------------------------------------
// one coordinate of a beam as FP64 values: d[i] (FP64 beams) or
// off + f[i] (FP32 beams: offset from the synchronous particle)
struct PlotCoord {
  const double *d;
  const float *f;
  double off;
};
void plot_points(const PlotCoord &x, const PlotCoord &y, const uint32_t *loss, uint32_t n, float2 *out,
                 cudaStream_t st);
// out (device): xmax, xmin, ymax, ymin; loss == nullptr counts every particle
void plot_maxmin(const PlotCoord &x, const PlotCoord &y, const uint32_t *loss, uint32_t n, PassScratch scr,
                 double *out, cudaStream_t st);
void plot_hist(const PlotCoord &x, const uint32_t *loss, uint32_t n, uint32_t nb, double mn, double mx,
               uint32_t *hist, cudaStream_t st);
// mm: xmax, xmin, ymax, ymin (host)
void plot_hist2d(const PlotCoord &x, const PlotCoord &y, const uint32_t *loss, uint32_t n, const double mm[4],
                 uint32_t nx, uint32_t ny, uint32_t *hist, cudaStream_t st);

}  // namespace hps
