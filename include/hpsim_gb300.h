/*
 * hpsim_gb300.h -- C ABI of the GB300 implementation of HPSim's per-element
 * particle-tracking path.
 *
 * The reference binds its tracking core through a CPython 2 extension
 * (src/pywrapper/src/hpsim_module.cpp:398-419) over an internal C/C++ layer:
 *   - extern "C" engine entry points, src/simulation/inc/simulation_engine_cu.h:4-25
 *   - the SCHEFF launcher API, src/simulation/inc/space_charge_cu.h:6-26
 *   - the Beam device API, src/beam/inc/beam_cu.h:7-40 and the Beam class,
 *     src/beam/inc/beam.h:35-312
 *   - BeamLine / element setters, src/beamline/inc/beamline{,_element}.h
 * Those layers keep their state in file-scope globals (one engine, one SCHEFF
 * solver per process).  This ABI exports the same operations keyed by opaque
 * handles, so several beams and simulators coexist; every call returns an
 * hps_status and hps_last_error() describes the most recent failure on the
 * calling thread.  No call takes or returns a torch type; all arrays are
 * plain host pointers with explicit lengths.
 *
 * Units follow the reference core: m, rad, MeV, MHz, T/m, MV/m, A.
 */
#ifndef HPSIM_GB300_H
#define HPSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#include "hps_layout.h"

#ifdef __cplusplus
extern "C" {
#endif

#define HPS_ABI_VERSION 1

typedef enum hps_status {
  HPS_OK = 0,
  HPS_ERR_INVALID = 1,      /* bad argument or handle */
  HPS_ERR_CUDA = 2,         /* CUDA runtime error (message in hps_last_error) */
  HPS_ERR_NOT_FOUND = 3,    /* element name not in the beamline */
  HPS_ERR_LATTICE = 4,      /* malformed lattice (the reference exits) */
  HPS_ERR_STATE = 5,        /* operation not valid in the current state */
  HPS_ERR_TIMEOUT = 6,      /* a bounded device wait gave up */
  HPS_ERR_NOMEM = 7,
  HPS_ERR_UNSUPPORTED = 8
} hps_status;

/* Particle-state precision of a beam.
 *   HPS_PREC_FP64: every coordinate in FP64, the reference's DOUBLE_PRECISION
 *                  build semantics (SCHEFF bins and fields in FP64).
 *   HPS_PREC_FP32: x, x', y, y' in FP32; phase and energy stored in FP32 as
 *                  offsets from an FP64 synchronous (on-axis) particle tracked
 *                  by the host; SCHEFF tables in FP32; moments summed in FP32
 *                  per thread and warp and combined in FP64 (the SCHEFF
 *                  statistics, which only size the mesh and scale the kick,
 *                  in FP32 throughout). */
typedef enum hps_precision { HPS_PREC_FP64 = 0, HPS_PREC_FP32 = 1 } hps_precision;

typedef struct hps_beam_s *hps_beam_t;
typedef struct hps_beamline_s *hps_beamline_t;
typedef struct hps_scheff_s *hps_scheff_t;
typedef struct hps_sim_s *hps_sim_t;
typedef struct hps_batch_s *hps_batch_t;

/* ---- library ------------------------------------------------------------ */
int hps_abi_version(void);
const char *hps_last_error(void);
const char *hps_status_string(int status);
/* set_gpu(id): src/beamline/src/init.cpp:12-18 */
hps_status hps_set_gpu(int device);
/* count of this library's kernel launches since load (for launch accounting) */
uint64_t hps_kernel_launch_count(void);

/* ---- Beam (src/beam/inc/beam.h:35-312) ---------------------------------- */
/* Beam(num, mass, charge, current): beam.cpp:69-75 + AllocateBeam :124-134.
 * num <= 2^31 (HPS_ERR_INVALID above: the reference's launch geometry, the
 * next power of two of num, and 32-bit particle indices). */
hps_status hps_beam_create(uint32_t num, double mass, double charge, double current,
                           int precision, hps_beam_t *out);
hps_status hps_beam_destroy(hps_beam_t beam);
hps_status hps_beam_info(hps_beam_t beam, uint32_t *num, int *precision);
/* InitBeamFromDistribution, beam.cpp:317-368 (loss/lloss may be NULL) */
hps_status hps_beam_set_distribution(hps_beam_t beam, const double *x, const double *xp,
                                     const double *y, const double *yp, const double *phi,
                                     const double *w, const uint32_t *loss,
                                     const uint32_t *lloss);
/* InitWaterbagBeam, beam.cpp:391-462: twiss = {ax,bx,ex, ay,by,ey, az,bz,ez} */
hps_status hps_beam_set_waterbag(hps_beam_t beam, const double twiss[9], double sync_phi,
                                 double sync_w, double freq, uint32_t seed);
/* InitDCBeam, beam.cpp:481-537: twiss = {ax,bx,ex, ay,by,ey} */
hps_status hps_beam_set_dc(hps_beam_t beam, const double twiss[6], double dphi,
                           double sync_phi, double sync_w, uint32_t seed);
/* CopyBeamFromDevice, beam.cu:227-242.  coord: HPS_COORD_*; FP32 beams are
 * returned as absolute FP64 values. */
hps_status hps_beam_get_coord(hps_beam_t beam, int coord, double *out);
hps_status hps_beam_get_loss(hps_beam_t beam, int longitudinal, uint32_t *out);
/* Save/Restore{Initial,Intermediate}Beam, beam.cpp:573-647: slot 0 = initial,
 * 1 = intermediate.  Snapshots stay on the device. */
hps_status hps_beam_save(hps_beam_t beam, int slot);
hps_status hps_beam_restore(hps_beam_t beam, int slot);
/* SetRefEnergy / SetRefPhase / freq, beam.cpp:1074-1105 */
hps_status hps_beam_set_ref_w(hps_beam_t beam, double w);
hps_status hps_beam_set_ref_phi(hps_beam_t beam, double phi);
hps_status hps_beam_get_ref(hps_beam_t beam, double *w, double *phi);
hps_status hps_beam_set_frequency(hps_beam_t beam, double freq);
/* scalar: 0 mass, 1 charge, 2 current, 3 freq, 4 design_w */
hps_status hps_beam_get_scalar(hps_beam_t beam, int which, double *out);
/* Beam::Update* (beam.cpp:757-1066).  op:
 *   0 UpdateLoss, 1 UpdateLongitudinalLoss, 2 UpdateGoodParticleCount,
 *   3 UpdateAvg(coord, good), 4 UpdateSig(coord, good), 5 UpdateEmittance,
 *   6 UpdateRelativePhi(good), 7 UpdateStatForSpaceCharge, 8 UpdateAvgXY,
 *   9 UpdateMaxRPhi */
hps_status hps_beam_update(hps_beam_t beam, int op, int coord, int good);
/* the per-beam device scalars of beam.h:175-263, HPS_ST_* below */
hps_status hps_beam_get_stat(hps_beam_t beam, int stat, double *out);
/* ApplyCut / Shift*, beam.cpp:1574-1648 */
hps_status hps_beam_apply_cut(hps_beam_t beam, char coord, double lo, double hi);
hps_status hps_beam_translate(hps_beam_t beam, int coord, double value);
/* side-effect-free statistics record (HPS_MON_*) */
hps_status hps_beam_monitor(hps_beam_t beam, double *out /* HPS_NMON */);

/* ---- headless plot data (src/graphics/inc/graphics_kernel.cu, launchers
 * src/graphics/src/graphics_kernel_call.cu) into plain memory instead of GL
 * buffers.  Coordinates are HPS_COORD_* (x, xp, y, yp, phi, w, phi_r).
 * Outputs go to host memory, or, with on_device != 0, to caller-allocated
 * device memory on the current device. */
#define HPS_PLOT_MAX_BINS 12288
/* SetPhaseSpaceData / Set2dPhaseSpaceDataKernel: 2*num floats (x, y) per
 * particle, lost particles at (0, 0) */
hps_status hps_plot_points(hps_beam_t beam, int cx, int cy, float *xy, int on_device);
/* FindMaxMin2D / BlockMaxMin2DKernel: out = xmax, xmin, ymax, ymin; with
 * live_only a lost particle counts as particle 0 (the reference's filler);
 * NaN values are skipped */
hps_status hps_plot_maxmin(hps_beam_t beam, int cx, int cy, int live_only, double out[4]);
/* UpdateHistogram / HistogramKernel + HistogramReduceKernel over live
 * particles, the reference's bin rule (see plot.cu) */
hps_status hps_plot_histogram(hps_beam_t beam, int coord, uint32_t nbins, double min, double max,
                              uint32_t *hist, int on_device);
/* UpdateHistogram2DKernelCall / Histogram2DKernel: nx*ny counts (row iy),
 * maxmin as hps_plot_maxmin returns it */
hps_status hps_plot_histogram2d(hps_beam_t beam, int cx, int cy, uint32_t nx, uint32_t ny,
                                const double maxmin[4], uint32_t *hist, int on_device);

#define HPS_ST_X_AVG 0
#define HPS_ST_X_AVG_GOOD 1
#define HPS_ST_XP_AVG 2
#define HPS_ST_Y_AVG 3
#define HPS_ST_Y_AVG_GOOD 4
#define HPS_ST_YP_AVG 5
#define HPS_ST_PHI_AVG 6
#define HPS_ST_PHI_AVG_R 7
#define HPS_ST_PHI_AVG_GOOD 8
#define HPS_ST_W_AVG 9
#define HPS_ST_W_AVG_GOOD 10
#define HPS_ST_X_SIG 11
#define HPS_ST_X_SIG_GOOD 12
#define HPS_ST_XP_SIG 13
#define HPS_ST_Y_SIG 14
#define HPS_ST_Y_SIG_GOOD 15
#define HPS_ST_YP_SIG 16
#define HPS_ST_PHI_SIG 17
#define HPS_ST_PHI_SIG_R 18
#define HPS_ST_PHI_SIG_GOOD 19
#define HPS_ST_W_SIG 20
#define HPS_ST_W_SIG_GOOD 21
#define HPS_ST_X_EMIT 22
#define HPS_ST_Y_EMIT 23
#define HPS_ST_Z_EMIT 24
#define HPS_ST_R_MAX 25
#define HPS_ST_ABS_PHI_MAX 26
#define HPS_ST_NUM_LOSS 27
#define HPS_ST_NUM_LLOSS 28
#define HPS_ST_NUM_GOOD 29
#define HPS_NST 30

/* ---- BeamLine (src/beamline/inc/beamline.h) ----------------------------- */
hps_status hps_beamline_create(hps_beamline_t *out);
hps_status hps_beamline_destroy(hps_beamline_t bl);
/* BeamLine::AddElement with an element record (include/hps_layout.h) */
hps_status hps_beamline_add(hps_beamline_t bl, int type, const char *name,
                            const double *params /* HPS_NPARAM */);
hps_status hps_beamline_size(hps_beamline_t bl, uint32_t *out);
/* BeamLine::GetElementModelIndex (case-insensitive), beamline.cpp:70-77 */
hps_status hps_beamline_find(hps_beamline_t bl, const char *name, uint32_t *index);
hps_status hps_beamline_get(hps_beamline_t bl, uint32_t index, int *type, char *name,
                            size_t name_cap, double *params /* HPS_NPARAM */);
/* element setters of beamline_element.h (one slot at a time) */
hps_status hps_beamline_set_param(hps_beamline_t bl, uint32_t index, int slot, double value);

/* ---- SCHEFF (src/simulation/inc/space_charge.h) ------------------------- */
/* Scheff(nr, nz, adj_bunch), space_charge.cpp:31-40.  nr and nz must be
 * powers of two, nz <= 512 (the reference's launch geometry requires it).
 * The charge table holds signed 64-bit integers in units of 2^-36 of a
 * particle (exact and order-independent), so one bin holds the charge of
 * fewer than 2^27 particles: beams of fewer than 2^27 (134,217,728)
 * particles cannot overflow it; a larger beam overflows only if 2^27 of
 * its particles fall into one bin. */
hps_status hps_scheff_create(uint32_t nr, uint32_t nz, uint32_t adj_bunch, hps_scheff_t *out);
hps_status hps_scheff_destroy(hps_scheff_t s);
/* parameter: 0 interval, 1 adj_bunch, 2 adj_bunch_cutoff_w, 3 mesh_size_cutoff_w,
 *            4 remesh_threshold, 5 fraction, 6 nr, 7 nz (6/7 read-only);
 * read-only counters since creation: 8 field solves (remeshes), 9 kicks of an
 * FP32 beam whose statistics took the loss-test and moments sweeps (the
 * element map before the kick could not certify them).
 * No reference counterpart: 10 the contraction kernel of FP32 beams (0, the
 * default: split-BF16 tensor cores where the mesh allows -- nz a power of
 * two in 128..512, nr in 16..64 -- else the FP32 ring convolution; 1: the
 * ring convolution always); read-only: 11 the solver holds the tensor-core
 * buffers, 12 a bounded wait of the tensor-core kernel gave up (1).
 * 13 the attached surrogate's layers: 0 on the tensor cores where the
 * layer's shape allows (c_out <= 128, c_in a power of two, w_in even), 1
 * (the default) on CUDA cores -- a solver evaluates the network on one plane,
 * where the CUDA-core layers are slightly faster (the tensor-core ones pay
 * from a batch of about four planes on); read-only: 14 layers of the
 * attached network on the tensor cores, 15 a tensor-core layer's bounded
 * wait gave up (1). */
hps_status hps_scheff_set(hps_scheff_t s, int param, double value);
hps_status hps_scheff_get(hps_scheff_t s, int param, double *value);
/* the solver's tables after its last kick (no reference counterpart): charge
 * (nr*nz), field ((nz+1)*(nr+1) pairs) of the FP32 (fp32 != 0) or FP64 tables,
 * mesh = {nr, nz, dr, dz, beta, num_on_mesh, remesh} */
hps_status hps_scheff_snapshot(hps_scheff_t s, int fp32, double *bins, double *field, double *mesh);
/* SetMeshSize, space_charge.cpp:61-73 */
hps_status hps_scheff_set_mesh_size(hps_scheff_t s, uint32_t nr, uint32_t nz);
/* The SCHEFF table stage on its own: Green's table (UpdateFldTbl1Kernel via
 * UpdateTblsKernelCall, space_charge.cu:148-187) and its contraction with a
 * charge table (UpdateFinalFldTblKernelCall, space_charge.cu:189-218).
 *   bins:  host, nr*nz charges, bin (zs, rs) at zs*nr + rs
 *   mesh:  host, {dr, dz, beta, freq, num_particle, current*fraction/mass, adj_bunch}
 *   field: host, (nz+1)*(nr+1) pairs (E_r, E_z) at zp*(nr+1) + rp
 * Allocates and frees its device buffers on every call. */
hps_status hps_scheff_field(uint32_t nr, uint32_t nz, const double *bins, const double *mesh, double *field);
/* hps_scheff_field for callers that must not allocate device memory while
 * they run (an online model re-solving the field inside a control cycle, a
 * host application whose own memory pool owns the device).  No counterpart
 * in the reference.  bins_dev and field_dev are device pointers supplied by
 * the caller, mesh is the same 7-double host array as above, stream a
 * cudaStream_t (NULL: default stream).  Nothing is allocated: the
 * intermediate tables live in one static device array of the library,
 * about 2.2 MB, kept on every GPU that loads the library until exit.  The
 * first call on a device looks that array's address up, so make the first
 * call before any stream capture.  Limit: nr*nz <= 4096 and
 * (nr+1)*nr*nz <= 135168 (e.g. 32 x 128); larger meshes return
 * HPS_ERR_INVALID.  Calls share the array: calls that overlap on the GPU
 * race.  A CUDA error already pending when the call starts is returned as
 * HPS_ERR_CUDA before any work is issued.  The looked-up address belongs to
 * the device's context: after cudaDeviceReset reload the library before
 * calling this again on that device. */
hps_status hps_scheff_field_noalloc(uint32_t nr, uint32_t nz, const double *bins_dev, const double *mesh,
                                    double *field_dev, void *stream);
/* hps_scheff_field through the kernels FP32 beams use (FP32 Green's table
 * and contraction); same arguments, field returned as doubles.  No
 * counterpart in the reference: it exposes the FP32 solver's table stage so
 * that its error against the FP64 table can be stated. */
hps_status hps_scheff_field_f32(uint32_t nr, uint32_t nz, const double *bins, const double *mesh, double *field);
/* hps_scheff_field_f32 with the contraction kernel chosen: 0 the one FP32
 * beams use for the mesh (the tensor cores where the mesh allows), 1 the
 * FP32 ring convolution on CUDA cores, 2 the split-BF16 tensor-core product
 * (tcgen05; nz a power of two in 128..512, nr in 16..64, else
 * HPS_ERR_UNSUPPORTED).  Same computation as UpdateFinalFldTblKernelCall,
 * src/simulation/src/space_charge.cu:189-218; the kernel choice has no
 * counterpart in the reference. */
hps_status hps_scheff_field_f32_kernel(uint32_t nr, uint32_t nz, const double *bins, const double *mesh,
                                       double *field, int kernel);

/* ---- Simulator (src/simulation/inc/simulation_engine.h) ----------------- */
/* SimulationEngine::InitEngine, simulation_engine.cpp:408-427 (scheff may be NULL) */
hps_status hps_sim_create(hps_beam_t beam, hps_beamline_t bl, hps_scheff_t scheff,
                          hps_sim_t *out);
hps_status hps_sim_destroy(hps_sim_t sim);
/* SimulationEngine::Simulate(start, end), simulation_engine.cpp:447-469:
 * element indices (inclusive); -1 selects the first / the last element. */
hps_status hps_sim_simulate(hps_sim_t sim, int32_t start, int32_t end);
hps_status hps_sim_reset(hps_sim_t sim);
/* SetSpaceCharge("on"/"off"), simulation_engine.h:58-64 */
hps_status hps_sim_set_space_charge(hps_sim_t sim, int on);
/* per-element monitor records: host array of capacity * HPS_NMON doubles,
 * filled for every simulated element (NULL disables). */
hps_status hps_sim_set_monitor(hps_sim_t sim, double *host_out, uint32_t capacity);
/* capture each simulate() range into a CUDA graph and replay it (default on) */
hps_status hps_sim_use_graph(hps_sim_t sim, int on);
/* wait for the simulator's stream */
hps_status hps_sim_synchronize(hps_sim_t sim);
/* device time of the last simulate() in milliseconds (CUDA events) */
hps_status hps_sim_last_time_ms(hps_sim_t sim, double *ms);
/* Per-phase CUDA-event timers (the reference's StartTimer/StopTimer around
 * Simulate, src/util/src/timer.cpp:4-18, broken down by phase).  While on,
 * simulate() issues launches directly (no graph) with an event pair around
 * every phase; hps_sim_profile_read returns the accumulated milliseconds and
 * phase counts per HPS_PROF_* class. */
#define HPS_PROF_DRIFT 0     /* partial drifts */
#define HPS_PROF_QUAD 1      /* half quads */
#define HPS_PROF_GAP1 2      /* RF gap first halves */
#define HPS_PROF_GAP2 3      /* RF gap second halves */
#define HPS_PROF_OTHER 4     /* buncher, steerer, rotation, apertures, dipoles, frequency changes */
#define HPS_PROF_SC_STATS 5  /* SCHEFF statistics sweeps + remesh decision */
#define HPS_PROF_SC_MESH 6   /* Green's table, deposit, contraction */
#define HPS_PROF_SC_KICK 7   /* SCHEFF kick (FP32 beams: kick and the element half after it, one sweep) */
#define HPS_PROF_MONITOR 8   /* per-element monitor records */
/* FP32 beams with a solver: the element half before a kick also takes the
 * first statistics sweep and is timed in its element's class. */
#define HPS_NPROF 9
hps_status hps_sim_profile(hps_sim_t sim, int on);
hps_status hps_sim_profile_read(hps_sim_t sim, double *ms /* HPS_NPROF */, uint64_t *count /* HPS_NPROF */,
                                int reset);

/* ---- batches (no reference counterpart): many independent simulators --
 * (each with its own beam and SpaceCharge; lattices may differ) run their
 * Simulate(start, end) in one graph launch: each simulator's captured range
 * is a child graph of one parent graph with no edges between them, so the
 * beams advance concurrently.  Results are those of running each simulator
 * alone.  Simulators must be able to run as graphs (graphs on, profiling
 * off, no mesh-size cut-off energy). */
hps_status hps_batch_create(const hps_sim_t *sims, uint32_t count, hps_batch_t *out);
hps_status hps_batch_destroy(hps_batch_t batch);
hps_status hps_batch_simulate(hps_batch_t batch, int32_t start, int32_t end);
hps_status hps_batch_last_time_ms(hps_batch_t batch, double *ms);
/* Lockstep form (default off): when every simulator of the batch issues the
 * same sequence of FP32 launches over the range (same element kinds in the
 * same order, same space-charge mesh and contraction kernel; set points,
 * beams and particle counts may differ), each launch runs once for all
 * beams: particle kernels over a grid of every beam's blocks, mesh kernels
 * with a grid dimension over the beams, the per-beam parameters in the
 * kernels' parameter space (up to 64 beams a launch).  Each beam keeps its
 * own block count, so its reductions run in the order they have alone; the
 * merged kernels are separate compilations, so results agree with the
 * child-graph form to FP32 rounding.  It is off by default because the
 * child-graph form is faster on the batch workloads measured (beams at
 * different phases overlap: a mesh kernel of one beam beside a particle
 * sweep of another).  A range with a launch that has no lockstep form
 * (FP64 beams, monitors, the field surrogate, adjacent bunches) runs as
 * child graphs.  hps_batch_last_mode reports which form the last simulate
 * ran in (1: lockstep) and, if not lockstep, why. */
hps_status hps_batch_set_lockstep(hps_batch_t batch, int on);
hps_status hps_batch_last_mode(hps_batch_t batch, int *lockstep, char *why, size_t why_cap);

/* ---- autotuner (no reference counterpart; it replaces the reference's fixed
 * launch geometry, e.g. the 64-block cap of src/beam/src/beam.cu:419 and the
 * contraction grid of src/simulation/src/space_charge.cu:189-200).  A launch
 * shape of an FP32 beam's simulation is shape[5] = {contraction kernel (0
 * split-BF16 tensor cores where the mesh allows, 1 FP32 CUDA cores),
 * deposit blocks per SM (1..8), particle-sweep blocks per SM (0: as many as
 * an SM holds, else a cap 1..16), deposit histogram adds (0 one shared-
 * memory atomic per particle and bin, 1 warp-aggregated: lanes with the
 * same bin sum their weights first), deposit threads per block (256, 512 or
 * 1024; 0 reads as 256)}.  hps_sim_autotune times candidate shapes on the
 * simulator's own simulate(start, end) with CUDA events (coordinate descent
 * over the knobs, the deposit's block size and blocks per SM together; each
 * candidate the median of `reps` runs
 * after an untimed one that captures its graph; every run starts from a
 * snapshot of the beam, solver and engine state, which is restored at the
 * end), keeps the fastest and caches it per (device, mesh, power-of-two
 * particle-count bucket, precision): a later call with the same key applies
 * the cached shape without timing (n_timed = 0).  shape_out receives the
 * chosen shape, ms_out up to ms_cap candidate times (ms), n_timed their
 * count.  FP64 beams have nothing to tune (the shape is returned as is).
 * hps_batch_autotune does the same for a batch (objective: the batch's
 * launch; the shape is applied to every simulator).  Tuning must not run
 * during a stream capture. */
hps_status hps_sim_autotune(hps_sim_t sim, int32_t start, int32_t end, int32_t reps, int32_t *shape_out,
                            double *ms_out, uint32_t ms_cap, uint32_t *n_timed);
hps_status hps_batch_autotune(hps_batch_t batch, int32_t start, int32_t end, int32_t reps, int32_t *shape_out,
                              double *ms_out, uint32_t ms_cap, uint32_t *n_timed);
hps_status hps_sim_get_shape(hps_sim_t sim, int32_t *shape_out /* 5 */);
hps_status hps_sim_set_shape(hps_sim_t sim, const int32_t *shape /* 5 */);

/* ---- SCHEFF field surrogate: network layers (no reference counterpart).
 * Device pointers; tensors [batch][channel][z][r]; x, w, y BF16, bias, dy,
 * dz, dx, dw, db FP32.  dims = {batch, c_in, c_out, h_in, w_in, stride (1|2),
 * up (1|2: nearest 2x upsampling of the input before the 3x3 convolution)};
 * output h = (h_in*up - 1)/stride + 1; c_in <= 512.  stream: a cudaStream_t
 * or NULL.  y = ReLU(conv + bias) (relu != 0) rounded to BF16, plus skip
 * (same shape as y, BF16, rounded again) when skip != NULL. */
hps_status hps_nn_conv_forward(const int32_t dims[7], const void *x, const void *w, const float *bias, int relu,
                               const void *skip, void *y, void *stream);
/* The same layer on the tensor cores (tcgen05 BF16 MMA, FP32 accumulation;
 * the inference kernel of a network attached to a solver): c_out <= 128,
 * c_in a power of two, w_in even.  This entry point lays the weights out as
 * the kernel's tiles in a temporary buffer, runs the layer and waits for it
 * (a test and measurement entry; attached networks keep their tiles).
 * HPS_ERR_INVALID for a shape the kernel does not take. */
hps_status hps_nn_conv_forward_tc(const int32_t dims[7], const void *x, const void *w, const float *bias, int relu,
                                  const void *skip, void *y, void *stream);
/* The tensor-core layer with caller-kept weight tiles: the tiles' bytes for
 * the layer (0: shape not taken), their layout from BF16 weights w (again
 * after the weights change), and the layer (asynchronous on stream; *err, a
 * device word, is set when a pipeline wait gave up). */
hps_status hps_nn_conv_tc_tile_bytes(const int32_t dims[7], uint64_t *bytes);
hps_status hps_nn_conv_tc_prepare(const int32_t dims[7], const void *w, void *tiles, void *stream);
hps_status hps_nn_conv_forward_tiles(const int32_t dims[7], const void *x, const void *tiles, const float *bias,
                                     int relu, const void *skip, void *y, unsigned int *err, void *stream);
/* dz = dy masked by the ReLU of y; dw, db = weight and bias gradients; dx
 * (may be NULL) = input gradient */
hps_status hps_nn_conv_backward(const int32_t dims[7], const void *x, const void *w, const void *y, int relu,
                                const float *dy, float *dz, float *dx, float *dw, float *db, void *stream);
/* y[b][c] += mean of the plane (BF16, in place) and its backward on FP32 */
hps_status hps_nn_gmean_forward(void *y, int32_t planes, int32_t hw, void *stream);
hps_status hps_nn_gmean_backward(float *d, int32_t planes, int32_t hw, void *stream);
/* squared error: per-block partial sums of wt (pred - target)^2 and dpred =
 * 2 wt (pred - target) / n, wt = weight[i / per_sample] (weight may be NULL) */
hps_status hps_nn_mse(const void *pred, const float *target, int64_t n, const float *weight, int64_t per_sample,
                      float *dpred, float *partial, int32_t nblocks, void *stream);
/* y = a + b (bf16 != 0: BF16 tensors, else FP32) */
hps_status hps_nn_add(const void *a, const void *b, void *y, int64_t n, int bf16, void *stream);
/* Adam on FP32 weights (step >= 1), refreshing their BF16 copy when w_bf16 != NULL */
hps_status hps_nn_adam(float *w, void *w_bf16, const float *g, float *m, float *v, int64_t n, float lr, float b1,
                       float b2, float eps, int32_t step, void *stream);
/* FP32 <-> BF16 (to_bf16: 1 FP32 -> BF16, 0 BF16 -> FP32) */
hps_status hps_nn_convert(const void *src, void *dst, int64_t n, int to_bf16, void *stream);

/* Attach a trained field network to a solver (FP64 and FP32 beams; the
 * network's field goes into the table of the beam's precision).  No
 * counterpart in the reference: it stands in for UpdateTblsKernelCall +
 * UpdateFinalFldTblKernelCall inside Scheff::Start,
 * src/simulation/src/space_charge.cpp:130-133.  Host arrays: arch[5*l..] = {c_in, c_out, stride, up,
 * relu} per layer (first c_in = 2, last c_out = 2, output on nz x nr);
 * gmean_after = the layer whose output gets its plane mean added (-1 none);
 * skip[l] = the earlier layer whose output layer l adds (-1 none);
 * weights[l] = BF16 bits [c_out][c_in][3][3], biases[l] = FP32 [c_out].
 * Input channels: charge * nr*nz / total and log(dz*gamma/dr); the field is
 * output * c1 * total / (out_scale * dr * dz*gamma).  Each kick that
 * remeshes on an nr x nz mesh without adjacent bunches evaluates it, solves
 * the plain sum (Green's function in FP32) at the last row and column and at
 * n_samples interior points, and keeps the network's field when its
 * relative residual there is <= tol; else the Green's table and the plain
 * contraction of the beam's precision run.  Replaces an attached network. */
hps_status hps_scheff_set_surrogate(hps_scheff_t s, int32_t n_layers, const int32_t *arch, int32_t gmean_after,
                                    const int32_t *skip, const uint16_t *const *weights, const float *const *biases,
                                    uint32_t nr, uint32_t nz, double out_scale, double tol, uint32_t n_samples);
hps_status hps_scheff_clear_surrogate(hps_scheff_t s);
/* kicks whose field was accepted / fell back, and the last residual */
hps_status hps_scheff_surrogate_stats(hps_scheff_t s, double *accepted, double *rejected, double *residual);

#ifdef __cplusplus
}
#endif
#endif
