// runtime.cu -- host runtime and C ABI (include/hpsim_gb300.h).
//
// Host objects mirror the reference's classes: Beam (src/beam/src/beam.cpp),
// BeamLine (src/beamline/src/beamline.cpp), Scheff (src/simulation/src/
// space_charge.cpp) and SimulationEngine (src/simulation/src/
// simulation_engine.{cpp,cu}).  All particle work is issued on the beam's
// CUDA stream; a simulate() call issues a fixed launch sequence (the
// space-charge decisions live on the device), which is captured once into a
// CUDA graph and replayed while the lattice and the engine's host state are
// unchanged.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hpsim_gb300.h"
#include "internal.h"
#include "lockstep.cuh"

namespace hps {

static std::atomic<uint64_t> g_launches{0};
static thread_local Recorder *g_recorder = nullptr;
Recorder *&recorder() { return g_recorder; }
// launches handed to a lockstep recorder are counted when the merged graph runs
void note_launch(int n) {
  if (!g_recorder) g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed);
}

static thread_local std::string g_err;

static hps_status fail(hps_status s, const std::string &msg) {
  g_err = msg;
  return s;
}
int set_error(int status, const char *msg) { return (int)fail((hps_status)status, msg); }

#define CK(call)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(HPS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static hps_status last_launch_status(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(HPS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return HPS_OK;
}

}  // namespace hps

using namespace hps;

// ---------------------------------------------------------------------------
// objects
// ---------------------------------------------------------------------------
struct hps_beam_s {
  uint32_t n = 0;
  int dev = -1;  // the device its memory lives on
  int prec = HPS_PREC_FP64;
  double mass = 0, charge = 0, current = 0, freq = 0, design_w = 0;
  uint32_t grid_size = 1, blck_size = 1;
  cudaStream_t stream = nullptr;
  // a second stream and two events: kernels that do not depend on each
  // other run side by side (a fork and a join in a captured graph)
  Fork fork{};
  DevBeam d{};
  PassScratch scr{};
  // device snapshots for Save/Restore (slot 0 initial, 1 intermediate)
  void *save[2][6] = {};
  uint32_t *save_loss[2] = {}, *save_lloss[2] = {};
  double save_design_w[2] = {}, save_freq[2] = {}, save_current[2] = {};
  double save_phi_ref[2] = {}, save_w_ref[2] = {};
  bool saved[2] = {false, false};
  // FP32 beams: 6 x n doubles on the device for host <-> device conversion
  double *stage = nullptr;
};

struct hps_beamline_s {
  std::vector<int> types;
  std::vector<std::string> names;
  std::vector<std::vector<double>> params;
  uint64_t version = 0;
};

struct hps_scheff_s {
  int dev = -1;  // the device its memory lives on
  // host mirror of SpaceCharge's members (space_charge.h:88-125)
  uint32_t nx, nz, nx_init, nz_init, adj_bunch;
  double fraction = 1.0, interval = 0.01, interval_init = 0.01, adj_bunch_w = 0.0, mesh_w = 0.0,
         remesh_val = 0.05;
  uint32_t nx_max, nz_max;
  ScState *d = nullptr;
  ScTables t{};
  uint64_t version = 0;
  SurNet *sur = nullptr;  // field surrogate, owned
  int sur_kernel = 1;     // its layers: 0 tensor cores where the layer allows, 1 CUDA cores (faster at batch 1)
  int contraction = 0;    // FP32 beams: 0 tensor cores where the mesh allows, 1 CUDA cores
};

// The host-side state of a simulator that a range advances (engine, beam
// and solver fields; phi_ref and w_ref are an FP32 beam's synchronous
// particle): a captured range stores it as it is at the range's end, and a
// lockstep recording saves and puts it back.
struct HostState {
  double design_w, wavelen, beam_freq, beam_current, beam_design_w, phi_ref, w_ref, fraction, interval;
  uint32_t ccl_cell_num, cur_id;
};

struct GraphEntry {
  uint64_t key = 0;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;  // the captured graph, kept for batches
  uint64_t serial = 0;          // bumped at every capture
  HostState after{};            // host state after the range
  uint64_t nkernels = 0;        // kernels in the captured graph
};

struct hps_sim_s {
  hps_beam_t beam = nullptr;
  hps_beamline_t bl = nullptr;
  hps_scheff_t sc = nullptr;
  bool sc_on = false;
  // engine globals of simulation_engine.cu:19-33
  uint32_t cur_id = 0, ccl_cell_num = 0;
  double design_w = 0, wavelen = 0;
  int prev_end = -1;
  // monitor
  double *mon_host = nullptr;
  uint32_t mon_cap = 0;
  double *mon_dev = nullptr;
  uint32_t mon_dev_cap = 0;
  bool use_graph = true;
  GraphEntry graph;
  // per-phase timers
  bool prof_on = false;
  std::vector<cudaEvent_t> prof_pool;
  std::vector<int> prof_cls;  // class of event pair k (events 2k, 2k+1)
  size_t prof_used = 0;
  double prof_ms[HPS_NPROF] = {};
  uint64_t prof_cnt[HPS_NPROF] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  // launch shapes of the FP32 kernels (hps_sim_autotune picks them)
  uint32_t sweep_cap = 0;   // particle sweeps: blocks per SM (0: all the SM holds)
  uint32_t dep_per_sm = 3;  // deposit: blocks per SM
  uint32_t dep_agg = 0;     // deposit: warp-aggregated histogram adds
  uint32_t dep_threads = 256;  // deposit: threads per block
};

// Many simulators run as one graph launch: each simulator's captured range
// is a child graph of one parent graph, with no edges between them.

struct hps_batch_s {
  std::vector<hps_sim_t> sims;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> serials;  // the child captures the parent was built from
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  // lockstep form (lockstep.cuh): one launch per kernel for every beam
  bool lockstep = false;
  int last_mode = 0;                 // 1: the last range ran in lockstep
  std::string ls_why;                // why it did not
  cudaStream_t side = nullptr;       // the Green's-table branch
  cudaGraphExec_t ls_exec = nullptr;
  uint64_t ls_key = 0, ls_nodes = 0;
  std::vector<HostState> ls_after;   // every simulator's host state after the range
  SegFork segfork;              // the side-stream fork and join events of merged launches
};

// ---------------------------------------------------------------------------
// beam helpers
// ---------------------------------------------------------------------------
namespace {

bool valid(hps_beam_t b) { return b != nullptr && b->d.loss != nullptr; }
// An object's kernels and copies run on the calling thread's current
// device, which must be the one its memory was allocated on (set_gpu
// selects it): a call from another device is refused.
hps_status device_check(int dev, const char *what) {
  int cur = -1;
  const cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return fail(HPS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  if (dev >= 0 && cur != dev)
    return fail(HPS_ERR_STATE, std::string(what) + ": the object lives on device " + std::to_string(dev) +
                                   ", the current device is " + std::to_string(cur) + " (call set_gpu first)");
  return HPS_OK;
}
#define ON_DEVICE(obj, what)                          \
  do {                                                \
    const hps_status dev_e_ = device_check((obj)->dev, what); \
    if (dev_e_) return dev_e_;                        \
  } while (0)
bool f32(hps_beam_t b) { return b->prec == HPS_PREC_FP32; }
size_t esize(hps_beam_t b) { return f32(b) ? sizeof(float) : sizeof(double); }
// the six coordinate arrays of the beam's own precision
void *coord_ptr(hps_beam_t b, int k) {
  const DevBeam &d = b->d;
  if (f32(b)) {
    float *p[] = {d.fx, d.fxp, d.fy, d.fyp, d.fphi, d.fw, d.fphi_r};
    return p[k];
  }
  double *p[] = {d.x, d.xp, d.y, d.yp, d.phi, d.w, d.phi_r};
  return p[k];
}

hps_status sync(hps_beam_t b) {
  CK(cudaStreamSynchronize(b->stream));
  return HPS_OK;
}

template <typename T>
hps_status dmalloc(T **p, size_t n) {
  CK(cudaMalloc((void **)p, (n ? n : 1) * sizeof(T)));
  CK(cudaMemset(*p, 0, (n ? n : 1) * sizeof(T)));
  return HPS_OK;
}

hps_status stage_alloc(hps_beam_t b) {
  if (b->stage) return HPS_OK;
  return dmalloc(&b->stage, (size_t)b->n * 6);
}

hps_status upload(hps_beam_t b, const double *x, const double *xp, const double *y, const double *yp,
                  const double *phi, const double *w, const uint32_t *loss, const uint32_t *lloss) {
  size_t nd = (size_t)b->n * sizeof(double), nu = (size_t)b->n * sizeof(uint32_t);
  cudaStream_t s = b->stream;
  const double *src[6] = {x, xp, y, yp, phi, w};
  if (f32(b)) {
    // FP64 host arrays -> staging -> FP32 offsets from particle 0's phase
    // and energy (the reference particle)
    hps_status e = stage_alloc(b);
    if (e) return e;
    const double *dst[6];
    for (int k = 0; k < 6; ++k) {
      dst[k] = b->stage + (size_t)k * b->n;
      CK(cudaMemcpyAsync((void *)dst[k], src[k], nd, cudaMemcpyHostToDevice, s));
    }
    b->d.phi_ref = b->n ? phi[0] : 0.0;
    b->d.w_ref = b->n ? w[0] : 0.0;
    beam32_from_double(b->d, dst, s);
  } else {
    for (int k = 0; k < 6; ++k) CK(cudaMemcpyAsync(coord_ptr(b, k), src[k], nd, cudaMemcpyHostToDevice, s));
  }
  if (loss) CK(cudaMemcpyAsync(b->d.loss, loss, nu, cudaMemcpyHostToDevice, s));
  else CK(cudaMemsetAsync(b->d.loss, 0, nu, s));
  if (lloss) CK(cudaMemcpyAsync(b->d.lloss, lloss, nu, cudaMemcpyHostToDevice, s));
  else CK(cudaMemsetAsync(b->d.lloss, 0, nu, s));
  return HPS_OK;
}

// Beam::InitPhiAvgGood, beam.cpp:655-661: UpdateLoss, UpdateAvgPhi(), copy
// to phi_avg_good
__global__ void k_copy_phi_avg(DevBeam b) { b.st->st[PHI_AVG_GOOD] = b.st->st[PHI_AVG]; }

hps_status init_phi_avg_good(hps_beam_t b) {
  beam_update_loss(b->d, b->scr, b->stream);
  if (f32(b)) beam32_update_avg(b->d, HPS_COORD_PHI, 0, b->scr, b->stream);
  else beam_update_avg(b->d, HPS_COORD_PHI, 0, b->scr, b->stream);
  k_copy_phi_avg<<<1, 1, 0, b->stream>>>(b->d);
  note_launch();
  return last_launch_status("init_phi_avg_good");
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int hps_abi_version(void) { return HPS_ABI_VERSION; }
const char *hps_last_error(void) { return g_err.c_str(); }
const char *hps_status_string(int s) {
  switch (s) {
    case HPS_OK: return "ok";
    case HPS_ERR_INVALID: return "invalid argument";
    case HPS_ERR_CUDA: return "CUDA error";
    case HPS_ERR_NOT_FOUND: return "element not found";
    case HPS_ERR_LATTICE: return "malformed lattice";
    case HPS_ERR_STATE: return "invalid state";
    case HPS_ERR_TIMEOUT: return "device wait timed out";
    case HPS_ERR_NOMEM: return "out of memory";
    case HPS_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}
uint64_t hps_kernel_launch_count(void) { return g_launches.load(); }

hps_status hps_set_gpu(int device) {
  CK(cudaSetDevice(device));
  return HPS_OK;
}

// ---- Beam -----------------------------------------------------------------
hps_status hps_beam_create(uint32_t num, double mass, double charge, double current, int precision,
                           hps_beam_t *out) {
  if (!out) return fail(HPS_ERR_INVALID, "hps_beam_create: null output");
  *out = nullptr;
  if (precision != HPS_PREC_FP64 && precision != HPS_PREC_FP32)
    return fail(HPS_ERR_UNSUPPORTED, "hps_beam_create: unknown precision");
  // the reference's launch geometry (next power of two of the count,
  // beam.cpp:148-168) and the 32-bit particle indices of the sweeps hold
  // up to 2^31 particles
  if (num > kMaxParticles) return fail(HPS_ERR_INVALID, "hps_beam_create: a beam holds at most 2^31 particles");
  hps_beam_t b = new hps_beam_s();
  b->n = num; b->mass = mass; b->charge = charge; b->current = current; b->prec = precision;
  cudaGetDevice(&b->dev);
  ref_launch(num, &b->grid_size, &b->blck_size);
  hps_status s = HPS_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete b; return fail(HPS_ERR_CUDA, cudaGetErrorString(e)); }
  b->fork.main = b->stream;
  if ((e = cudaStreamCreateWithFlags(&b->fork.side, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&b->fork.ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&b->fork.ev_join, cudaEventDisableTiming)) != cudaSuccess) {
    hps_beam_destroy(b);
    return fail(HPS_ERR_CUDA, cudaGetErrorString(e));
  }
  DevBeam &d = b->d;
  d.n = num; d.mass = mass; d.charge = charge;
  if (precision == HPS_PREC_FP64) {
    if ((s = dmalloc(&d.x, num)) || (s = dmalloc(&d.xp, num)) || (s = dmalloc(&d.y, num)) ||
        (s = dmalloc(&d.yp, num)) || (s = dmalloc(&d.phi, num)) || (s = dmalloc(&d.phi_r, num)) ||
        (s = dmalloc(&d.w, num))) {}
  } else {
    if ((s = dmalloc(&d.fx, num)) || (s = dmalloc(&d.fxp, num)) || (s = dmalloc(&d.fy, num)) ||
        (s = dmalloc(&d.fyp, num)) || (s = dmalloc(&d.fphi, num)) || (s = dmalloc(&d.fphi_r, num)) ||
        (s = dmalloc(&d.fw, num))) {}
  }
  if (s || (s = dmalloc(&d.loss, num)) || (s = dmalloc(&d.lloss, num)) || (s = dmalloc(&d.st, 1)) ||
      (s = dmalloc(&b->scr.part, (size_t)kMaxPassBlocks * 32)) || (s = dmalloc(&b->scr.counter, 1))) {
    hps_beam_destroy(b);
    return s;
  }
  *out = b;
  return HPS_OK;
}

hps_status hps_beam_destroy(hps_beam_t b) {
  if (!b) return HPS_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  DevBeam &d = b->d;
  void *ptrs[] = {d.x,   d.xp,  d.y,   d.yp,     d.phi,  d.phi_r, d.w,    d.fx,          d.fxp,
                  d.fy,  d.fyp, d.fphi, d.fphi_r, d.fw,   d.loss,  d.lloss, d.st, b->scr.part,
                  b->scr.counter, b->stage};
  for (void *p : ptrs) if (p) cudaFree(p);
  for (int s = 0; s < 2; ++s) {
    for (int k = 0; k < 6; ++k) if (b->save[s][k]) cudaFree(b->save[s][k]);
    if (b->save_loss[s]) cudaFree(b->save_loss[s]);
    if (b->save_lloss[s]) cudaFree(b->save_lloss[s]);
  }
  if (b->fork.side) { cudaStreamSynchronize(b->fork.side); cudaStreamDestroy(b->fork.side); }
  if (b->fork.ev_fork) cudaEventDestroy(b->fork.ev_fork);
  if (b->fork.ev_join) cudaEventDestroy(b->fork.ev_join);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return HPS_OK;
}

hps_status hps_beam_info(hps_beam_t b, uint32_t *num, int *precision) {
  if (!valid(b)) return fail(HPS_ERR_INVALID, "bad beam handle");
  if (num) *num = b->n;
  if (precision) *precision = b->prec;
  return HPS_OK;
}

hps_status hps_beam_set_distribution(hps_beam_t b, const double *x, const double *xp, const double *y,
                                     const double *yp, const double *phi, const double *w,
                                     const uint32_t *loss, const uint32_t *lloss) {
  if (!valid(b) || !x || !xp || !y || !yp || !phi || !w) return fail(HPS_ERR_INVALID, "set_distribution: null array");
  ON_DEVICE(b, __func__);
  hps_status s = upload(b, x, xp, y, yp, phi, w, loss, lloss);
  if (s) return s;
  // the reference particle sits on axis (beam.cpp:344-358)
  if (b->n) {
    uint32_t u = 0;
    for (int k = 0; k < 4; ++k) CK(cudaMemsetAsync(coord_ptr(b, k), 0, esize(b), b->stream));
    if (loss) CK(cudaMemcpyAsync(b->d.loss, &u, 4, cudaMemcpyHostToDevice, b->stream));
    if (lloss) CK(cudaMemcpyAsync(b->d.lloss, &u, 4, cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));  // the scalars above live on this stack frame
  }
  s = init_phi_avg_good(b);
  if (s) return s;
  return sync(b);
}

// Beam::InitWaterbagBeam, beam.cpp:391-462 (host generation with the C
// library's rand(), identical sequence to the reference on glibc)
hps_status hps_beam_set_waterbag(hps_beam_t b, const double t[9], double r_sync_phi, double r_sync_w,
                                 double r_freq, uint32_t r_seed) {
  if (!valid(b) || !t) return fail(HPS_ERR_INVALID, "set_waterbag: bad argument");
  ON_DEVICE(b, __func__);
  uint32_t n = b->n;
  std::vector<double> xh(n), xph(n), yh(n), yph(n), phih(n), wh(n);
  if (r_seed == 0) std::srand((unsigned)std::time(nullptr));
  else std::srand(r_seed);
  double rsq = 1.0;
  double gx = (1.0 + t[0] * t[0]) / t[1];
  double xmx = std::sqrt(t[2] / gx), xpmx = std::sqrt(t[2] * gx), dx = -t[0] / gx;
  double gy = (1.0 + t[3] * t[3]) / t[4];
  double ymx = std::sqrt(t[5] / gy), ypmx = std::sqrt(t[5] * gy), dy = -t[3] / gy;
  double gz = (1.0 + t[6] * t[6]) / t[7];
  double zmx = std::sqrt(t[8] / gz), zpmx = t[8] / zmx, dz = -t[6] / gz;
  double wave_len = 29979.2458 / r_freq;
  b->freq = r_freq;
  double gm = r_sync_w / b->mass + 1.0;
  double beta = std::sqrt(1.0 - 1.0 / (gm * gm));
  for (uint32_t i = 0; i < n; ++i) {
    double r1, r2, r3, r4, r5, r6;
    do {
      do { r1 = 2.0 * std::rand() / RAND_MAX - 1.0; r2 = 2.0 * std::rand() / RAND_MAX - 1.0; }
      while (r1 * r1 + r2 * r2 > 1.0);
      do { r3 = 2.0 * std::rand() / RAND_MAX - 1.0; r4 = 2.0 * std::rand() / RAND_MAX - 1.0; }
      while (r3 * r3 + r4 * r4 > 1.0);
      do { r5 = 2.0 * std::rand() / RAND_MAX - 1.0; r6 = 2.0 * std::rand() / RAND_MAX - 1.0; }
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
  hps_status s = upload(b, xh.data(), xph.data(), yh.data(), yph.data(), phih.data(), wh.data(), nullptr, nullptr);
  if (s) return s;
  s = init_phi_avg_good(b);
  if (s) return s;
  return sync(b);
}

// Beam::InitDCBeam, beam.cpp:481-537
hps_status hps_beam_set_dc(hps_beam_t b, const double t[6], double r_dphi, double r_sync_phi,
                           double r_sync_w, uint32_t r_seed) {
  if (!valid(b) || !t) return fail(HPS_ERR_INVALID, "set_dc: bad argument");
  ON_DEVICE(b, __func__);
  uint32_t n = b->n;
  std::vector<double> xh(n), xph(n), yh(n), yph(n), phih(n), wh(n);
  if (r_seed == 0) std::srand((unsigned)std::time(nullptr));
  else std::srand(r_seed);
  double rsq = 1.0;
  double gx = (1.0 + t[0] * t[0]) / t[1];
  double xmx = std::sqrt(t[2] / gx), xpmx = std::sqrt(t[2] * gx), dx = -t[0] / gx;
  double gy = (1.0 + t[3] * t[3]) / t[4];
  double ymx = std::sqrt(t[5] / gy), ypmx = std::sqrt(t[5] * gy), dy = -t[3] / gy;
  for (uint32_t i = 0; i < n; ++i) {
    double r1, r2, r3, r4, r5;
    do {
      do { r1 = 2.0 * std::rand() / RAND_MAX - 1.0; r2 = 2.0 * std::rand() / RAND_MAX - 1.0; }
      while (r1 * r1 + r2 * r2 > 1.0);
      do { r3 = 2.0 * std::rand() / RAND_MAX - 1.0; r4 = 2.0 * std::rand() / RAND_MAX - 1.0; }
      while (r3 * r3 + r4 * r4 > 1.0);
    } while (r1 * r1 + r2 * r2 + r3 * r3 + r4 * r4 > 1.0);
    r1 *= rsq; r2 *= rsq; r3 *= rsq; r4 *= rsq;
    r5 = 2.0 * (double)(i + 1.0) / (double)n - 1.0;
    xh[i] = 0.01 * (r1 * xmx + dx * r2 * xpmx);
    xph[i] = r2 * xpmx;
    yh[i] = 0.01 * (r3 * ymx + dy * r4 * ypmx);
    yph[i] = r4 * ypmx;
    phih[i] = r5 * r_dphi + r_sync_phi;
    wh[i] = r_sync_w;
  }
  if (n) { xh[0] = 0.0; xph[0] = 0.0; yh[0] = 0.0; yph[0] = 0.0; }
  hps_status s = upload(b, xh.data(), xph.data(), yh.data(), yph.data(), phih.data(), wh.data(), nullptr, nullptr);
  if (s) return s;
  s = init_phi_avg_good(b);
  if (s) return s;
  return sync(b);
}

hps_status hps_beam_get_coord(hps_beam_t b, int coord, double *out) {
  if (!valid(b) || !out || coord < 0 || coord > HPS_COORD_PHI_R) return fail(HPS_ERR_INVALID, "get_coord: bad argument");
  ON_DEVICE(b, __func__);
  if (f32(b)) {
    hps_status e = stage_alloc(b);
    if (e) return e;
    beam32_to_double(b->d, coord, b->stage, b->stream);
    CK(cudaMemcpyAsync(out, b->stage, (size_t)b->n * 8, cudaMemcpyDeviceToHost, b->stream));
  } else {
    CK(cudaMemcpyAsync(out, coord_ptr(b, coord), (size_t)b->n * 8, cudaMemcpyDeviceToHost, b->stream));
  }
  return sync(b);
}

hps_status hps_beam_get_loss(hps_beam_t b, int longitudinal, uint32_t *out) {
  if (!valid(b) || !out) return fail(HPS_ERR_INVALID, "get_loss: bad argument");
  ON_DEVICE(b, __func__);
  CK(cudaMemcpyAsync(out, longitudinal ? b->d.lloss : b->d.loss, (size_t)b->n * 4, cudaMemcpyDeviceToHost,
                     b->stream));
  return sync(b);
}

hps_status hps_beam_save(hps_beam_t b, int slot) {
  if (!valid(b) || slot < 0 || slot > 1) return fail(HPS_ERR_INVALID, "save: bad argument");
  ON_DEVICE(b, __func__);
  size_t nd = (size_t)b->n * esize(b), nu = (size_t)b->n * 4;
  hps_status s;
  for (int k = 0; k < 6; ++k) {
    if (!b->save[slot][k]) {
      unsigned char *p = nullptr;
      if ((s = dmalloc(&p, nd))) return s;
      b->save[slot][k] = p;
    }
    CK(cudaMemcpyAsync(b->save[slot][k], coord_ptr(b, k), nd, cudaMemcpyDeviceToDevice, b->stream));
  }
  b->save_phi_ref[slot] = b->d.phi_ref;
  b->save_w_ref[slot] = b->d.w_ref;
  if (!b->save_loss[slot] && (s = dmalloc(&b->save_loss[slot], b->n))) return s;
  if (!b->save_lloss[slot] && (s = dmalloc(&b->save_lloss[slot], b->n))) return s;
  CK(cudaMemcpyAsync(b->save_loss[slot], b->d.loss, nu, cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaMemcpyAsync(b->save_lloss[slot], b->d.lloss, nu, cudaMemcpyDeviceToDevice, b->stream));
  b->save_design_w[slot] = b->design_w;
  b->save_freq[slot] = b->freq;
  b->save_current[slot] = b->current;
  b->saved[slot] = true;
  return sync(b);
}

// Beam::Restore*Beam, beam.cpp:606-647: then UpdateAvgPhi(true) and
// UpdateRelativePhi(true)
hps_status hps_beam_restore(hps_beam_t b, int slot) {
  if (!valid(b) || slot < 0 || slot > 1) return fail(HPS_ERR_INVALID, "restore: bad argument");
  ON_DEVICE(b, __func__);
  if (!b->saved[slot]) return fail(HPS_ERR_STATE, "restore: no beam has been saved in this slot");
  size_t nd = (size_t)b->n * esize(b), nu = (size_t)b->n * 4;
  for (int k = 0; k < 6; ++k)
    CK(cudaMemcpyAsync(coord_ptr(b, k), b->save[slot][k], nd, cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaMemcpyAsync(b->d.loss, b->save_loss[slot], nu, cudaMemcpyDeviceToDevice, b->stream));
  CK(cudaMemcpyAsync(b->d.lloss, b->save_lloss[slot], nu, cudaMemcpyDeviceToDevice, b->stream));
  b->design_w = b->save_design_w[slot];
  b->freq = b->save_freq[slot];
  b->current = b->save_current[slot];
  b->d.phi_ref = b->save_phi_ref[slot];
  b->d.w_ref = b->save_w_ref[slot];
  if (f32(b)) {
    beam32_update_avg(b->d, HPS_COORD_PHI, 1, b->scr, b->stream);
    beam32_update_relative_phi(b->d, 1, b->stream);
  } else {
    beam_update_avg(b->d, HPS_COORD_PHI, 1, b->scr, b->stream);
    beam_update_relative_phi(b->d, 1, b->stream);
  }
  hps_status s = last_launch_status("restore");
  if (s) return s;
  return sync(b);
}

hps_status hps_beam_set_ref_w(hps_beam_t b, double w) {
  if (!valid(b)) return fail(HPS_ERR_INVALID, "bad beam handle");
  ON_DEVICE(b, __func__);
  if (f32(b)) beam32_set_ref(b->d, HPS_COORD_W, w, b->stream);
  else beam_set_ref(b->d, HPS_COORD_W, w, b->stream);
  b->design_w = w;
  return sync(b);
}
hps_status hps_beam_set_ref_phi(hps_beam_t b, double phi) {
  if (!valid(b)) return fail(HPS_ERR_INVALID, "bad beam handle");
  ON_DEVICE(b, __func__);
  if (f32(b)) beam32_set_ref(b->d, HPS_COORD_PHI, phi, b->stream);
  else beam_set_ref(b->d, HPS_COORD_PHI, phi, b->stream);
  return sync(b);
}
hps_status hps_beam_get_ref(hps_beam_t b, double *w, double *phi) {
  if (!valid(b) || b->n == 0) return fail(HPS_ERR_INVALID, "bad beam handle");
  ON_DEVICE(b, __func__);
  if (f32(b)) {
    float fw = 0.f, fp = 0.f;
    CK(cudaMemcpyAsync(&fw, b->d.fw, 4, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaMemcpyAsync(&fp, b->d.fphi, 4, cudaMemcpyDeviceToHost, b->stream));
    hps_status s = sync(b);
    if (s) return s;
    if (w) *w = b->d.w_ref + (double)fw;
    if (phi) *phi = b->d.phi_ref + (double)fp;
    return HPS_OK;
  }
  if (w) CK(cudaMemcpyAsync(w, b->d.w, 8, cudaMemcpyDeviceToHost, b->stream));
  if (phi) CK(cudaMemcpyAsync(phi, b->d.phi, 8, cudaMemcpyDeviceToHost, b->stream));
  return sync(b);
}
hps_status hps_beam_set_frequency(hps_beam_t b, double f) {
  if (!valid(b)) return fail(HPS_ERR_INVALID, "bad beam handle");
  b->freq = f;
  return HPS_OK;
}
hps_status hps_beam_get_scalar(hps_beam_t b, int which, double *out) {
  if (!valid(b) || !out) return fail(HPS_ERR_INVALID, "bad argument");
  switch (which) {
    case 0: *out = b->mass; break;
    case 1: *out = b->charge; break;
    case 2: *out = b->current; break;
    case 3: *out = b->freq; break;
    case 4: *out = b->design_w; break;
    default: return fail(HPS_ERR_INVALID, "get_scalar: unknown scalar");
  }
  return HPS_OK;
}

hps_status hps_beam_update(hps_beam_t b, int op, int coord, int good) {
  if (!valid(b)) return fail(HPS_ERR_INVALID, "bad beam handle");
  ON_DEVICE(b, __func__);
  const DevBeam &d = b->d;
  if ((op == 3 || op == 4) && (coord < 0 || coord > HPS_COORD_PHI_R))
    return fail(HPS_ERR_INVALID, "beam_update: bad coordinate");
  const bool f = f32(b);
  switch (op) {
    case 0: beam_update_loss(d, b->scr, b->stream); break;
    case 1: f ? beam32_update_longitudinal_loss(d, b->scr, b->stream)
              : beam_update_longitudinal_loss(d, b->scr, b->stream); break;
    case 2: beam_update_good_count(d, b->scr, b->stream); break;
    case 3: f ? beam32_update_avg(d, coord, good, b->scr, b->stream)
              : beam_update_avg(d, coord, good, b->scr, b->stream); break;
    case 4: f ? beam32_update_sig(d, coord, good, b->scr, b->stream)
              : beam_update_sig(d, coord, good, b->scr, b->stream); break;
    case 5: f ? beam32_update_emittance(d, b->scr, b->stream) : beam_update_emittance(d, b->scr, b->stream); break;
    case 6: f ? beam32_update_relative_phi(d, good, b->stream) : beam_update_relative_phi(d, good, b->stream); break;
    case 7: f ? beam32_update_stat_for_sc(d, b->scr, b->stream) : beam_update_stat_for_sc(d, b->scr, b->stream); break;
    case 8: f ? beam32_update_avg_xy(d, b->scr, b->stream) : beam_update_avg_xy(d, b->scr, b->stream); break;
    case 9: f ? beam32_update_max_r_phi(d, b->scr, b->stream) : beam_update_max_r_phi(d, b->scr, b->stream); break;
    default: return fail(HPS_ERR_INVALID, "beam_update: unknown op");
  }
  hps_status s = last_launch_status("beam_update");
  if (s) return s;
  return sync(b);
}

hps_status hps_beam_get_stat(hps_beam_t b, int stat, double *out) {
  if (!valid(b) || !out || stat < 0 || stat >= HPS_NST) return fail(HPS_ERR_INVALID, "get_stat: bad argument");
  ON_DEVICE(b, __func__);
  BeamStats h;
  CK(cudaMemcpyAsync(&h, b->d.st, sizeof(h), cudaMemcpyDeviceToHost, b->stream));
  hps_status s = sync(b);
  if (s) return s;
  if (stat < NSTAT) *out = h.st[stat];
  else if (stat == HPS_ST_NUM_LOSS) *out = h.num_loss;
  else if (stat == HPS_ST_NUM_LLOSS) *out = h.num_lloss;
  else *out = h.num_good;
  return HPS_OK;
}

hps_status hps_beam_apply_cut(hps_beam_t b, char coord, double lo, double hi) {
  if (!valid(b)) return fail(HPS_ERR_INVALID, "bad beam handle");
  ON_DEVICE(b, __func__);
  char c = (char)std::tolower((unsigned char)coord);
  int k = c == 'x' ? HPS_COORD_X : c == 'y' ? HPS_COORD_Y : c == 'w' ? HPS_COORD_W : c == 'p' ? HPS_COORD_PHI : -1;
  if (k < 0) return HPS_OK;  // the reference leaves the beam untouched
  if (f32(b)) beam32_apply_cut(b->d, k, lo, hi, b->stream);
  else beam_apply_cut(b->d, k, lo, hi, b->stream);
  hps_status s = last_launch_status("apply_cut");
  if (s) return s;
  return sync(b);
}

hps_status hps_beam_translate(hps_beam_t b, int coord, double v) {
  if (!valid(b) || coord < 0 || coord > HPS_COORD_W) return fail(HPS_ERR_INVALID, "translate: bad argument");
  ON_DEVICE(b, __func__);
  if (f32(b)) beam32_shift(b->d, coord, v, b->stream);
  else beam_shift(b->d, coord, v, b->stream);
  if (coord == HPS_COORD_PHI) {  // Beam::ShiftPhi re-initialises <phi>_good
    hps_status s = init_phi_avg_good(b);
    if (s) return s;
  }
  hps_status s = last_launch_status("translate");
  if (s) return s;
  return sync(b);
}

hps_status hps_beam_monitor(hps_beam_t b, double *out) {
  if (!valid(b) || !out) return fail(HPS_ERR_INVALID, "monitor: bad argument");
  ON_DEVICE(b, __func__);
  double *dm = nullptr;
  CK(cudaMalloc((void **)&dm, HPS_NMON * sizeof(double)));
  if (f32(b)) beam32_monitor(b->d, nullptr, dm, 0, b->scr, b->stream);
  else beam_monitor(b->d, nullptr, dm, 0, b->scr, b->stream);
  cudaMemcpyAsync(out, dm, HPS_NMON * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
  hps_status s = sync(b);
  cudaFree(dm);
  return s;
}

// ---- headless plot data (src/graphics/src/graphics_kernel_call.cu) ----------
static PlotCoord plot_coord(hps_beam_t b, int c) {
  PlotCoord p{};
  if (f32(b)) {
    p.f = (const float *)coord_ptr(b, c);
    p.off = c == HPS_COORD_PHI ? b->d.phi_ref : c == HPS_COORD_W ? b->d.w_ref : 0.0;
  } else {
    p.d = (const double *)coord_ptr(b, c);
  }
  return p;
}
static bool plot_coord_ok(int c) { return c >= 0 && c <= HPS_COORD_PHI_R; }

// a device buffer for a result the caller wants on the host (else theirs)
static hps_status plot_out(void *user, size_t bytes, int on_device, void **dev) {
  if (on_device) { *dev = user; return HPS_OK; }
  CK(cudaMalloc(dev, bytes));
  return HPS_OK;
}
static hps_status plot_finish(hps_beam_t b, void *user, void *dev, size_t bytes, int on_device) {
  if (!on_device) cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDeviceToHost, b->stream);
  hps_status s = last_launch_status("plot");
  if (!s) s = sync(b);
  if (!on_device) cudaFree(dev);
  return s;
}

hps_status hps_plot_points(hps_beam_t b, int cx, int cy, float *xy, int on_device) {
  if (!valid(b) || !xy || !plot_coord_ok(cx) || !plot_coord_ok(cy)) return fail(HPS_ERR_INVALID, "plot_points: bad argument");
  ON_DEVICE(b, __func__);
  const size_t bytes = (size_t)b->n * sizeof(float2);
  void *dev = nullptr;
  hps_status s = plot_out(xy, bytes, on_device, &dev);
  if (s) return s;
  plot_points(plot_coord(b, cx), plot_coord(b, cy), b->d.loss, b->n, (float2 *)dev, b->stream);
  return plot_finish(b, xy, dev, bytes, on_device);
}

hps_status hps_plot_maxmin(hps_beam_t b, int cx, int cy, int live_only, double out[4]) {
  if (!valid(b) || !out || !plot_coord_ok(cx) || !plot_coord_ok(cy)) return fail(HPS_ERR_INVALID, "plot_maxmin: bad argument");
  ON_DEVICE(b, __func__);
  void *dev = nullptr;
  hps_status s = plot_out(out, 4 * sizeof(double), 0, &dev);
  if (s) return s;
  plot_maxmin(plot_coord(b, cx), plot_coord(b, cy), live_only ? b->d.loss : nullptr, b->n, b->scr, (double *)dev,
              b->stream);
  return plot_finish(b, out, dev, 4 * sizeof(double), 0);
}

hps_status hps_plot_histogram(hps_beam_t b, int coord, uint32_t nbins, double mn, double mx, uint32_t *hist,
                              int on_device) {
  if (!valid(b) || !hist || !plot_coord_ok(coord) || nbins < 1 || nbins > HPS_PLOT_MAX_BINS || !(mx > mn))
    return fail(HPS_ERR_INVALID, "plot_histogram: bad argument (1 <= nbins <= 12288, max > min)");
  ON_DEVICE(b, __func__);
  const size_t bytes = (size_t)nbins * sizeof(uint32_t);
  void *dev = nullptr;
  hps_status s = plot_out(hist, bytes, on_device, &dev);
  if (s) return s;
  plot_hist(plot_coord(b, coord), b->d.loss, b->n, nbins, mn, mx, (uint32_t *)dev, b->stream);
  return plot_finish(b, hist, dev, bytes, on_device);
}

hps_status hps_plot_histogram2d(hps_beam_t b, int cx, int cy, uint32_t nx, uint32_t ny, const double maxmin[4],
                                uint32_t *hist, int on_device) {
  if (!valid(b) || !hist || !maxmin || !plot_coord_ok(cx) || !plot_coord_ok(cy) || nx < 1 || ny < 1 ||
      (uint64_t)nx * ny > (1ull << 26))
    return fail(HPS_ERR_INVALID, "plot_histogram2d: bad argument");
  ON_DEVICE(b, __func__);
  const size_t bytes = (size_t)nx * ny * sizeof(uint32_t);
  void *dev = nullptr;
  hps_status s = plot_out(hist, bytes, on_device, &dev);
  if (s) return s;
  plot_hist2d(plot_coord(b, cx), plot_coord(b, cy), b->d.loss, b->n, maxmin, nx, ny, (uint32_t *)dev, b->stream);
  return plot_finish(b, hist, dev, bytes, on_device);
}

// ---- BeamLine ---------------------------------------------------------------
hps_status hps_beamline_create(hps_beamline_t *out) {
  if (!out) return fail(HPS_ERR_INVALID, "null output");
  *out = new hps_beamline_s();
  return HPS_OK;
}
hps_status hps_beamline_destroy(hps_beamline_t bl) {
  delete bl;
  return HPS_OK;
}
hps_status hps_beamline_add(hps_beamline_t bl, int type, const char *name, const double *params) {
  if (!bl || !name || !params) return fail(HPS_ERR_INVALID, "beamline_add: bad argument");
  if (type < HPS_ELEM_DRIFT || type > HPS_ELEM_DIPOLE) return fail(HPS_ERR_INVALID, "beamline_add: unknown type");
  bl->types.push_back(type);
  bl->names.push_back(name);
  bl->params.emplace_back(params, params + HPS_NPARAM);
  bl->version++;
  return HPS_OK;
}
hps_status hps_beamline_size(hps_beamline_t bl, uint32_t *out) {
  if (!bl || !out) return fail(HPS_ERR_INVALID, "bad argument");
  *out = (uint32_t)bl->types.size();
  return HPS_OK;
}
static bool ieq(const std::string &a, const std::string &b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
  return true;
}
hps_status hps_beamline_find(hps_beamline_t bl, const char *name, uint32_t *index) {
  if (!bl || !name || !index) return fail(HPS_ERR_INVALID, "bad argument");
  for (size_t i = 0; i < bl->names.size(); ++i)
    if (ieq(bl->names[i], name)) { *index = (uint32_t)i; return HPS_OK; }
  return fail(HPS_ERR_NOT_FOUND, std::string("Invalid beamline element name, please check it! (") + name + ")");
}
hps_status hps_beamline_get(hps_beamline_t bl, uint32_t i, int *type, char *name, size_t cap, double *params) {
  if (!bl || i >= bl->types.size()) return fail(HPS_ERR_INVALID, "beamline_get: bad index");
  if (type) *type = bl->types[i];
  if (name && cap) { std::strncpy(name, bl->names[i].c_str(), cap - 1); name[cap - 1] = 0; }
  if (params) std::memcpy(params, bl->params[i].data(), HPS_NPARAM * sizeof(double));
  return HPS_OK;
}
hps_status hps_beamline_set_param(hps_beamline_t bl, uint32_t i, int slot, double v) {
  if (!bl || i >= bl->types.size() || slot < 0 || slot >= HPS_NPARAM) return fail(HPS_ERR_INVALID, "set_param: bad argument");
  bl->params[i][slot] = v;
  bl->version++;
  return HPS_OK;
}

// ---- SCHEFF -----------------------------------------------------------------
static bool pow2(uint32_t v) { return v && !(v & (v - 1)); }

static hps_status scheff_upload(hps_scheff_t s) {
  ScState h{};
  CK(cudaMemcpy(&h, s->d, sizeof(h), cudaMemcpyDeviceToHost));
  h.nx = s->nx; h.nz = s->nz; h.nx_init = s->nx_init; h.nz_init = s->nz_init;
  h.nx_max = s->nx_max; h.nz_max = s->nz_max;
  h.adj_bunch = s->adj_bunch; h.adj_bunch_w = s->adj_bunch_w; h.mesh_w = s->mesh_w;
  h.remesh_val = s->remesh_val; h.interval = s->interval; h.interval_init = s->interval_init;
  CK(cudaMemcpy(s->d, &h, sizeof(h), cudaMemcpyHostToDevice));
  s->version++;
  return HPS_OK;
}

static void scheff_free_tables(hps_scheff_t s) {
  void *p[] = {s->t.bin_fx, s->t.fld1, s->t.fld2, s->t.ffld1, s->t.ffld2, s->t.c32, s->t.tcg, s->t.tcp};
  for (void *q : p)
    if (q) cudaFree(q);
  s->t = ScTables{};
}

// the tensor-core contraction's buffers for the largest mesh (FP32 beams),
// when that mesh allows it and the solver does not ask for CUDA cores
static hps_status scheff_alloc_tc(hps_scheff_t s) {
  if (s->t.tcg) cudaFree(s->t.tcg);
  if (s->t.tcp) cudaFree(s->t.tcp);
  s->t.tcg = nullptr;
  s->t.tcp = nullptr;
  s->t.tc_nr = s->t.tc_nz = 0;
  if (s->contraction != 0 || !sc32_tc_mesh(s->nx_max, s->nz_max)) return HPS_OK;
  size_t pb = 0;
  const size_t gb = sc32_tc_bytes(s->nx_max, s->nz_max, &pb);
  unsigned char *g = nullptr;
  float *p = nullptr;
  hps_status st;
  if ((st = dmalloc(&g, gb))) return st;
  if ((st = dmalloc(&p, pb / sizeof(float)))) { cudaFree(g); return st; }
  s->t.tcg = g;
  s->t.tcp = p;
  s->t.tc_nr = s->nx_max;
  s->t.tc_nz = s->nz_max;
  return HPS_OK;
}

static hps_status scheff_alloc_tables(hps_scheff_t s) {
  scheff_free_tables(s);
  hps_status st;
  size_t nx = s->nx_max, nz = s->nz_max;
  if ((st = dmalloc(&s->t.bin_fx, nx * nz))) return st;
  if ((st = dmalloc(&s->t.fld1, (nx + 1) * nx * nz * 2))) return st;
  if ((st = dmalloc(&s->t.fld2, (nz + 1) * (nx + 1) * 2))) return st;
  if ((st = dmalloc(&s->t.ffld1, (nx + 1) * nx * nz * 2))) return st;
  if ((st = dmalloc(&s->t.ffld2, (nz + 1) * (nx + 1) * 2))) return st;
  if ((st = dmalloc(&s->t.c32, 1))) return st;
  if ((st = scheff_alloc_tc(s))) return st;
  sc_configure(nx * nz * sizeof(unsigned long long));
  return HPS_OK;
}

hps_status hps_scheff_create(uint32_t nr, uint32_t nz, uint32_t adj_bunch, hps_scheff_t *out) {
  if (!out) return fail(HPS_ERR_INVALID, "null output");
  *out = nullptr;
  if (!pow2(nr) || !pow2(nz) || nz > 512 || nr > 256)
    return fail(HPS_ERR_INVALID, "SCHEFF mesh: nr and nz must be powers of two, nz <= 512, nr <= 256");
  hps_scheff_t s = new hps_scheff_s();
  cudaGetDevice(&s->dev);
  s->nx = s->nx_init = nr; s->nz = s->nz_init = nz; s->adj_bunch = adj_bunch;
  s->nx_max = nr; s->nz_max = nz;
  hps_status st;
  if ((st = dmalloc(&s->d, 1)) || (st = scheff_alloc_tables(s)) || (st = scheff_upload(s))) {
    hps_scheff_destroy(s);
    return st;
  }
  *out = s;
  return HPS_OK;
}

hps_status hps_scheff_destroy(hps_scheff_t s) {
  if (!s) return HPS_OK;
  cudaDeviceSynchronize();
  if (s->d) cudaFree(s->d);
  scheff_free_tables(s);
  delete s->sur;
  delete s;
  return HPS_OK;
}

// SpaceCharge setters, space_charge.h:43-87
hps_status hps_scheff_set(hps_scheff_t s, int param, double v) {
  if (!s) return fail(HPS_ERR_INVALID, "bad scheff handle");
  ON_DEVICE(s, __func__);
  switch (param) {
    case 0: s->interval = v; s->interval_init = v; break;
    case 1: s->adj_bunch = (uint32_t)v; break;
    case 2: s->adj_bunch_w = v; break;
    case 3: s->mesh_w = v; break;
    case 4: s->remesh_val = v; break;
    case 5: s->fraction = v; break;
    case 10: {
      if (v != 0.0 && v != 1.0) return fail(HPS_ERR_INVALID, "scheff_set: contraction kernel is 0 or 1");
      if ((int)v == s->contraction) return HPS_OK;
      CK(cudaDeviceSynchronize());
      s->contraction = (int)v;
      hps_status st = scheff_alloc_tc(s);
      if (st) return st;
      break;
    }
    case 13: {
      if (v != 0.0 && v != 1.0) return fail(HPS_ERR_INVALID, "scheff_set: surrogate layer kernel is 0 or 1");
      s->sur_kernel = (int)v;
      if (s->sur) {
        CK(cudaDeviceSynchronize());
        s->sur->use_tc = s->sur_kernel == 0;
      }
      s->version++;
      break;
    }
    default: return fail(HPS_ERR_INVALID, "scheff_set: unknown or read-only parameter");
  }
  return scheff_upload(s);
}
hps_status hps_scheff_get(hps_scheff_t s, int param, double *v) {
  if (!s || !v) return fail(HPS_ERR_INVALID, "bad argument");
  ON_DEVICE(s, __func__);
  switch (param) {
    case 0: *v = s->interval; break;
    case 1: *v = s->adj_bunch; break;
    case 2: *v = s->adj_bunch_w; break;
    case 3: *v = s->mesh_w; break;
    case 4: *v = s->remesh_val; break;
    case 5: *v = s->fraction; break;
    case 6: *v = s->nx; break;
    case 7: *v = s->nz; break;
    case 8:
    case 9:
    case 12: {  // counters and flags kept by the kernels
      ScState h;
      if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(&h, s->d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(HPS_ERR_CUDA, "scheff_get: reading the solver state failed");
      *v = param == 8 ? (double)h.n_solves : param == 9 ? (double)h.n_stat_sweeps : (double)h.tc_error;
      break;
    }
    case 10: *v = s->contraction; break;
    case 11: *v = s->t.tcg != nullptr; break;
    case 13: *v = s->sur_kernel; break;
    case 14:
    case 15: {
      int k = 0;
      unsigned int err = 0;
      if (s->sur && sur_conv_state(*s->sur, &k, &err)) return fail(HPS_ERR_CUDA, "scheff_get: reading the surrogate state failed");
      *v = param == 14 ? (double)k : (double)err;
      break;
    }
    default: return fail(HPS_ERR_INVALID, "scheff_get: unknown parameter");
  }
  return HPS_OK;
}
// The solver's tables after its last kick: charge (nr*nz, bin (zs, rs) at
// zs*nr + rs), field ((nz+1)*(nr+1) pairs) of the FP32 or FP64 tables, and
// mesh = {nr, nz, dr, dz, beta, num_on_mesh, remesh}; arrays sized for the
// largest mesh.
hps_status hps_scheff_snapshot(hps_scheff_t s, int fp32, double *bins, double *field, double *mesh) {
  if (!s || !bins || !field || !mesh) return fail(HPS_ERR_INVALID, "scheff_snapshot: bad argument");
  ON_DEVICE(s, __func__);
  CK(cudaDeviceSynchronize());
  ScState h;
  CK(cudaMemcpy(&h, s->d, sizeof(h), cudaMemcpyDeviceToHost));
  const size_t nb = (size_t)h.nx * h.nz, nf = (size_t)(h.nz + 1) * (h.nx + 1) * 2;
  std::vector<unsigned long long> fx(nb);
  CK(cudaMemcpy(fx.data(), s->t.bin_fx, nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  for (size_t k = 0; k < nb; ++k) bins[k] = (double)(long long)fx[k] * kBinInvScale;
  if (fp32) {
    std::vector<float> f(nf);
    CK(cudaMemcpy(f.data(), s->t.ffld2, nf * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < nf; ++k) field[k] = f[k];
  } else {
    CK(cudaMemcpy(field, s->t.fld2, nf * sizeof(double), cudaMemcpyDeviceToHost));
  }
  mesh[0] = h.nx; mesh[1] = h.nz; mesh[2] = h.dr; mesh[3] = h.dz; mesh[4] = h.beta;
  mesh[5] = h.num_on_mesh; mesh[6] = h.remesh;
  return HPS_OK;
}

// Scheff::SetMeshSize, space_charge.cpp:61-73 (tables reallocated and zeroed)
hps_status hps_scheff_set_mesh_size(hps_scheff_t s, uint32_t nr, uint32_t nz) {
  if (!s) return fail(HPS_ERR_INVALID, "bad scheff handle");
  ON_DEVICE(s, __func__);
  if (!pow2(nr) || !pow2(nz) || nz > 512 || nr > 256)
    return fail(HPS_ERR_INVALID, "SCHEFF mesh: nr and nz must be powers of two, nz <= 512, nr <= 256");
  if (nr == s->nx && nz == s->nz) return HPS_OK;
  s->nx = nr; s->nz = nz;
  s->nx_max = std::max(s->nx_max, nr);
  s->nz_max = std::max(s->nz_max, nz);
  hps_status st = scheff_alloc_tables(s);
  if (st) return st;
  return scheff_upload(s);
}

hps_status hps_scheff_set_surrogate(hps_scheff_t s, int32_t n_layers, const int32_t *arch, int32_t gmean_after,
                                    const int32_t *skip, const uint16_t *const *weights, const float *const *biases,
                                    uint32_t nr, uint32_t nz, double out_scale, double tol, uint32_t n_samples) {
  if (!s) return fail(HPS_ERR_INVALID, "bad scheff handle");
  ON_DEVICE(s, __func__);
  CK(cudaDeviceSynchronize());
  SurNet *n = new SurNet();
  std::string err;
  const int r = sur_build(*n, n_layers, arch, gmean_after, skip, weights, biases, nr, nz, out_scale, tol, n_samples,
                          err);
  if (r) {
    delete n;
    return fail(r == 1 ? HPS_ERR_INVALID : HPS_ERR_CUDA, ("scheff_set_surrogate: " + err).c_str());
  }
  n->use_tc = s->sur_kernel == 0;
  delete s->sur;
  s->sur = n;
  s->version++;
  return HPS_OK;
}

hps_status hps_scheff_clear_surrogate(hps_scheff_t s) {
  if (!s) return fail(HPS_ERR_INVALID, "bad scheff handle");
  ON_DEVICE(s, __func__);
  if (!s->sur) return HPS_OK;
  CK(cudaDeviceSynchronize());
  delete s->sur;
  s->sur = nullptr;
  s->version++;
  return HPS_OK;
}

hps_status hps_scheff_surrogate_stats(hps_scheff_t s, double *accepted, double *rejected, double *residual) {
  if (!s || !s->sur) return fail(HPS_ERR_INVALID, "scheff_surrogate_stats: no surrogate attached");
  ON_DEVICE(s, __func__);
  if (sur_read(*s->sur, accepted, rejected, residual)) return fail(HPS_ERR_CUDA, "scheff_surrogate_stats: read failed");
  return HPS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------
namespace {

struct Ctx {
  hps_sim_t s;
  hps_beam_t b;
  hps_beamline_t bl;
  hps_scheff_t sc;
  bool kicked = false;  // a SCHEFF kick of this simulation call has been issued
};

const double *P(hps_beamline_t bl, uint32_t i) { return bl->params[i].data(); }

void prof_mark(Ctx &c, int cls, bool begin) {
  hps_sim_t s = c.s;
  if (!s->prof_on) return;
  size_t k = begin ? 2 * s->prof_used : 2 * s->prof_used + 1;
  while (s->prof_pool.size() <= k) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    s->prof_pool.push_back(e);
  }
  cudaEventRecord(s->prof_pool[k], c.b->stream);
  if (!begin) {
    if (s->prof_cls.size() <= s->prof_used) s->prof_cls.resize(s->prof_used + 1);
    s->prof_cls[s->prof_used] = cls;
    s->prof_used++;
  }
}
#define PHASE(cls, ...)            \
  do {                              \
    prof_mark(c, cls, true);        \
    __VA_ARGS__;                    \
    prof_mark(c, cls, false);       \
  } while (0)
int T(hps_beamline_t bl, int64_t i) {
  return (i >= 0 && i < (int64_t)bl->types.size()) ? bl->types[i] : 0;
}

// the arguments of one SCHEFF kick of the given length
ScKickArgs kick_args(Ctx &c, double length) {
  hps_beam_t b = c.b;
  ScKickArgs a;
  a.freq = b->freq;
  a.current = b->current;
  a.frac = c.sc->fraction;
  a.length = length;
  a.skip_stride = (uint64_t)b->grid_size * (b->blck_size / 4);
  a.deposit_ok = (b->blck_size / 4) > 0;
  a.stats_ok = b->n > 2;
  a.deposit_smem = (size_t)c.sc->nx_max * c.sc->nz_max * sizeof(unsigned long long);
  a.nx_max = c.sc->nx_max;
  a.nz_max = c.sc->nz_max;
  a.adj_possible = c.sc->adj_bunch != 0;
  a.mesh_fixed = c.sc->mesh_w == 0.0 && c.sc->nx == c.sc->nx_max && c.sc->nz == c.sc->nz_max;
  a.dep_per_sm = c.s->dep_per_sm;
  a.dep_agg = c.s->dep_agg;
  a.dep_threads = c.s->dep_threads;
  return a;
}

// FP32 beams with a solver: the element half before the kick also takes the
// kick's statistics (PUSH_SCSTATS), the half after it runs behind the kick
// in one sweep (PUSH_AFTER_KICK).  Every launch of the unfused sequence is
// valid from four particles on (blck_size/4 > 0, n > 2).
struct Fuse32 {
  bool on;
  PushFuse pre, post;
};
Fuse32 fuse32(Ctx &c) {
  Fuse32 z{};
  hps_beam_t b = c.b;
  const uint64_t stride = (uint64_t)b->grid_size * (b->blck_size / 4);
  z.on = f32(b) && c.s->sc_on && c.sc && b->n >= 4 && stride != 0 && (stride & (stride - 1)) == 0;
  if (!z.on) return z;
  z.pre.mode = PUSH_SCSTATS;
  z.pre.scr = b->scr;
  z.pre.sc = c.sc->d;
  z.pre.t = c.sc->t;
  z.pre.t.fld2 = nullptr;
  z.post.mode = PUSH_AFTER_KICK;
  z.post.sc = c.sc->d;
  z.post.t = c.sc->t;
  z.post.t.fld2 = nullptr;
  z.post.skip_mask = stride - 1;
  return z;
}

// the PUSH_SCSTATS form for the half before a kick of the given length
const PushFuse *pre_for(Ctx &c, const Fuse32 &z, double length, PushFuse *out) {
  if (!z.on) return nullptr;
  *out = z.pre;
  const ScKickArgs a = kick_args(c, length);
  out->h = sc32_host(c.b->d, a);
  out->freq = a.freq;
  out->frac = a.frac;
  out->s_last = c.kicked;  // results depend on the call's inputs only
  return out;
}

// fused: what the PUSH_SCSTATS half left of the statistics, and the mesh;
// the kick runs with the next half
void sc_apply(Ctx &c, double length, bool fused = false) {
  if (!(c.s->sc_on && c.sc)) return;
  c.kicked = true;
  hps_beam_t b = c.b;
  const ScKickArgs a = kick_args(c, length);
  if (f32(b)) {
    sc32_configure();
    if (fused) {
      PHASE(HPS_PROF_SC_STATS, sc32_stats_after_push(b->d, c.sc->d, c.sc->t, a, b->scr, b->stream));
      PHASE(HPS_PROF_SC_MESH, sc32_mesh(b->d, c.sc->d, c.sc->t, a, b->scr, b->stream, c.sc->sur, &b->fork));
      return;
    }
    PHASE(HPS_PROF_SC_STATS, sc32_stats(b->d, c.sc->d, c.sc->t, a, b->scr, b->stream));
    PHASE(HPS_PROF_SC_MESH, sc32_mesh(b->d, c.sc->d, c.sc->t, a, b->scr, b->stream, c.sc->sur, &b->fork));
    PHASE(HPS_PROF_SC_KICK, sc32_kick(b->d, c.sc->d, c.sc->t, a, b->stream));
    return;
  }
  ScTables t = c.sc->t;
  t.ffld2 = nullptr;  // FP64 beams use fld2
  PHASE(HPS_PROF_SC_STATS, sc_stats(b->d, c.sc->d, t, a, b->scr, b->stream));
  PHASE(HPS_PROF_SC_MESH, sc_mesh(b->d, c.sc->d, t, a, b->scr, b->stream, c.sc->sur));
  PHASE(HPS_PROF_SC_KICK, sc_kick(b->d, c.sc->d, t, a, b->stream));
}

// PrepSimulateRFGap, simulation_engine.cu:163-175
void prep_gap(Ctx &c, const GapArgs &g) {
  hps_beam_t b = c.b;
  if (b->freq != g.frequency) {
    c.s->wavelen = CLIGHT / g.frequency;
    double ratio = g.frequency / b->freq;
    b->current *= g.frequency / b->freq;
    if (f32(b)) PHASE(HPS_PROF_OTHER, beam32_change_frequency(b->d, ratio, b->scr, b->stream));
    else PHASE(HPS_PROF_OTHER, beam_change_frequency(b->d, ratio, b->scr, b->stream));
    b->freq = g.frequency;
  }
}

void monitor_at(Ctx &c, uint32_t i) {
  hps_beam_t b = c.b;
  const ScState *sc = (c.s->sc_on && c.sc) ? c.sc->d : nullptr;
  double *dst = c.s->mon_dev + (size_t)i * HPS_NMON;
  if (f32(b)) PHASE(HPS_PROF_MONITOR, beam32_monitor(b->d, sc, dst, i, b->scr, b->stream));
  else PHASE(HPS_PROF_MONITOR, beam_monitor(b->d, sc, dst, i, b->scr, b->stream));
}

// the element visitors of simulation_engine.cu:125-373
hps_status visit(Ctx &c, uint32_t i) {
  hps_sim_t s = c.s;
  hps_beam_t b = c.b;
  hps_beamline_t bl = c.bl;
  const double *p = P(bl, i);
  DevBeam &d = b->d;
  const bool f = f32(b);
  cudaStream_t st = b->stream;
  uint32_t eid = s->cur_id;
  const Fuse32 z = fuse32(c);
  const PushFuse *post = z.on ? &z.post : nullptr;
  PushFuse pre_buf;
  auto pre = [&](double length) { return pre_for(c, z, length, &pre_buf); };
  // a half that runs behind the kick is timed as the kick
  auto post_cls = [&](int cls) { return z.on ? (int)HPS_PROF_SC_KICK : cls; };
  switch (bl->types[i]) {
    case HPS_ELEM_DRIFT: {
      int nk = 1;
      double length = p[HPS_P_LENGTH];
      if (s->sc_on && c.sc) nk = (int)std::ceil(length / c.sc->interval);
      double hf = 0.5 * length / nk;
      for (int k = 0; k < nk; ++k) {
        PHASE(HPS_PROF_DRIFT, f ? push32_partial_drift(d, s->wavelen, hf, p[HPS_P_APERTURE], eid, st, pre(2.0 * hf))
                                : push_partial_drift(d, s->wavelen, hf, p[HPS_P_APERTURE], eid, st));
        sc_apply(c, 2.0 * hf, z.on);
        PHASE(post_cls(HPS_PROF_DRIFT), f ? push32_partial_drift(d, s->wavelen, hf, p[HPS_P_APERTURE], eid, st, post)
                                : push_partial_drift(d, s->wavelen, hf, p[HPS_P_APERTURE], eid, st));
      }
      break;
    }
    case HPS_ELEM_QUAD:
      if (b->blck_size / 2 > 0)
        PHASE(HPS_PROF_QUAD,
              f ? push32_half_quad(d, s->wavelen, p[HPS_P_LENGTH], p[HPS_P_APERTURE], p[HPS_P_GRADIENT], eid, st,
                                   pre(p[HPS_P_LENGTH]))
                : push_half_quad(d, s->wavelen, p[HPS_P_LENGTH], p[HPS_P_APERTURE], p[HPS_P_GRADIENT], eid, st));
      sc_apply(c, p[HPS_P_LENGTH], z.on);
      if (b->blck_size / 2 > 0)
        PHASE(post_cls(HPS_PROF_QUAD),
              f ? push32_half_quad(d, s->wavelen, p[HPS_P_LENGTH], p[HPS_P_APERTURE], p[HPS_P_GRADIENT], eid, st, post)
                : push_half_quad(d, s->wavelen, p[HPS_P_LENGTH], p[HPS_P_APERTURE], p[HPS_P_GRADIENT], eid, st));
      break;
    case HPS_ELEM_RFGAP_DTL: {
      GapArgs g;
      load_gap_args(p, &g);
      prep_gap(c, g);
      double phi_in = 0.0;
      uint32_t sz = (uint32_t)bl->types.size(), cur = s->cur_id;
      if (cur == 1 || (cur > 1 && T(bl, cur - 2) != HPS_ELEM_RFGAP_DTL)) {
        if (cur + 2 < sz && T(bl, cur + 2) == HPS_ELEM_RFGAP_DTL)
          phi_in = g.phase_ref - 0.5 * (P(bl, cur + 2)[HPS_P_RF_PHASE_REF] - g.phase_ref);
        else if (cur + 1 >= sz)
          return fail(HPS_ERR_LATTICE, "BeamLine is not set up correctly: there should be a quad following a DTL gap");
        else phi_in = g.phase_ref;
      } else if (cur > 1) {
        phi_in = 0.5 * (P(bl, cur - 2)[HPS_P_RF_PHASE_REF] + g.phase_ref);
      } else {
        return fail(HPS_ERR_LATTICE, "A quad is missing before the DTL gap");
      }
      if (T(bl, (int64_t)cur - 1) != HPS_ELEM_QUAD || T(bl, (int64_t)cur + 1) != HPS_ELEM_QUAD)
        return fail(HPS_ERR_LATTICE, "a DTL gap needs a quad on each side");
      g.q1 = P(bl, cur - 1)[HPS_P_LENGTH];
      g.q2 = P(bl, cur + 1)[HPS_P_LENGTH];
      g.design_w_in = s->design_w;
      g.phi_in = phi_in;
      g.ccl = 0;
      g.ccl_cell_num = 0;
      s->wavelen = CLIGHT / g.frequency;  // d_wavelen written by the first-half kernel
      g.wl = s->wavelen;
      if (b->blck_size / 2 > 0) PHASE(HPS_PROF_GAP1, f ? push32_gap_first(d, g, st, pre(g.length)) : push_gap_first(d, g, st));
      sc_apply(c, g.length, z.on);
      if (b->blck_size / 2 > 0)
        PHASE(post_cls(HPS_PROF_GAP2), f ? push32_gap_second(d, g, st, post) : push_gap_second(d, g, st));
      s->design_w = g.energy_out;
      b->design_w = s->design_w;
      break;
    }
    case HPS_ELEM_RFGAP_CCL: {
      GapArgs g;
      load_gap_args(p, &g);
      prep_gap(c, g);
      uint32_t cur = s->cur_id;
      if (cur == 0 || T(bl, (int64_t)cur - 1) != HPS_ELEM_RFGAP_CCL) s->ccl_cell_num = 0;
      double phi_in, phi_out, cp = g.phase_ref;
      if (s->ccl_cell_num == 0) {
        int tn = T(bl, cur + 1);
        if (tn != HPS_ELEM_RFGAP_CCL && tn != HPS_ELEM_RFGAP_DTL)
          return fail(HPS_ERR_LATTICE, "the first CCL gap of a tank needs an RF gap after it");
        double nxt = P(bl, cur + 1)[HPS_P_RF_PHASE_REF];
        phi_in = cp - 0.5 * (nxt - cp);
        phi_out = 0.5 * (nxt + cp);
      } else if (T(bl, cur + 1) != HPS_ELEM_RFGAP_CCL) {
        double prv = P(bl, cur - 1)[HPS_P_RF_PHASE_REF];
        phi_in = 0.5 * (cp + prv);
        phi_out = cp + 0.5 * (cp - prv);
      } else {
        phi_in = 0.5 * (cp + P(bl, cur - 1)[HPS_P_RF_PHASE_REF]);
        phi_out = 0.5 * (cp + P(bl, cur + 1)[HPS_P_RF_PHASE_REF]);
      }
      g.q1 = g.q2 = 0.0;
      g.design_w_in = s->design_w;
      g.ccl = 1;
      uint32_t gcb = b->blck_size / 4 > 1 ? b->blck_size / 4 : b->blck_size;
      s->wavelen = CLIGHT / g.frequency;
      g.wl = s->wavelen;
      g.phi_in = phi_in;
      g.ccl_cell_num = 0;
      if (gcb > 0) PHASE(HPS_PROF_GAP1, f ? push32_gap_first(d, g, st, pre(g.length)) : push_gap_first(d, g, st));
      sc_apply(c, g.length, z.on);
      g.phi_in = phi_out;
      g.ccl_cell_num = s->ccl_cell_num;
      if (gcb > 0) PHASE(post_cls(HPS_PROF_GAP2), f ? push32_gap_second(d, g, st, post) : push_gap_second(d, g, st));
      s->ccl_cell_num++;
      s->design_w = g.energy_out;
      b->design_w = s->design_w;
      break;
    }
    case HPS_ELEM_ROTATION:
      PHASE(HPS_PROF_OTHER, f ? push32_rotation(d, p[HPS_P_ROT_ANGLE], st) : push_rotation(d, p[HPS_P_ROT_ANGLE], st));
      break;
    case HPS_ELEM_SPCHCOMP:
      if (s->sc_on && c.sc) c.sc->fraction = p[HPS_P_SPC_FRACTION];
      break;
    case HPS_ELEM_APERTURE_C:
    case HPS_ELEM_APERTURE_R:
      if (p[HPS_P_APT_IN] == 0.0) break;
      PHASE(HPS_PROF_OTHER, beam_update_loss(d, b->scr, st);
            f ? beam32_update_avg_xy(d, b->scr, st) : beam_update_avg_xy(d, b->scr, st);
            f ? push32_aperture(d, bl->types[i] == HPS_ELEM_APERTURE_R, p, eid, st)
              : push_aperture(d, bl->types[i] == HPS_ELEM_APERTURE_R, p, eid, st));
      break;
    case HPS_ELEM_DIAGNOSTICS:
      break;
    case HPS_ELEM_STEERER: {
      double blh = p[HPS_P_STR_BLH], blv = p[HPS_P_STR_BLV];
      if (blh > 1e-10 || blv > 1e-10)
        PHASE(HPS_PROF_OTHER, f ? push32_steerer(d, blh, blv, st) : push_steerer(d, blh, blv, st));
      break;
    }
    case HPS_ELEM_BUNCHER: {
      if (p[HPS_P_BUN_ON] == 0.0) break;
      double bf = p[HPS_P_BUN_FREQ];
      s->wavelen = CLIGHT / bf;
      PHASE(HPS_PROF_OTHER,
            f ? push32_buncher(d, s->wavelen, s->design_w, bf, p[HPS_P_BUN_VOLTAGE], p[HPS_P_BUN_PHASE],
                               p[HPS_P_APERTURE], bf / b->freq, eid, st)
              : push_buncher(d, s->wavelen, s->design_w, bf, p[HPS_P_BUN_VOLTAGE], p[HPS_P_BUN_PHASE],
                             p[HPS_P_APERTURE], bf / b->freq, eid, st));
      break;
    }
    case HPS_ELEM_DIPOLE:
      if (b->blck_size / 4 > 0)
        PHASE(HPS_PROF_OTHER,
              f ? push32_dipole(d, p, s->wavelen, 0, st, pre(p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE])) : push_dipole(d, p, s->wavelen, 0, st));
      sc_apply(c, p[HPS_P_DIP_RADIUS] * p[HPS_P_DIP_ANGLE], z.on);
      if (b->blck_size / 4 > 0)
        PHASE(post_cls(HPS_PROF_OTHER),
              f ? push32_dipole(d, p, s->wavelen, 1, st, post) : push_dipole(d, p, s->wavelen, 1, st));
      break;
    default:
      return fail(HPS_ERR_LATTICE, "unknown element type");
  }
  return HPS_OK;
}

// SimulationEngine::Simulate, simulation_engine.cpp:447-469
hps_status run_range(Ctx &c, int start_index, int end_index, bool monitor) {
  hps_sim_t s = c.s;
  for (int i = 0; i <= end_index; ++i) {
    if (i >= start_index || c.bl->types[i] == HPS_ELEM_SPCHCOMP) {
      s->cur_id = (uint32_t)i;
      hps_status st = visit(c, (uint32_t)i);
      if (st) return st;
      if (monitor) monitor_at(c, (uint32_t)i);
    }
  }
  return last_launch_status("simulate");
}

uint64_t mix(uint64_t h, uint64_t v) {
  h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
  return h;
}
uint64_t mixd(uint64_t h, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  return mix(h, u);
}

// One simulate(start, end) call of a simulator: the checks and the host
// state it starts from (SimulationEngine::Simulate, simulation_engine.cpp:
// 73-95), and whether it runs as a captured graph.
struct RunPlan {
  Ctx c{};
  int n = 0, start_index = 0, end_index = 0;
  bool empty = false, monitor = false, graph = false, host_sync = false;
  uint64_t key = 0;
  double solves0 = 0.0;
};

hps_status plan_run(hps_sim_t s, int32_t start, int32_t end, RunPlan *p) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  p->c = Ctx{s, s->beam, s->bl, s->sc};
  Ctx &c = p->c;
  const int n = (int)c.bl->types.size();
  p->n = n;
  if (n == 0) { p->empty = true; return HPS_OK; }
  p->start_index = start < 0 ? 0 : start;
  p->end_index = end < 0 ? n - 1 : end;
  if (p->start_index >= n || p->end_index >= n) return fail(HPS_ERR_INVALID, "simulate: element index out of range");
  // prev_end_element_index_ is an int set to UINT_MAX, i.e. -1
  // (simulation_engine.cpp:51, simulation_engine.h:66): the first call does
  // not reset, so the design energy and wavelength are the beam's at the
  // simulator's creation
  if (p->start_index < s->prev_end) hps_sim_reset(s);
  s->prev_end = p->end_index;
  hps_beam_t b = c.b;
  cudaStream_t st = b->stream;
  b->d.sweep_cap = s->sweep_cap;
  p->monitor = s->mon_host && s->mon_cap >= (uint32_t)n;
  if (p->monitor && s->mon_dev_cap < (uint32_t)n) {
    if (s->mon_dev) cudaFree(s->mon_dev);
    s->mon_dev = nullptr;
    hps_status e = dmalloc(&s->mon_dev, (size_t)n * HPS_NMON);
    if (e) return e;
    s->mon_dev_cap = n;
  }
  if (p->monitor && c.sc) {
    ScState h;
    CK(cudaMemcpyAsync(&h, c.sc->d, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    p->solves0 = h.n_solves;
  }
  // graphs need the host-side state to be a function of the inputs; the
  // mesh-size cut-off reads the solver's interval back after every kick
  p->host_sync = s->sc_on && c.sc && c.sc->mesh_w != 0.0;
  p->graph = s->use_graph && !p->host_sync && !s->prof_on;
  s->prof_used = 0;
  if (p->graph) {
    uint64_t key = 0;
    key = mix(key, (uint64_t)p->start_index);
    key = mix(key, (uint64_t)p->end_index);
    key = mix(key, c.bl->version);
    key = mix(key, (uint64_t)(uintptr_t)c.bl);
    key = mix(key, c.sc ? c.sc->version : 0);
    key = mix(key, (uint64_t)s->sc_on);
    key = mix(key, (uint64_t)p->monitor);
    key = mix(key, (uint64_t)s->cur_id);
    key = mix(key, (uint64_t)s->ccl_cell_num);
    key = mixd(key, s->design_w);
    key = mixd(key, s->wavelen);
    key = mixd(key, b->freq);
    key = mixd(key, b->current);
    key = mixd(key, b->design_w);
    key = mixd(key, c.sc ? c.sc->fraction : 0.0);
    key = mixd(key, c.sc ? c.sc->interval : 0.0);
    // FP32 beams: the synchronous particle the launch parameters derive from
    key = mix(key, (uint64_t)b->prec);
    key = mixd(key, b->d.phi_ref);
    key = mixd(key, b->d.w_ref);
    // launch shapes
    key = mix(key, (uint64_t)s->sweep_cap);
    key = mix(key, (uint64_t)s->dep_per_sm);
    key = mix(key, (uint64_t)s->dep_agg);
    key = mix(key, (uint64_t)s->dep_threads);
    key = mix(key, c.sc ? (uint64_t)c.sc->contraction : 0);
    p->key = key | 1ull;
  }
  return HPS_OK;
}

HostState host_get(hps_sim_t s) {
  HostState h;
  hps_beam_t b = s->beam;
  h.design_w = s->design_w; h.wavelen = s->wavelen; h.ccl_cell_num = s->ccl_cell_num; h.cur_id = s->cur_id;
  h.beam_freq = b->freq; h.beam_current = b->current; h.beam_design_w = b->design_w;
  h.phi_ref = b->d.phi_ref; h.w_ref = b->d.w_ref;
  h.fraction = s->sc ? s->sc->fraction : 0.0;
  h.interval = s->sc ? s->sc->interval : 0.0;
  return h;
}
void host_put(hps_sim_t s, const HostState &h) {
  hps_beam_t b = s->beam;
  s->design_w = h.design_w; s->wavelen = h.wavelen; s->ccl_cell_num = h.ccl_cell_num; s->cur_id = h.cur_id;
  b->freq = h.beam_freq; b->current = h.beam_current; b->design_w = h.beam_design_w;
  b->d.phi_ref = h.phi_ref; b->d.w_ref = h.w_ref;
  if (s->sc) { s->sc->fraction = h.fraction; s->sc->interval = h.interval; }
}

// The simulator's graph for the plan: the cached one when the host state
// matches (the host state then moves to the end of the range, as a replay
// does), else a new capture (which moves it while recording).  The graph is
// kept uninstantiated too, for batches.  Nothing is launched.
hps_status prepare_graph(RunPlan &p) {
  Ctx &c = p.c;
  hps_sim_t s = c.s;
  hps_beam_t b = c.b;
  cudaStream_t st = b->stream;
  GraphEntry &g = s->graph;
  if (g.exec && g.key == p.key) {
    host_put(s, g.after);
    note_launch((int)g.nkernels);  // a replay launches the captured kernels again
    return HPS_OK;
  }
  // a capture that fails leaves the host state as it was before the range
  const HostState before = host_get(s);
  cudaGraph_t gr = nullptr;
  uint64_t launches0 = g_launches.load();
  cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return fail(HPS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
  hps_status e = run_range(c, p.start_index, p.end_index, p.monitor);
  g.nkernels = g_launches.load() - launches0;
  ce = cudaStreamEndCapture(st, &gr);
  if (e || ce != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    host_put(s, before);
    return e ? e : fail(HPS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
  }
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g.exec = nullptr;
  g.graph = gr;
  g.serial++;
  g.key = 0;
  cudaError_t ie = cudaGraphInstantiate(&g.exec, gr, 0);
  if (ie != cudaSuccess) {
    g.exec = nullptr;
    host_put(s, before);
    return fail(HPS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
  }
  g.key = p.key;
  g.after = host_get(s);
  return HPS_OK;
}

// the monitor's per-kick solve counts from the solver's cumulative counter
void finish_monitor(const RunPlan &p) {
  const Ctx &c = p.c;
  if (!(p.monitor && c.sc && c.s->sc_on)) return;
  double prev = p.solves0;
  for (int i = 0; i <= p.end_index; ++i) {
    if (!(i >= p.start_index || c.bl->types[i] == HPS_ELEM_SPCHCOMP)) continue;
    double *m = c.s->mon_host + (size_t)i * HPS_NMON;
    double cum = m[HPS_MON_SC_REMESH];
    m[HPS_MON_SC_REMESH] = cum - prev;
    prev = cum;
  }
}

}  // namespace

extern "C" {

hps_status hps_sim_create(hps_beam_t beam, hps_beamline_t bl, hps_scheff_t scheff, hps_sim_t *out) {
  if (!out || !valid(beam) || !bl) return fail(HPS_ERR_INVALID, "sim_create: bad argument");
  ON_DEVICE(beam, __func__);
  if (scheff && scheff->dev != beam->dev)
    return fail(HPS_ERR_INVALID, "sim_create: the beam and the SpaceCharge live on different devices");
  hps_sim_t s = new hps_sim_s();
  s->beam = beam; s->bl = bl; s->sc = scheff;
  s->sc_on = scheff != nullptr;
  s->prev_end = -1;
  cudaEventCreate(&s->ev0);
  cudaEventCreate(&s->ev1);
  hps_sim_reset(s);
  *out = s;
  return HPS_OK;
}

hps_status hps_sim_destroy(hps_sim_t s) {
  if (!s) return HPS_OK;
  // the beam may already be gone (a garbage collector finalises objects in
  // any order): wait for the device, not for the beam's stream
  cudaDeviceSynchronize();
  if (s->graph.exec) cudaGraphExecDestroy(s->graph.exec);
  if (s->graph.graph) cudaGraphDestroy(s->graph.graph);
  if (s->mon_dev) cudaFree(s->mon_dev);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  for (cudaEvent_t e : s->prof_pool) cudaEventDestroy(e);
  delete s;
  return HPS_OK;
}

// Reset, simulation_engine.cu:101-111
hps_status hps_sim_reset(hps_sim_t s) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  s->cur_id = 0;
  s->ccl_cell_num = 0;
  s->design_w = s->beam->design_w;
  s->wavelen = CLIGHT / s->beam->freq;
  return HPS_OK;
}

hps_status hps_sim_set_space_charge(hps_sim_t s, int on) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  s->sc_on = on != 0;
  return HPS_OK;
}

hps_status hps_sim_set_monitor(hps_sim_t s, double *host_out, uint32_t capacity) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  s->mon_host = host_out;
  s->mon_cap = host_out ? capacity : 0;
  return HPS_OK;
}

hps_status hps_sim_use_graph(hps_sim_t s, int on) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  s->use_graph = on != 0;
  return HPS_OK;
}

hps_status hps_sim_synchronize(hps_sim_t s) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  return sync(s->beam);
}

hps_status hps_sim_profile(hps_sim_t s, int on) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  s->prof_on = on != 0;
  return HPS_OK;
}

hps_status hps_sim_profile_read(hps_sim_t s, double *ms, uint64_t *count, int reset) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  for (int k = 0; k < HPS_NPROF; ++k) {
    if (ms) ms[k] = s->prof_ms[k];
    if (count) count[k] = s->prof_cnt[k];
    if (reset) { s->prof_ms[k] = 0.0; s->prof_cnt[k] = 0; }
  }
  return HPS_OK;
}

hps_status hps_sim_last_time_ms(hps_sim_t s, double *ms) {
  if (!s || !ms) return fail(HPS_ERR_INVALID, "bad argument");
  *ms = s->last_ms;
  return HPS_OK;
}

hps_status hps_sim_simulate(hps_sim_t s, int32_t start, int32_t end) {
  if (!s) return fail(HPS_ERR_INVALID, "bad sim handle");
  ON_DEVICE(s->beam, __func__);
  RunPlan p;
  hps_status e = plan_run(s, start, end, &p);
  if (e || p.empty) return e;
  hps_sim_t sim = s;
  Ctx &c = p.c;
  cudaStream_t st = c.b->stream;
  CK(cudaEventRecord(sim->ev0, st));
  if (p.graph) {
    e = prepare_graph(p);
    if (e) return e;
    CK(cudaGraphLaunch(sim->graph.exec, st));
  } else {
    for (int i = 0; i <= p.end_index; ++i) {
      if (i >= p.start_index || c.bl->types[i] == HPS_ELEM_SPCHCOMP) {
        sim->cur_id = (uint32_t)i;
        e = visit(c, (uint32_t)i);
        if (e) return e;
        if (p.monitor) monitor_at(c, (uint32_t)i);
        if (p.host_sync) {
          ScState h;
          CK(cudaMemcpyAsync(&h, c.sc->d, sizeof(h), cudaMemcpyDeviceToHost, st));
          CK(cudaStreamSynchronize(st));
          c.sc->interval = h.interval;
          c.sc->nx = h.nx;
          c.sc->nz = h.nz;
        }
      }
    }
  }
  CK(cudaEventRecord(sim->ev1, st));
  e = last_launch_status("simulate");
  if (e) return e;
  if (p.monitor) {
    CK(cudaMemcpyAsync(sim->mon_host, sim->mon_dev, (size_t)p.n * HPS_NMON * sizeof(double), cudaMemcpyDeviceToHost,
                       st));
  }
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, sim->ev0, sim->ev1);
  sim->last_ms = ms;
  for (size_t k = 0; k < sim->prof_used; ++k) {
    float pm = 0.f;
    cudaEventElapsedTime(&pm, sim->prof_pool[2 * k], sim->prof_pool[2 * k + 1]);
    sim->prof_ms[sim->prof_cls[k]] += pm;
    sim->prof_cnt[sim->prof_cls[k]] += 1;
  }
  sim->prof_used = 0;
  finish_monitor(p);
  return HPS_OK;
}


// ---- batches of independent simulators ----------------------------------------
hps_status hps_batch_create(const hps_sim_t *sims, uint32_t count, hps_batch_t *out) {
  if (!sims || !count || !out) return fail(HPS_ERR_INVALID, "batch_create: bad argument");
  std::vector<hps_sim_t> v(sims, sims + count);
  for (uint32_t i = 0; i < count; ++i) {
    if (!v[i]) return fail(HPS_ERR_INVALID, "batch_create: null simulator");
    for (uint32_t j = 0; j < i; ++j) {
      if (v[j] == v[i] || v[j]->beam == v[i]->beam)
        return fail(HPS_ERR_INVALID, "batch_create: every simulator of a batch needs its own beam");
      if (v[i]->sc && v[j]->sc == v[i]->sc)
        return fail(HPS_ERR_INVALID, "batch_create: every simulator of a batch needs its own SpaceCharge");
    }
    if (v[i]->beam->dev != v[0]->beam->dev)
      return fail(HPS_ERR_INVALID, "batch_create: the simulators live on different devices");
  }
  ON_DEVICE(v[0]->beam, __func__);  // the batch's streams and events are made on it
  hps_batch_t bt = new hps_batch_s();
  bt->sims = v;
  if (cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&bt->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->segfork.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->segfork.ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&bt->ev0) != cudaSuccess || cudaEventCreate(&bt->ev1) != cudaSuccess) {
    hps_batch_destroy(bt);
    return fail(HPS_ERR_CUDA, "batch_create: stream or events");
  }
  *out = bt;
  return HPS_OK;
}

hps_status hps_batch_destroy(hps_batch_t bt) {
  if (!bt) return HPS_OK;
  if (bt->stream) cudaStreamSynchronize(bt->stream);
  if (bt->exec) cudaGraphExecDestroy(bt->exec);
  if (bt->ls_exec) cudaGraphExecDestroy(bt->ls_exec);
  if (bt->segfork.ev_fork) cudaEventDestroy(bt->segfork.ev_fork);
  if (bt->segfork.ev_join) cudaEventDestroy(bt->segfork.ev_join);
  if (bt->side) cudaStreamDestroy(bt->side);
  if (bt->ev0) cudaEventDestroy(bt->ev0);
  if (bt->ev1) cudaEventDestroy(bt->ev1);
  if (bt->stream) cudaStreamDestroy(bt->stream);
  delete bt;
  return HPS_OK;
}

}  // extern "C"

namespace {

// The batch's range in lockstep (lockstep.cuh): the cached graph when every
// simulator's plan matches, else each simulator's range recorded (its launches
// handed to the recorder; a stray launch is swallowed by a throw-away stream
// capture and makes the batch fall back), the records merged into one
// captured graph.  *ran = false: the range has a launch without a lockstep
// form (every simulator's host state is put back).  Nothing is launched.
hps_status lockstep_prepare(hps_batch_t bt, std::vector<RunPlan> &plans, bool *ran) {
  const size_t m = bt->sims.size();
  *ran = false;
  uint64_t key = 0x6c6f636b73746570ull;
  for (const RunPlan &p : plans) key = mix(key, p.key);
  if (bt->ls_exec && key == bt->ls_key) {
    for (size_t k = 0; k < m; ++k) host_put(bt->sims[k], bt->ls_after[k]);
    note_launch((int)bt->ls_nodes);
    *ran = true;
    return HPS_OK;
  }
  std::vector<HostState> before(m);
  for (size_t k = 0; k < m; ++k) before[k] = host_get(bt->sims[k]);
  std::vector<Recorder> recs(m);
  std::string why;
  for (size_t k = 0; k < m && why.empty(); ++k) {
    const RunPlan &p = plans[k];
    cudaStream_t st = bt->sims[k]->beam->stream;
    recorder() = &recs[k];
    const cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    hps_status e = HPS_OK;
    if (ce == cudaSuccess) {
      RunPlan q = p;
      e = run_range(q.c, q.start_index, q.end_index, false);
    }
    cudaGraph_t junk = nullptr;
    const cudaError_t ee = ce == cudaSuccess ? cudaStreamEndCapture(st, &junk) : ce;
    size_t stray = 0;  // work that went to the stream instead of the recorder
    if (junk) {
      cudaGraphGetNodes(junk, nullptr, &stray);
      cudaGraphDestroy(junk);
    }
    recorder() = nullptr;
    cudaGetLastError();
    if (e || ce != cudaSuccess || ee != cudaSuccess) why = "recording the range failed";
    else if (!recs[k].unsupported.empty()) why = recs[k].unsupported;
    else if (stray) why = "a launch or copy without a lockstep form";
  }
  for (size_t k = 1; k < m && why.empty(); ++k) {
    if (recs[k].recs.size() != recs[0].recs.size()) { why = "the simulators' launch sequences differ"; break; }
    for (size_t j = 0; j < recs[0].recs.size(); ++j)
      if (recs[k].recs[j].merge != recs[0].recs[j].merge || recs[k].recs[j].p.size() != recs[0].recs[j].p.size() ||
          recs[k].recs[j].shape != recs[0].recs[j].shape) {
        why = "the simulators' launch sequences differ";
        break;
      }
  }
  if (recs.empty() || recs[0].recs.empty()) why = why.empty() ? "nothing to launch" : why;
  if (!why.empty()) {
    for (size_t k = 0; k < m; ++k) host_put(bt->sims[k], before[k]);
    bt->ls_why = why;
    return HPS_OK;
  }
  std::vector<HostState> after(m);
  for (size_t k = 0; k < m; ++k) after[k] = host_get(bt->sims[k]);
  SegFork &a = bt->segfork;
  auto merge_all = [&]() {
    std::vector<const Rec *> v(m);
    for (size_t j = 0; j < recs[0].recs.size(); ++j) {
      for (size_t k = 0; k < m; ++k) v[k] = &recs[k].recs[j];
      v[0]->merge(v, a, bt->stream, bt->side);
    }
  };
  // nothing runs when the merged graph cannot be built: the simulators keep
  // the host state they had before the range
  auto undo = [&](const char *what, cudaError_t err) {
    for (size_t k = 0; k < m; ++k) host_put(bt->sims[k], before[k]);
    return fail(HPS_ERR_CUDA, std::string(what) + cudaGetErrorString(err));
  };
  cudaGraph_t gr = nullptr;
  const cudaError_t be = cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal);
  if (be != cudaSuccess) return undo("lockstep capture: ", be);
  merge_all();
  const cudaError_t ce = cudaStreamEndCapture(bt->stream, &gr);
  if (ce != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    return undo("lockstep capture: ", ce);
  }
  size_t nodes = 0;
  cudaGraphGetNodes(gr, nullptr, &nodes);
  cudaGraphExec_t ex = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&ex, gr, 0);
  cudaGraphDestroy(gr);
  if (ie != cudaSuccess) return undo("lockstep instantiate: ", ie);
  if (bt->ls_exec) cudaGraphExecDestroy(bt->ls_exec);
  bt->ls_exec = ex;
  bt->ls_key = key;
  bt->ls_nodes = nodes;
  bt->ls_after = after;
  note_launch((int)nodes);
  *ran = true;
  return HPS_OK;
}

}  // namespace

extern "C" {

hps_status hps_batch_set_lockstep(hps_batch_t bt, int on) {
  if (!bt) return fail(HPS_ERR_INVALID, "bad batch handle");
  bt->lockstep = on != 0;
  return HPS_OK;
}

hps_status hps_batch_last_mode(hps_batch_t bt, int *lockstep, char *why, size_t why_cap) {
  if (!bt || !lockstep) return fail(HPS_ERR_INVALID, "bad argument");
  *lockstep = bt->last_mode;
  if (why && why_cap) {
    std::strncpy(why, bt->last_mode ? "" : bt->ls_why.c_str(), why_cap - 1);
    why[why_cap - 1] = 0;
  }
  return HPS_OK;
}

// Simulator::Simulate(start, end) on every simulator of the batch in one
// graph launch: the lockstep graph when the batch is in lockstep and its
// launches merge, else a parent graph of the simulators' captured ranges.
// Each simulator must be able to run as a graph (graphs on, profiling off,
// no mesh-size cut-off energy).
hps_status hps_batch_simulate(hps_batch_t bt, int32_t start, int32_t end) {
  if (!bt) return fail(HPS_ERR_INVALID, "bad batch handle");
  ON_DEVICE(bt->sims[0]->beam, __func__);
  const size_t m = bt->sims.size();
  std::vector<RunPlan> plans(m);
  for (size_t k = 0; k < m; ++k) {
    CK(cudaStreamSynchronize(bt->sims[k]->beam->stream));  // the beam's own work first
    hps_status e = plan_run(bt->sims[k], start, end, &plans[k]);
    if (e) return e;
    if (!plans[k].empty && !plans[k].graph)
      return fail(HPS_ERR_STATE, "batch_simulate: a simulator cannot run as a graph (graphs off, profiling on, "
                                 "or a mesh-size cut-off energy)");
  }
  bool ls = bt->lockstep && m > 1;
  for (const RunPlan &p : plans)
    if (p.empty || p.monitor) ls = false;
  if (!ls) bt->ls_why = bt->lockstep ? "a simulator records monitors or has an empty range, or one simulator"
                                     : "lockstep switched off";
  bt->last_mode = 0;
  if (ls) {
    bool ran = false;
    hps_status e = lockstep_prepare(bt, plans, &ran);
    if (e) return e;
    if (ran) {
      CK(cudaEventRecord(bt->ev0, bt->stream));
      CK(cudaGraphLaunch(bt->ls_exec, bt->stream));
      CK(cudaEventRecord(bt->ev1, bt->stream));
      e = last_launch_status("batch_simulate");
      if (e) return e;
      CK(cudaStreamSynchronize(bt->stream));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, bt->ev0, bt->ev1);
      bt->last_ms = ms;
      for (size_t k = 0; k < m; ++k) bt->sims[k]->last_ms = ms;
      bt->last_mode = 1;
      return HPS_OK;
    }
  }
  // nothing runs when the batch graph cannot be built: every simulator
  // keeps the host state it had before the range
  std::vector<HostState> before(m);
  for (size_t k = 0; k < m; ++k) before[k] = host_get(bt->sims[k]);
  auto undo = [&](hps_status e) {
    for (size_t k = 0; k < m; ++k) host_put(bt->sims[k], before[k]);
    return e;
  };
  std::vector<uint64_t> serials(m, 0);
  for (size_t k = 0; k < m; ++k) {
    if (plans[k].empty) continue;
    hps_status e = prepare_graph(plans[k]);
    if (e) return undo(e);
    serials[k] = bt->sims[k]->graph.serial;
  }
  if (!bt->exec || serials != bt->serials) {
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    bt->exec = nullptr;
    cudaGraph_t parent;
    const cudaError_t ge = cudaGraphCreate(&parent, 0);
    if (ge != cudaSuccess) return undo(fail(HPS_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(ge)));
    for (size_t k = 0; k < m; ++k) {
      if (plans[k].empty) continue;
      cudaGraphNode_t node;
      cudaError_t ce = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, bt->sims[k]->graph.graph);
      if (ce != cudaSuccess) {
        cudaGraphDestroy(parent);
        return undo(fail(HPS_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(ce)));
      }
    }
    cudaError_t ie = cudaGraphInstantiate(&bt->exec, parent, 0);
    cudaGraphDestroy(parent);
    if (ie != cudaSuccess) {
      bt->exec = nullptr;
      return undo(fail(HPS_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(ie)));
    }
    bt->serials = serials;
  }
  CK(cudaEventRecord(bt->ev0, bt->stream));
  CK(cudaGraphLaunch(bt->exec, bt->stream));
  CK(cudaEventRecord(bt->ev1, bt->stream));
  for (size_t k = 0; k < m; ++k) {
    const RunPlan &p = plans[k];
    if (p.empty || !p.monitor) continue;
    hps_sim_t s = bt->sims[k];
    CK(cudaMemcpyAsync(s->mon_host, s->mon_dev, (size_t)p.n * HPS_NMON * sizeof(double), cudaMemcpyDeviceToHost,
                       bt->stream));
  }
  hps_status e = last_launch_status("batch_simulate");
  if (e) return e;
  CK(cudaStreamSynchronize(bt->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, bt->ev0, bt->ev1);
  bt->last_ms = ms;
  for (size_t k = 0; k < m; ++k) {
    if (plans[k].empty) continue;
    bt->sims[k]->last_ms = ms;
    finish_monitor(plans[k]);
  }
  return HPS_OK;
}

hps_status hps_batch_last_time_ms(hps_batch_t bt, double *ms) {
  if (!bt || !ms) return fail(HPS_ERR_INVALID, "bad argument");
  *ms = bt->last_ms;
  return HPS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
namespace {

// A simulator's state before tuning: the beam on the device, its host-side
// fields, the solver's device state and the engine's host state, so that
// every trial starts from the same point and tuning leaves no trace.
struct Snapshot {
  hps_sim_t s = nullptr;
  void *dev[8] = {};
  BeamStats st{};
  ScState sc{};
  double b_design_w = 0, b_freq = 0, b_current = 0, phi_ref = 0, w_ref = 0;
  double design_w = 0, wavelen = 0, fraction = 0, interval = 0;
  uint32_t cur_id = 0, ccl = 0;
  int prev_end = -1;
};

void snap_free(Snapshot &z) {
  for (void *&p : z.dev)
    if (p) { cudaFree(p); p = nullptr; }
}

hps_status snap_take(hps_sim_t s, Snapshot &z) {
  hps_beam_t b = s->beam;
  z.s = s;
  const size_t nd = (size_t)b->n * esize(b), nu = (size_t)b->n * 4;
  for (int k = 0; k < 8; ++k) {
    const size_t bytes = k < 6 ? nd : nu;
    CK(cudaMalloc(&z.dev[k], bytes ? bytes : 1));
    const void *src = k < 6 ? coord_ptr(b, k) : (k == 6 ? (void *)b->d.loss : (void *)b->d.lloss);
    CK(cudaMemcpyAsync(z.dev[k], src, bytes, cudaMemcpyDeviceToDevice, b->stream));
  }
  CK(cudaMemcpyAsync(&z.st, b->d.st, sizeof(BeamStats), cudaMemcpyDeviceToHost, b->stream));
  if (s->sc) CK(cudaMemcpyAsync(&z.sc, s->sc->d, sizeof(ScState), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  z.b_design_w = b->design_w; z.b_freq = b->freq; z.b_current = b->current;
  z.phi_ref = b->d.phi_ref; z.w_ref = b->d.w_ref;
  z.design_w = s->design_w; z.wavelen = s->wavelen; z.cur_id = s->cur_id; z.ccl = s->ccl_cell_num;
  z.prev_end = s->prev_end;
  if (s->sc) { z.fraction = s->sc->fraction; z.interval = s->sc->interval; }
  return HPS_OK;
}

hps_status snap_put(const Snapshot &z) {
  hps_sim_t s = z.s;
  hps_beam_t b = s->beam;
  const size_t nd = (size_t)b->n * esize(b), nu = (size_t)b->n * 4;
  for (int k = 0; k < 8; ++k) {
    void *dst = k < 6 ? coord_ptr(b, k) : (k == 6 ? (void *)b->d.loss : (void *)b->d.lloss);
    CK(cudaMemcpyAsync(dst, z.dev[k], k < 6 ? nd : nu, cudaMemcpyDeviceToDevice, b->stream));
  }
  CK(cudaMemcpyAsync(b->d.st, &z.st, sizeof(BeamStats), cudaMemcpyHostToDevice, b->stream));
  if (s->sc) CK(cudaMemcpyAsync(s->sc->d, &z.sc, sizeof(ScState), cudaMemcpyHostToDevice, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  b->design_w = z.b_design_w; b->freq = z.b_freq; b->current = z.b_current;
  b->d.phi_ref = z.phi_ref; b->d.w_ref = z.w_ref;
  s->design_w = z.design_w; s->wavelen = z.wavelen; s->cur_id = z.cur_id; s->ccl_cell_num = z.ccl;
  s->prev_end = z.prev_end;
  if (s->sc) { s->sc->fraction = z.fraction; s->sc->interval = z.interval; }
  return HPS_OK;
}

// one launch shape: contraction kernel of FP32 beams (solver parameter 10),
// deposit blocks per SM, sweep blocks per SM (0: all the SM holds), the
// deposit's warp-aggregated histogram adds, the deposit's threads per block
struct Shape {
  int contraction;
  uint32_t dep_per_sm, sweep_cap, dep_agg, dep_threads;
};

hps_status shape_apply(hps_sim_t s, const Shape &sh) {
  s->dep_per_sm = sh.dep_per_sm;
  s->sweep_cap = sh.sweep_cap;
  s->dep_agg = sh.dep_agg;
  s->dep_threads = sh.dep_threads;
  if (s->sc && s->sc->contraction != sh.contraction) {
    hps_status e = hps_scheff_set(s->sc, 10, (double)sh.contraction);
    if (e) return e;
  }
  return HPS_OK;
}

std::mutex g_tune_mutex;
std::map<std::string, Shape> g_tune_cache;

// the cache key: device, mesh, particle count (power-of-two bucket), precision
std::string tune_key(hps_sim_t s, const char *what) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp pr{};
  cudaGetDeviceProperties(&pr, dev);
  uint32_t bucket = 0;
  while ((1u << bucket) < s->beam->n && bucket < 31) ++bucket;
  char buf[512];
  std::snprintf(buf, sizeof buf, "%s|%d|%s|%u|%u|%u|%d", what, dev, pr.name, s->sc ? s->sc->nx_max : 0u,
                s->sc ? s->sc->nz_max : 0u, bucket, s->beam->prec);
  return buf;
}

// The search: coordinate descent over the four knobs (contraction kernel,
// then deposit blocks per SM, then sweep blocks per SM, then aggregated
// deposit adds), each candidate
// timed as the median of `reps` runs after one untimed run (which captures
// its graph), every run from the snapshot.  run() simulates and returns the
// device time in ms.
template <class Run, class Restore>
hps_status tune_search(const std::vector<hps_sim_t> &sims, bool fp32, bool tc_ok, int reps, Run run,
                       Restore restore, Shape *best_out, std::vector<double> *times) {
  Shape best{sims[0]->sc ? sims[0]->sc->contraction : 0, sims[0]->dep_per_sm, sims[0]->sweep_cap,
             sims[0]->dep_agg, sims[0]->dep_threads};
  if (!fp32) { *best_out = best; return HPS_OK; }
  auto measure = [&](const Shape &sh, double *ms) -> hps_status {
    for (hps_sim_t s : sims) {
      hps_status e = shape_apply(s, sh);
      if (e) return e;
    }
    std::vector<double> v;
    for (int r = 0; r <= reps; ++r) {
      hps_status e = restore();
      if (e) return e;
      double t = 0.0;
      e = run(&t);
      if (e) return e;
      if (r > 0) v.push_back(t);
    }
    std::sort(v.begin(), v.end());
    *ms = v[v.size() / 2];
    if (times) times->push_back(*ms);
    return HPS_OK;
  };
  double best_ms = 0.0;
  hps_status e = measure(best, &best_ms);
  if (e) return e;
  std::vector<Shape> cands;
  if (tc_ok) cands.push_back({1 - best.contraction, best.dep_per_sm, best.sweep_cap, best.dep_agg, best.dep_threads});
  for (int stage = 0; stage < 4; ++stage) {
    if (stage == 1) {
      // the deposit's grid: blocks of 256, 512 or 1024 threads, blocks per
      // SM within the 1024 threads an SM holds at 64 registers a thread
      const uint32_t grids[6][2] = {{256, 2}, {256, 3}, {256, 4}, {512, 1}, {512, 2}, {1024, 1}};
      for (const auto &g : grids)
        if (g[0] != best.dep_threads || g[1] != best.dep_per_sm)
          cands.push_back({best.contraction, g[1], best.sweep_cap, best.dep_agg, g[0]});
    } else if (stage == 2) {
      for (uint32_t c : {0u, 2u})
        if (c != best.sweep_cap)
          cands.push_back({best.contraction, best.dep_per_sm, c, best.dep_agg, best.dep_threads});
    } else if (stage == 3) {
      cands.push_back({best.contraction, best.dep_per_sm, best.sweep_cap, 1u - best.dep_agg, best.dep_threads});
    }
    for (const Shape &sh : cands) {
      double ms = 0.0;
      if ((e = measure(sh, &ms))) return e;
      if (ms < best_ms) { best_ms = ms; best = sh; }
    }
    cands.clear();
  }
  *best_out = best;
  return HPS_OK;
}

void report(const Shape &b, const std::vector<double> &t, int32_t *shape_out, double *ms_out, uint32_t ms_cap,
            uint32_t *n_out) {
  if (shape_out) {
    shape_out[0] = b.contraction;
    shape_out[1] = (int32_t)b.dep_per_sm;
    shape_out[2] = (int32_t)b.sweep_cap;
    shape_out[3] = (int32_t)b.dep_agg;
    shape_out[4] = (int32_t)b.dep_threads;
  }
  if (ms_out)
    for (size_t k = 0; k < t.size() && k < ms_cap; ++k) ms_out[k] = t[k];
  if (n_out) *n_out = (uint32_t)t.size();
}

}  // namespace

extern "C" {

hps_status hps_sim_autotune(hps_sim_t s, int32_t start, int32_t end, int32_t reps, int32_t *shape_out, double *ms_out,
                            uint32_t ms_cap, uint32_t *n_timed) {
  if (!s || reps < 1 || reps > 64) return fail(HPS_ERR_INVALID, "sim_autotune: bad argument");
  ON_DEVICE(s->beam, __func__);
  const std::string key = tune_key(s, "sim");
  std::vector<double> times;
  Shape best{};
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      hps_status e = shape_apply(s, it->second);
      if (e) return e;
      report(it->second, times, shape_out, ms_out, ms_cap, n_timed);
      return HPS_OK;
    }
  }
  Snapshot z;
  hps_status e = snap_take(s, z);
  if (e) { snap_free(z); return e; }
  const bool fp32 = f32(s->beam) && s->sc && s->sc_on;
  const bool tc_ok = fp32 && sc32_tc_mesh(s->sc->nx_max, s->sc->nz_max);
  auto run = [&](double *ms) -> hps_status {
    hps_status r = hps_sim_simulate(s, start, end);
    if (r) return r;
    *ms = s->last_ms;
    return HPS_OK;
  };
  auto restore = [&]() { return snap_put(z); };
  e = tune_search({s}, fp32, tc_ok, reps, run, restore, &best, &times);
  if (!e) e = shape_apply(s, best);
  if (!e) e = snap_put(z);
  snap_free(z);
  if (e) return e;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = best;
  }
  report(best, times, shape_out, ms_out, ms_cap, n_timed);
  return HPS_OK;
}

hps_status hps_batch_autotune(hps_batch_t bt, int32_t start, int32_t end, int32_t reps, int32_t *shape_out,
                              double *ms_out, uint32_t ms_cap, uint32_t *n_timed) {
  if (!bt || bt->sims.empty() || reps < 1 || reps > 64) return fail(HPS_ERR_INVALID, "batch_autotune: bad argument");
  ON_DEVICE(bt->sims[0]->beam, __func__);
  const std::string key = tune_key(bt->sims[0], bt->lockstep ? "batch-lockstep" : "batch") + "|" +
                          std::to_string(bt->sims.size());
  std::vector<double> times;
  Shape best{};
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      for (hps_sim_t s : bt->sims) {
        hps_status e = shape_apply(s, it->second);
        if (e) return e;
      }
      report(it->second, times, shape_out, ms_out, ms_cap, n_timed);
      return HPS_OK;
    }
  }
  std::vector<Snapshot> zs(bt->sims.size());
  hps_status e = HPS_OK;
  for (size_t k = 0; k < zs.size() && !e; ++k) e = snap_take(bt->sims[k], zs[k]);
  bool fp32 = true, tc_ok = true;
  for (hps_sim_t s : bt->sims) {
    fp32 = fp32 && f32(s->beam) && s->sc && s->sc_on;
    tc_ok = tc_ok && s->sc && sc32_tc_mesh(s->sc->nx_max, s->sc->nz_max);
  }
  auto run = [&](double *ms) -> hps_status {
    hps_status r = hps_batch_simulate(bt, start, end);
    if (r) return r;
    *ms = bt->last_ms;
    return HPS_OK;
  };
  auto restore = [&]() -> hps_status {
    for (const Snapshot &z : zs) {
      hps_status r = snap_put(z);
      if (r) return r;
    }
    return HPS_OK;
  };
  if (!e) e = tune_search(bt->sims, fp32, fp32 && tc_ok, reps, run, restore, &best, &times);
  for (hps_sim_t s : bt->sims)
    if (!e) e = shape_apply(s, best);
  if (!e) e = restore();
  for (Snapshot &z : zs) snap_free(z);
  if (e) return e;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = best;
  }
  report(best, times, shape_out, ms_out, ms_cap, n_timed);
  return HPS_OK;
}

hps_status hps_sim_get_shape(hps_sim_t s, int32_t *shape_out) {
  if (!s || !shape_out) return fail(HPS_ERR_INVALID, "sim_get_shape: bad argument");
  shape_out[0] = s->sc ? s->sc->contraction : 0;
  shape_out[1] = (int32_t)s->dep_per_sm;
  shape_out[2] = (int32_t)s->sweep_cap;
  shape_out[3] = (int32_t)s->dep_agg;
  shape_out[4] = (int32_t)s->dep_threads;
  return HPS_OK;
}

hps_status hps_sim_set_shape(hps_sim_t s, const int32_t *shape) {
  if (!s || !shape || shape[0] < 0 || shape[0] > 1 || shape[1] < 1 || shape[1] > 8 || shape[2] < 0 || shape[2] > 16 ||
      shape[3] < 0 || shape[3] > 1 || (shape[4] != 0 && shape[4] != 256 && shape[4] != 512 && shape[4] != 1024))
    return fail(HPS_ERR_INVALID, "sim_set_shape: bad argument");
  return shape_apply(s, Shape{shape[0], (uint32_t)shape[1], (uint32_t)shape[2], (uint32_t)shape[3],
                              shape[4] ? (uint32_t)shape[4] : 256u});
}

}  // extern "C"
