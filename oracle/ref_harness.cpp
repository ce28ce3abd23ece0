// ref_harness.cpp -- runs the reference's own tracking code on the host CPU.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/ when
// the reference tree is present, never shipped.  It pins the FP64
// restatement in hps_oracle.c to the reference implementation:
//
//  * the reference's device code -- simulation_kernel.cu, space_charge_kernel.cu,
//    beam_kernel.cu -- is #included here and compiled by the host compiler
//    (CUDA's headers turn __global__/__device__/__constant__ into nothing for
//    a non-CUDA compiler);
//  * the reference's host classes -- beam.cpp, space_charge.cpp,
//    simulation_engine.cpp, beamline*.cpp, utility.cpp, py_wrapper.cpp -- are
//    compiled unmodified from their own files;
//  * what cannot run without a GPU is supplied here: a CUDA runtime over host
//    memory, and the three launcher files (beam.cu, space_charge.cu,
//    simulation_engine.cu) restated with every <<<grid, block>>> launch
//    executed block by block, thread by thread, on one host thread.
//    The cudaEvent timer around Simulate is replaced by a silent one.
//    Reductions whose kernels synchronise threads are launched with one block
//    of one thread (the kernels' block_size = 1 instantiation), which sums in
//    a different order than the GPU but with the reference's own code.
//
// Build: -DDOUBLE_PRECISION (the reference's FP64 build), -std=c++14.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime_api.h>

// ---------------------------------------------------------------------------
// launch-index state and device intrinsics used by the reference kernels
// ---------------------------------------------------------------------------
namespace hps_emul {
struct idx3 { unsigned int x, y, z; };
idx3 thread_idx, block_idx, block_dim, grid_dim;
}  // namespace hps_emul
#define threadIdx hps_emul::thread_idx
#define blockIdx hps_emul::block_idx
#define blockDim hps_emul::block_dim
#define gridDim hps_emul::grid_dim

static inline double rsqrt(double v) { return 1.0 / std::sqrt(v); }
static inline void __syncthreads() {}
static inline float atomicAdd(float *a, float v) { float o = *a; *a = o + v; return o; }
static inline unsigned int atomicAdd(unsigned int *a, int v) { unsigned int o = *a; *a = o + v; return o; }
static inline unsigned long long atomicCAS(unsigned long long *a, unsigned long long cmp,
                                           unsigned long long v) {
  unsigned long long o = *a;
  if (o == cmp) *a = v;
  return o;
}
static inline long long __double_as_longlong(double d) { long long r; std::memcpy(&r, &d, 8); return r; }
static inline double __longlong_as_double(long long v) { double r; std::memcpy(&r, &v, 8); return r; }
using std::abs;

// shared-memory backing for SharedMemory<T> and the float contraction kernel
int __smem[1 << 14];
double __smem_d[1 << 14];
float bin_smem[1 << 16];

#include "beam.h"
#include "beamline.h"
#include "simulation_kernel.cu"
#include "space_charge_kernel.cu"
#include "beam_kernel.cu"

#include "beamline.h"
#include "beam_cu.h"
#include "simulation_engine.h"
#include "simulation_engine_cu.h"
#include "space_charge.h"
#include "space_charge_cu.h"
#include "utility.h"
#include "timer.h"

// ---------------------------------------------------------------------------
// launch emulation: every block, every thread, in order
// ---------------------------------------------------------------------------
template <typename F, typename... A>
static void launch(dim3 g, dim3 b, F f, A... a) {
  if (g.x == 0 || g.y == 0 || b.x == 0 || b.y == 0) return;  // invalid launch: nothing runs
  hps_emul::grid_dim = {g.x, g.y, 1};
  hps_emul::block_dim = {b.x, b.y, 1};
  for (unsigned by = 0; by < g.y; ++by)
    for (unsigned bx = 0; bx < g.x; ++bx)
      for (unsigned ty = 0; ty < b.y; ++ty)
        for (unsigned tx = 0; tx < b.x; ++tx) {
          hps_emul::block_idx = {bx, by, 0};
          hps_emul::thread_idx = {tx, ty, 0};
          f(a...);
        }
}
template <typename F, typename... A>
static void launch1(F f, A... a) { launch(dim3(1), dim3(1), f, a...); }

// ---------------------------------------------------------------------------
// CUDA runtime over host memory.  Allocations come from a bump arena so that
// successive allocations have increasing addresses, as cudaMalloc gives for
// the reference's small scalar buffers (the mesh-size launcher compares two
// such pointers).
// ---------------------------------------------------------------------------
static std::map<void *, size_t> g_big;
static char *g_arena = nullptr;
static size_t g_arena_used = 0;
static const size_t kArena = size_t(64) << 20;

extern "C" {
cudaError_t cudaMalloc(void **p, size_t sz) {
  if (!g_arena) g_arena = (char *)std::calloc(1, kArena);
  size_t a = (sz + 255) & ~size_t(255);
  if (sz <= 4096 && g_arena_used + a <= kArena) {
    *p = g_arena + g_arena_used;
    g_arena_used += a;
    return cudaSuccess;
  }
  *p = std::calloc(1, sz ? sz : 1);
  g_big[*p] = sz;
  return cudaSuccess;
}
cudaError_t cudaFree(void *p) {
  auto it = g_big.find(p);
  if (it != g_big.end()) { std::free(p); g_big.erase(it); }
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { std::memmove(d, s, n); return cudaSuccess; }
cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind, cudaStream_t) {
  std::memmove(d, s, n);
  return cudaSuccess;
}
cudaError_t cudaMemset(void *d, int v, size_t n) { std::memset(d, v, n); return cudaSuccess; }
cudaError_t cudaHostAlloc(void **p, size_t sz, unsigned int) { *p = std::calloc(1, sz); return cudaSuccess; }
cudaError_t cudaHostGetDevicePointer(void **d, void *h, unsigned int) { *d = h; return cudaSuccess; }
cudaError_t cudaFreeHost(void *p) { std::free(p); return cudaSuccess; }
cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = nullptr; return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) { *ms = 0.f; return cudaSuccess; }
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaStreamCreate(cudaStream_t *s) { *s = nullptr; return cudaSuccess; }
cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
}

// timer.h replacements (the reference's timer prints every Simulate call)
void StartTimer(cudaEvent_t *, cudaEvent_t *) {}
void StopTimer(cudaEvent_t *, cudaEvent_t *, std::string) {}

// ---------------------------------------------------------------------------
// beam.cu launchers (reference: src/beam/src/beam.cu)
// ---------------------------------------------------------------------------
template <typename T>
static void dalloc(T **p, size_t n) { cudaMalloc((void **)p, n * sizeof(T)); std::memset(*p, 0, n * sizeof(T)); }

void CreateBeamOnDevice(Beam *b) {
  uint n = b->num_particle;
  dalloc(&b->x, n); dalloc(&b->y, n); dalloc(&b->phi, n); dalloc(&b->phi_r, n);
  dalloc(&b->xp, n); dalloc(&b->yp, n); dalloc(&b->w, n);
  dalloc(&b->loss, n); dalloc(&b->lloss, n);
  double **s[] = {&b->x_avg, &b->x_avg_good, &b->xp_avg, &b->y_avg, &b->y_avg_good, &b->yp_avg,
                  &b->phi_avg, &b->phi_avg_r, &b->phi_avg_good, &b->w_avg, &b->w_avg_good,
                  &b->x_sig, &b->x_sig_good, &b->xp_sig, &b->y_sig, &b->y_sig_good, &b->yp_sig,
                  &b->phi_sig, &b->phi_sig_r, &b->phi_sig_good, &b->w_sig, &b->w_sig_good,
                  &b->x_emit, &b->x_emit_good, &b->y_emit, &b->y_emit_good, &b->z_emit,
                  &b->z_emit_good, &b->r_max, &b->abs_phi_max};
  for (double **q : s) dalloc(q, 1);
  dalloc(&b->num_loss, 1); dalloc(&b->num_lloss, 1); dalloc(&b->num_good, 1);
}
void CreatePartialsOnDevice(Beam *b, uint g, uint) {
  dalloc(&b->partial_int1, g + 1);
  dalloc(&b->partial_double2, (g + 1) * 2);
  dalloc(&b->partial_double3, (g + 1) * 3);
}
void FreePartialsOnDevice(Beam *b) { cudaFree(b->partial_int1); cudaFree(b->partial_double2); cudaFree(b->partial_double3); }
void FreeBeamOnDevice(Beam *b) {
  cudaFree(b->x); cudaFree(b->y); cudaFree(b->phi); cudaFree(b->phi_r); cudaFree(b->xp);
  cudaFree(b->yp); cudaFree(b->w); cudaFree(b->loss); cudaFree(b->lloss);
  FreePartialsOnDevice(b);
}
void UpdateBeamOnDevice(Beam *b, double *x, double *xp, double *y, double *yp, double *phi,
                        double *w, uint *loss, uint *lloss) {
  size_t n = b->num_particle;
  std::memcpy(b->x, x, n * 8); std::memcpy(b->xp, xp, n * 8); std::memcpy(b->y, y, n * 8);
  std::memcpy(b->yp, yp, n * 8); std::memcpy(b->phi, phi, n * 8); std::memcpy(b->w, w, n * 8);
  if (loss) std::memcpy(b->loss, loss, n * 4); else std::memset(b->loss, 0, n * 4);
  if (lloss) std::memcpy(b->lloss, lloss, n * 4); else std::memset(b->lloss, 0, n * 4);
}
void CopyBeamFromDevice(Beam *b, double *x, double *xp, double *y, double *yp, double *phi,
                        double *w, uint *loss, uint *lloss, uint *nl) {
  size_t n = b->num_particle;
  std::memcpy(x, b->x, n * 8); std::memcpy(xp, b->xp, n * 8); std::memcpy(y, b->y, n * 8);
  std::memcpy(yp, b->yp, n * 8); std::memcpy(phi, b->phi, n * 8); std::memcpy(w, b->w, n * 8);
  std::memcpy(loss, b->loss, n * 4); std::memcpy(lloss, b->lloss, n * 4);
  *nl = *b->num_loss;
}
void CopyParticleFromDevice(Beam *b, uint i, double *x, double *xp, double *y, double *yp,
                            double *phi, double *w, uint *loss, uint *lloss) {
  *x = b->x[i]; *xp = b->xp[i]; *y = b->y[i]; *yp = b->yp[i]; *phi = b->phi[i]; *w = b->w[i];
  *loss = b->loss[i]; *lloss = b->lloss[i];
}
void UpdateLossCountKernelCall(Beam *b, bool ll) {
  uint *part = b->partial_int1;
  launch1(LossReduceKernel<1>, ll ? b->lloss : b->loss, part, b->num_particle, 1u);
  if (!ll) *b->num_loss = part[0]; else *b->num_lloss = part[0];
}
void UpdateGoodParticleCountKernelCall(Beam *b) {
  uint *part = b->partial_int1;
  launch1(GoodParticleCountReduceKernel<1>, b->loss, b->lloss, part, b->num_particle, 1u);
  *b->num_good = part[0];
}
void UpdateAvgOfOneVariableKernelCall(Beam *b, double *x, double *avg, bool good) {
  double *p = b->partial_double2;
  launch1(XReduceKernel<double, 1>, x, p, b->num_particle, b->loss, 1u, good ? b->lloss : (uint *)nullptr);
  if (!good) launch1(UpdateVariableAvgKernel, avg, p, b->num_particle, b->num_loss);
  else launch1(UpdateVariableAvgWithLlossKernel, avg, p, b->num_good);
}
void UpdateSigmaOfOneVariableKernelCall(Beam *b, double *x, double *sig, bool good) {
  double *p = b->partial_double2;
  launch1(XX2ReduceKernel<double, 1>, x, p, b->num_particle, b->loss, 1u, good ? b->lloss : (uint *)nullptr);
  if (!good) launch1(UpdateVariableSigmaKernel, sig, p, p + 1, b->num_particle, b->num_loss);
  else launch1(UpdateVariableSigmaWithLlossKernel, sig, p, p + 1, b->num_good);
}
void UpdateAvgXYKernelCall(Beam *b) {
  double *p1 = b->partial_double2, *p2 = b->partial_double3;
  launch1(XYReduceKernel<double, 1>, b->x, b->y, p1, p2, b->num_particle, b->loss, 1u);
  launch1(UpdateHorizontalAvgXYKernel, b->x_avg, b->y_avg, p1, p2, b->num_particle, b->num_loss);
}
void UpdateMaxRPhiKernelCall(Beam *b) {
  double *p1 = b->partial_double2, *p2 = b->partial_double3;
  launch1(MaxR2PhiReduceKernel<double, 1>, b->x, b->y, b->phi_r, b->loss, b->x_avg, b->y_avg,
          b->phi_avg_r, p1, p2, b->num_particle, 1u);
  launch1(UpdateMaxRPhiKernel, b->r_max, b->abs_phi_max, p1, p2);
}
void UpdateAvgSigXYKernelCall(Beam *b) {
  double *p1 = b->partial_double2, *p2 = b->partial_double3;
  launch1(XYX2Y2ReduceKernel<double, 1>, b->x, b->y, p1, p2, b->num_particle, b->loss, b->lloss, 1u);
  launch1(UpdateHorizontalAvgSigKernel, b->x_avg_good, b->x_sig_good, b->y_avg_good, b->y_sig_good,
          p1, p2, b->num_particle, b->num_loss);
}
static void emit_call(Beam *b, double *u, double *up, double *avg, double *sig, double *pavg,
                      double *psig, double *eps) {
  double *p1 = b->partial_double2, *p2 = b->partial_double3;
  launch1(EmittanceReduceKernel<double, 1>, u, up, p1, p2, b->num_particle, b->loss, 1u);
  launch1(UpdateTransverseEmittanceKernel, avg, sig, pavg, psig, eps, p1, p2, b->num_particle,
          b->num_loss, b->w, b->mass);
}
void UpdateHorizontalEmittanceKernelCall(Beam *b) {
  emit_call(b, b->x, b->xp, b->x_avg, b->x_sig, b->xp_avg, b->xp_sig, b->x_emit);
}
void UpdateVerticalEmittanceKernelCall(Beam *b) {
  emit_call(b, b->y, b->yp, b->y_avg, b->y_sig, b->yp_avg, b->yp_sig, b->y_emit);
}
void UpdateLongitudinalEmittanceKernelCall(Beam *b) {
  double *p1 = b->partial_double2, *p2 = b->partial_double3;
  launch1(EmittanceReduceKernel<double, 1>, b->phi_r, b->w, p1, p2, b->num_particle, b->loss, 1u);
  launch1(UpdateLongitudinalEmittanceKernel, b->phi_avg_r, b->phi_sig_r, b->w_avg, b->w_sig,
          b->z_emit, p1, p2, b->num_particle, b->num_loss);
}
void SetDoubleValue(double *arr, uint i, double v) { launch1(SetValueKernel<double>, arr, i, v); }
void ShiftVariableKernelCall(Beam *b, double *var, double v) {
  launch(dim3(b->grid_size), dim3(b->blck_size), ShiftVariableKernel<double>, var, v, b->num_particle);
}
void UpdateRelativePhiKernelCall(Beam *b, bool good) {
  launch(dim3(b->grid_size), dim3(b->blck_size), UpdateRelativePhiKernel, b->phi_r, b->phi,
         good ? b->phi_avg_good : b->phi, b->num_particle);
}
void CutBeamKernelCall(double *c, uint *loss, double lo, double hi, uint n, uint g, uint bk) {
  launch(dim3(g), dim3(bk), CutBeamKernel, c, loss, lo, hi, n);
}
void ChangeFrequnecyKernelCall(Beam *b, double r) {
  launch(dim3(b->grid_size), dim3(b->blck_size), ChangeFrequencyKernel, b->phi, r, b->num_particle);
}
void UpdateLongitudinalLossCoordinateKernelCall(Beam *b) {
  launch(dim3(b->grid_size), dim3(b->blck_size), UpdateLongitudinalLossCoordinateKernel, b->lloss,
         b->phi, b->phi_avg_good, b->num_particle);
}

// ---------------------------------------------------------------------------
// space_charge.cu launchers (reference: src/simulation/src/space_charge.cu)
// ---------------------------------------------------------------------------
namespace {
uint sc_nr, sc_nz;
Beam *sc_beam;
double sc_beta, sc_freq, sc_frac;
uint sc_adj;
// tables of the most recently initialised Scheff (table-level fixtures)
double2 *g_fld1, *g_fld2;
double *g_bin;
}  // namespace

void Initialize(SpaceChargeParam prm, double2 **f1, double2 **f2, double **bin) {
  sc_nr = prm.nx; sc_nz = prm.nz;
  d_scheff_param = prm;
  dalloc(bin, (size_t)sc_nr * sc_nz);
  dalloc(f1, (size_t)sc_nr * sc_nz * (sc_nr + 1));
  dalloc(f2, (size_t)(sc_nz + 1) * (sc_nr + 1));
  g_fld1 = *f1; g_fld2 = *f2; g_bin = *bin;
}
void FreeMeshTables(double2 *f1, double2 *f2, double *bin) { cudaFree(bin); cudaFree(f1); cudaFree(f2); }
void SetParameters(Beam *b, uint nr, uint nz, double frac, uint adj, double beta) {
  sc_beam = b; sc_freq = b->freq; sc_beta = beta; sc_frac = frac; sc_adj = adj; sc_nr = nr; sc_nz = nz;
}
void ResetBinTbl(double *bin) { std::memset(bin, 0, (size_t)sc_nr * sc_nz * sizeof(double)); }
void ResetFldTbl(double2 *f2) { std::memset(f2, 0, (size_t)(sc_nz + 1) * (sc_nr + 1) * sizeof(double2)); }
void UpdateMeshKernelCall() {
  if (sc_adj != 0) {
    sc_beam->UpdateMaxRPhi();
    launch1(UpdateScheffMeshSizeKernel, sc_beam->r_max, (double *)nullptr, sc_freq, sc_beta, 1.0);
  } else if (sc_beam->x_sig_good > sc_beam->y_sig_good) {
    launch1(UpdateScheffMeshSizeKernel, sc_beam->x_sig_good, sc_beam->phi_sig_good, sc_freq, sc_beta, 3.0);
  } else {
    launch1(UpdateScheffMeshSizeKernel, sc_beam->y_sig_good, sc_beam->phi_sig_good, sc_freq, sc_beta, 3.0);
  }
}
void UpdateTblsKernelCall(double2 *f1, double *bin) {
  uint bx = sc_nz;
  uint by = (512 / sc_nz < sc_nr) ? 512 / sc_nz : sc_nr;
  uint gx = sc_nr / by, gy = sc_nr + 1;
  launch(dim3(gx, gy), dim3(bx, by), UpdateFldTbl1Kernel, f1, sc_freq, sc_beta,
         sc_beam->num_particle, sc_beam->current * sc_frac / sc_beam->mass, sc_adj);
  launch1(InitNumOnMesh);
  launch(dim3(sc_beam->grid_size), dim3(sc_beam->blck_size / 4), DistributeParticleKernel, bin,
         sc_beam->x, sc_beam->y, sc_beam->phi_r, sc_beam->loss, sc_beam->lloss,
         sc_beam->x_avg_good, sc_beam->y_avg_good, sc_beam->phi_avg_r, sc_beam->x_sig_good,
         sc_beam->y_sig_good, sc_beam->num_particle, sc_beta, sc_freq);
}
void UpdateFinalFldTblKernelCall(double2 *f2, double *bin, double2 *f1) {
  launch(dim3(sc_nr + 2), dim3(1024), UpdateFldTbl2KernelDouble, f2, bin, f1);
}
void KickBeamKernelCall(double2 *f2, double len, double rr, double rz, double rq, double rg) {
  launch(dim3(sc_beam->grid_size), dim3(sc_beam->blck_size / 4), ApplySpchKickKernel, sc_beam->x,
         sc_beam->y, sc_beam->phi_r, sc_beam->xp, sc_beam->yp, sc_beam->w, sc_beam->loss,
         sc_beam->lloss, sc_beam->x_avg_good, sc_beam->y_avg_good, sc_beam->phi_avg_r,
         sc_beam->x_sig_good, sc_beam->y_sig_good, sc_beam->mass, sc_beam->num_particle,
         sc_beam->current * sc_frac, sc_freq, sc_beta, sc_adj, len, f2, rr, rz, rq, rg);
}

// ---------------------------------------------------------------------------
// simulation_engine.cu launchers (reference: src/simulation/src/simulation_engine.cu)
// ---------------------------------------------------------------------------
namespace {
SpaceCharge *e_spch;
Beam *e_beam;
BeamLine *e_bl;
SimulationParam *e_param;
uint e_grid, e_blck, e_cur, e_ccl;
double e_design_w;
RFGapParameter e_rf;
DipoleParameter e_dp;
}  // namespace

extern "C" {
void SetConstOnDevice(SimulationConstOnDevice *c) { d_const = *c; }
void Cleanup() {}
void UpdateBlIndex(uint i) { e_cur = i; }
void Reset() {
  e_cur = 0; e_ccl = 0;
  e_design_w = e_beam->design_w;
  launch1(UpdateWaveLengthKernel, e_beam->freq);
  e_grid = e_beam->grid_size; e_blck = e_beam->blck_size;
}
void Init(Beam *b, BeamLine *bl, SpaceCharge *sp, SimulationParam &prm) {
  e_spch = sp; e_beam = b; e_bl = bl; e_param = &prm;
  Reset();
}
void SimulateDrift(Drift *d) {
  int nk = 1;
  double len = d->GetLength();
  if (e_param->space_charge_on) nk = (int)std::ceil(len / e_spch->GetInterval());
  double hf = 0.5 * len / nk;
  for (int k = 0; k < nk; ++k) {
    launch(dim3(e_grid), dim3(e_blck), SimulatePartialDriftKernel, e_beam->x, e_beam->y, e_beam->phi,
           e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, hf, d->GetAperture(), e_cur);
    if (e_param->space_charge_on) e_spch->Start(e_beam, 2.0 * hf);
    launch(dim3(e_grid), dim3(e_blck), SimulatePartialDriftKernel, e_beam->x, e_beam->y, e_beam->phi,
           e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, hf, d->GetAperture(), e_cur);
  }
}
void SimulateQuad(Quad *q) {
  launch(dim3(e_grid), dim3(e_blck / 2), SimulateHalfQuadKernel, e_beam->x, e_beam->y, e_beam->phi,
         e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, q->GetLength(), q->GetAperture(),
         q->GetGradient(), e_cur);
  if (e_param->space_charge_on) e_spch->Start(e_beam, q->GetLength());
  launch(dim3(e_grid), dim3(e_blck / 2), SimulateHalfQuadKernel, e_beam->x, e_beam->y, e_beam->phi,
         e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, q->GetLength(), q->GetAperture(),
         q->GetGradient(), e_cur);
}
static void prep_gap(RFGap *g) {
  e_rf = *g->GetParametersOnDevice();
  if (e_beam->freq != g->GetFrequency()) {
    double f = g->GetFrequency();
    launch1(UpdateWaveLengthKernel, f);
    e_beam->ChangeFrequency(f);
  }
}
void SimulateDTLRFGap(RFGap *g) {
  prep_gap(g);
  double phi_in = 0.0;
  uint sz = e_bl->GetSize();
  if (e_cur == 1 || (e_cur > 1 && (*e_bl)[e_cur - 2]->GetType() != "RFGap-DTL")) {
    if (e_cur + 2 < sz && (*e_bl)[e_cur + 2]->GetType() == "RFGap-DTL") {
      RFGap *nx = dynamic_cast<RFGap *>((*e_bl)[e_cur + 2]);
      phi_in = g->GetRefPhase() - 0.5 * (nx->GetRefPhase() - g->GetRefPhase());
    } else if (e_cur + 1 >= sz) {
      throw std::runtime_error("malformed DTL lattice");
    } else {
      phi_in = g->GetRefPhase();
    }
  } else if (e_cur > 1) {
    RFGap *pv = dynamic_cast<RFGap *>((*e_bl)[e_cur - 2]);
    phi_in = 0.5 * (pv->GetRefPhase() + g->GetRefPhase());
  } else {
    throw std::runtime_error("malformed DTL lattice");
  }
  Quad *q1 = dynamic_cast<Quad *>((*e_bl)[e_cur - 1]);
  Quad *q2 = dynamic_cast<Quad *>((*e_bl)[e_cur + 1]);
  if (!q1 || !q2) throw std::runtime_error("malformed DTL lattice");
  double l1 = q1->GetLength(), l2 = q2->GetLength();
  launch(dim3(e_grid), dim3(e_blck / 2), SimulateRFGapFirstHalfKernel, e_beam->x, e_beam->y,
         e_beam->phi, e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, e_design_w, phi_in, &e_rf,
         g->GetLength(), l1, l2, false);
  if (e_param->space_charge_on) e_spch->Start(e_beam, g->GetLength());
  launch(dim3(e_grid), dim3(e_blck / 2), SimulateRFGapSecondHalfKernel, e_beam->x, e_beam->y,
         e_beam->phi, e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, e_design_w, phi_in, &e_rf,
         g->GetLength(), 0u, l1, l2, false);
  e_design_w = g->GetEnergyOut();
  e_beam->design_w = e_design_w;
}
void SimulateCCLRFGap(RFGap *g) {
  prep_gap(g);
  if (e_cur == 0 || (*e_bl)[e_cur - 1]->GetType() != "RFGap-CCL") e_ccl = 0;
  double phi_in = 0, phi_out = 0;
  uint sz = e_bl->GetSize();
  auto type_at = [&](uint i) { return i < sz ? (*e_bl)[i]->GetType() : std::string(); };
  if (e_ccl == 0) {
    RFGap *nx = dynamic_cast<RFGap *>((*e_bl)[e_cur + 1]);
    if (!nx) throw std::runtime_error("malformed CCL lattice");
    double cur = g->GetRefPhase(), nxt = nx->GetRefPhase();
    phi_in = cur - 0.5 * (nxt - cur);
    phi_out = 0.5 * (nxt + cur);
  } else if (type_at(e_cur + 1) != "RFGap-CCL") {
    RFGap *pv = dynamic_cast<RFGap *>((*e_bl)[e_cur - 1]);
    double cur = g->GetRefPhase(), prv = pv->GetRefPhase();
    phi_in = 0.5 * (cur + prv);
    phi_out = cur + 0.5 * (cur - prv);
  } else {
    RFGap *nx = dynamic_cast<RFGap *>((*e_bl)[e_cur + 1]);
    RFGap *pv = dynamic_cast<RFGap *>((*e_bl)[e_cur - 1]);
    double cur = g->GetRefPhase();
    phi_in = 0.5 * (cur + pv->GetRefPhase());
    phi_out = 0.5 * (cur + nx->GetRefPhase());
  }
  uint gcb = e_blck / 4 > 1 ? e_blck / 4 : e_blck;
  launch(dim3(e_grid), dim3(gcb), SimulateRFGapFirstHalfKernel, e_beam->x, e_beam->y, e_beam->phi,
         e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, e_design_w, phi_in, &e_rf,
         g->GetLength(), 0.0, 0.0, true);
  if (e_param->space_charge_on) e_spch->Start(e_beam, g->GetLength());
  launch(dim3(e_grid), dim3(gcb), SimulateRFGapSecondHalfKernel, e_beam->x, e_beam->y, e_beam->phi,
         e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, e_design_w, phi_out, &e_rf,
         g->GetLength(), e_ccl++, 0.0, 0.0, true);
  e_design_w = g->GetEnergyOut();
  e_beam->design_w = e_design_w;
}
void SimulateRotation(Rotation *r) {
  launch(dim3(e_grid), dim3(e_blck), SimulateRotationKernel, e_beam->x, e_beam->y, e_beam->xp,
         e_beam->yp, e_beam->loss, r->GetAngle());
}
void SimulateSpaceChargeCompensation(SpaceChargeCompensation *s) {
  if (e_param->space_charge_on) e_spch->SetFraction(s->GetFraction());
}
void SimulateApertureCircular(ApertureCircular *a) {
  if (!a->IsIn()) return;
  e_beam->UpdateLoss();
  e_beam->UpdateAvgXY();
  launch(dim3(e_grid), dim3(e_blck), SimulateCircularApertureKernel, e_beam->x, e_beam->y,
         e_beam->loss, a->GetAperture(), e_beam->x_avg, e_beam->y_avg, (int)e_cur);
}
void SimulateApertureRectangular(ApertureRectangular *a) {
  if (!a->IsIn()) return;
  e_beam->UpdateLoss();
  e_beam->UpdateAvgXY();
  launch(dim3(e_grid), dim3(e_blck), SimulateRectangularApertureKernel, e_beam->x, e_beam->y,
         e_beam->loss, a->GetApertureXLeft(), a->GetApertureXRight(), a->GetApertureYTop(),
         a->GetApertureYBottom(), e_beam->x_avg, e_beam->y_avg, (int)e_cur);
}
void SimulateDiagnostics(Diagnostics *) {}
void SimulateSteerer(Steerer *s) {
  double blh = s->GetIntegratedFieldHorizontal(), blv = s->GetIntegratedFieldVertical();
  if (blh > 1e-10 || blv > 1e-10)
    launch(dim3(e_grid), dim3(e_blck), SimulateSteererKernel, e_beam->xp, e_beam->yp, e_beam->w,
           e_beam->loss, blh, blv);
}
void SimulateBuncher(Buncher *b) {
  if (!b->IsOn()) return;
  double bf = b->GetFrequency();
  launch1(UpdateWaveLengthKernel, bf);
  launch(dim3(e_grid), dim3(e_blck), SimulateBuncherKernel, e_beam->x, e_beam->y, e_beam->phi,
         e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, e_design_w, bf, b->GetVoltage(),
         b->GetPhase(), b->GetAperture(), bf / e_beam->freq, e_cur);
}
void SimulateDipole(Dipole *d) {
  e_dp = *d->GetParametersOnDevice();
  launch(dim3(e_grid), dim3(e_blck / 4), SimulateFirstHalfDipoleKernel, e_beam->x, e_beam->y,
         e_beam->phi, e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, &e_dp);
  if (e_param->space_charge_on) e_spch->Start(e_beam, d->GetRadius() * d->GetAngle());
  launch(dim3(e_grid), dim3(e_blck / 4), SimulateSecondHalfDipoleKernel, e_beam->x, e_beam->y,
         e_beam->phi, e_beam->xp, e_beam->yp, e_beam->w, e_beam->loss, &e_dp);
}
}  // extern "C"

// ---------------------------------------------------------------------------
// C API for the ctypes test driver
// ---------------------------------------------------------------------------
#include "../include/hps_layout.h"

struct RefScheffBox { Scheff *s; };

extern "C" {
void *ref_beam_create(uint n, double mass, double charge, double current) {
  return new Beam(n, mass, charge, current);
}
void ref_beam_free(void *b) { delete (Beam *)b; }
void ref_beam_set_waterbag(void *bp, const double *t, double phi, double w, double f, uint seed) {
  ((Beam *)bp)->InitWaterbagBeam(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], phi, w, f, seed);
}
void ref_beam_set_dc(void *bp, double ax, double bx, double ex, double ay, double by, double ey,
                     double dphi, double sphi, double sw, uint seed) {
  ((Beam *)bp)->InitDCBeam(ax, bx, ex, ay, by, ey, dphi, sphi, sw, seed);
}
void ref_beam_set_distribution(void *bp, const double *x, const double *xp, const double *y,
                               const double *yp, const double *phi, const double *w,
                               const uint *loss, const uint *lloss) {
  Beam *b = (Beam *)bp;
  size_t n = b->num_particle;
  std::vector<double> vx(x, x + n), vxp(xp, xp + n), vy(y, y + n), vyp(yp, yp + n), vp(phi, phi + n),
      vw(w, w + n);
  std::vector<uint> vl, vll;
  if (loss) vl.assign(loss, loss + n);
  if (lloss) vll.assign(lloss, lloss + n);
  b->InitBeamFromDistribution(vx, vxp, vy, vyp, vp, vw, loss ? &vl : nullptr, lloss ? &vll : nullptr);
}
// Beam::PrintToFile and Beam(file) (beam.cpp:47-60, 179-298, 670-707)
void ref_beam_print(void *b, const char *file, const char *msg) { ((Beam *)b)->PrintToFile(file, msg); }
void *ref_beam_from_file(const char *file) { return new Beam(std::string(file)); }
uint ref_beam_size(void *b) { return ((Beam *)b)->num_particle; }
void ref_beam_scalars(void *bp, double *out) {
  Beam *b = (Beam *)bp;
  out[0] = b->mass; out[1] = b->charge; out[2] = b->current; out[3] = b->freq; out[4] = b->design_w;
}
void ref_beam_set_ref_w(void *b, double w) { ((Beam *)b)->SetRefEnergy(w); }
void ref_beam_set_ref_phi(void *b, double p) { ((Beam *)b)->SetRefPhase(p); }
void ref_beam_set_frequency(void *b, double f) { ((Beam *)b)->freq = f; }
void ref_beam_get(void *bp, double *x, double *xp, double *y, double *yp, double *phi, double *w,
                  uint *loss, uint *lloss) {
  Beam *b = (Beam *)bp;
  uint nl;
  CopyBeamFromDevice(b, x, xp, y, yp, phi, w, loss, lloss, &nl);
}
// side-effect-free monitor record (same definition as orc_beam_monitor)
void ref_beam_monitor(void *bp, double *out) {
  Beam *b = (Beam *)bp;
  uint n = b->num_particle;
  for (int k = 0; k < HPS_NMON; ++k) out[k] = 0.0;
  if (!n) return;
  double s[17] = {0};
  double ref = b->phi[0], pi = 3.14159265358979323846, twopi = pi * 2.0;
  for (uint i = 0; i < n; ++i) {
    if (b->loss[i] + b->lloss[i] == 0) s[16] += 1.0;
    if (b->loss[i] != 0) continue;
    double tmp = b->phi[i] - ref + pi, sign = 1.0;
    if (tmp < 0) { sign = -1.0; tmp = -tmp; }
    double pr = sign * (std::fmod(tmp, twopi) - pi);
    double x = b->x[i], xp = b->xp[i], y = b->y[i], yp = b->yp[i], w = b->w[i];
    s[0] += 1; s[1] += x; s[2] += x * x; s[3] += xp; s[4] += xp * xp; s[5] += x * xp;
    s[6] += y; s[7] += y * y; s[8] += yp; s[9] += yp * yp; s[10] += y * yp;
    s[11] += pr; s[12] += pr * pr; s[13] += w; s[14] += w * w; s[15] += pr * w;
  }
  double m = s[0];
  out[HPS_MON_NALIVE] = m;
  out[HPS_MON_NGOOD] = s[16];
  double g1 = b->w[0] / b->mass, bg = std::sqrt(g1 * (g1 + 2.0));
  if (m > 0) {
    for (int pl = 0; pl < 2; ++pl) {
      const double *q = s + 1 + 5 * pl;
      double a = q[0] / m, a2 = q[1] / m, ap = q[2] / m, ap2 = q[3] / m, aap = q[4] / m;
      int base = pl ? HPS_MON_Y_AVG : HPS_MON_X_AVG;
      out[base] = a; out[base + 1] = std::sqrt(a2 - a * a); out[base + 2] = ap;
      out[base + 3] = std::sqrt(ap2 - ap * ap);
      out[base + 4] = std::sqrt((a2 - a * a) * (ap2 - ap * ap) - (aap - a * ap) * (aap - a * ap)) * bg;
    }
    double p = s[11] / m, p2 = s[12] / m, w = s[13] / m, w2 = s[14] / m, pw = s[15] / m;
    double pv = p2 - p * p, wv = w2 - w * w, cv = pw - p * w;
    out[HPS_MON_PHIR_AVG] = p; out[HPS_MON_PHIR_SIG] = std::sqrt(pv);
    out[HPS_MON_W_AVG] = w; out[HPS_MON_W_SIG] = std::sqrt(wv);
    out[HPS_MON_Z_EMIT] = std::sqrt(pv * wv - cv * cv);
  }
  out[HPS_MON_W0] = b->w[0];
  out[HPS_MON_PHI0] = b->phi[0];
}

void *ref_beamline_create() { return new BeamLine(); }
void ref_beamline_free(void *bl) { delete (BeamLine *)bl; }
int ref_beamline_add(void *blp, int type, const char *name, const double *p) {
  BeamLine *bl = (BeamLine *)blp;
  std::string nm(name);
  BeamLineElement *e = nullptr;
  switch (type) {
    case HPS_ELEM_DRIFT: { Drift *d = new Drift(nm); e = d; break; }
    case HPS_ELEM_QUAD: { Quad *q = new Quad(nm); q->SetGradient(p[HPS_P_GRADIENT]); e = q; break; }
    case HPS_ELEM_RFGAP_DTL:
    case HPS_ELEM_RFGAP_CCL: {
      RFGap *g = new RFGap(nm, type == HPS_ELEM_RFGAP_DTL ? "RFGap-DTL" : "RFGap-CCL");
      g->SetLength(p[HPS_P_LENGTH]);
      g->SetFrequency(p[HPS_P_RF_FREQ]);
      g->SetCellLengthOverBetaLambda(p[HPS_P_RF_CLBL]);
      g->SetRFAmplitude(p[HPS_P_RF_AMP]);
      g->SetRefPhase(p[HPS_P_RF_PHASE_REF]);
      g->SetPhaseShift(p[HPS_P_RF_PHASE_SHIFT]);
      g->SetEnergyOut(p[HPS_P_RF_ENERGY_OUT]);
      g->SetBetaCenter(p[HPS_P_RF_BETA_CENTER]);
      g->SetDg(p[HPS_P_RF_DG]);
      g->SetT(p[HPS_P_RF_T]); g->SetTp(p[HPS_P_RF_TP]); g->SetSp(p[HPS_P_RF_SP]);
      g->SetFitBetaCenter(p[HPS_P_RF_FIT_BETA_CENTER]);
      g->SetFitBetaMin(p[HPS_P_RF_FIT_BETA_MIN]);
      g->SetFitT0(p[15]); g->SetFitT1(p[16]); g->SetFitT2(p[17]); g->SetFitT3(p[18]);
      g->SetFitT4(p[19]); g->SetFitT5(p[20]);
      g->SetFitS1(p[21]); g->SetFitS2(p[22]); g->SetFitS3(p[23]); g->SetFitS4(p[24]); g->SetFitS5(p[25]);
      e = g;
      break;
    }
    case HPS_ELEM_BUNCHER: {
      Buncher *b = new Buncher(nm);
      if (p[HPS_P_BUN_ON] != 0.0) b->TurnOn(); else b->TurnOff();
      b->SetVoltage(p[HPS_P_BUN_VOLTAGE]); b->SetFrequency(p[HPS_P_BUN_FREQ]); b->SetPhase(p[HPS_P_BUN_PHASE]);
      e = b;
      break;
    }
    case HPS_ELEM_STEERER: {
      Steerer *s = new Steerer(nm);
      s->SetIntegratedFieldHorizontal(p[HPS_P_STR_BLH]); s->SetIntegratedFieldVertical(p[HPS_P_STR_BLV]);
      e = s;
      break;
    }
    case HPS_ELEM_APERTURE_C: {
      ApertureCircular *a = new ApertureCircular(nm);
      if (p[HPS_P_APT_IN] != 0.0) a->SetIn(); else a->SetOut();
      e = a;
      break;
    }
    case HPS_ELEM_APERTURE_R: {
      ApertureRectangular *a = new ApertureRectangular(nm);
      if (p[HPS_P_APT_IN] != 0.0) a->SetIn(); else a->SetOut();
      a->SetApertureXLeft(p[HPS_P_APT_XL]); a->SetApertureXRight(p[HPS_P_APT_XR]);
      a->SetApertureYTop(p[HPS_P_APT_YT]); a->SetApertureYBottom(p[HPS_P_APT_YB]);
      e = a;
      break;
    }
    case HPS_ELEM_DIAGNOSTICS: e = new Diagnostics(nm); break;
    case HPS_ELEM_ROTATION: { Rotation *r = new Rotation(nm); r->SetAngle(p[HPS_P_ROT_ANGLE]); e = r; break; }
    case HPS_ELEM_SPCHCOMP: {
      SpaceChargeCompensation *s = new SpaceChargeCompensation(nm);
      s->SetFraction(p[HPS_P_SPC_FRACTION]);
      e = s;
      break;
    }
    case HPS_ELEM_DIPOLE: {
      Dipole *d = new Dipole(nm);
      d->SetRadius(p[HPS_P_DIP_RADIUS]); d->SetAngle(p[HPS_P_DIP_ANGLE]);
      d->SetEdgeAngleIn(p[HPS_P_DIP_EDGE_IN]); d->SetEdgeAngleOut(p[HPS_P_DIP_EDGE_OUT]);
      d->SetHalfGap(p[HPS_P_DIP_HALF_GAP]); d->SetK1(p[HPS_P_DIP_K1]); d->SetK2(p[HPS_P_DIP_K2]);
      d->SetFieldIndex(p[HPS_P_DIP_FIELD_INDEX]); d->SetKineticEnergy(p[HPS_P_DIP_KINETIC_ENERGY]);
      e = d;
      break;
    }
    default: return -1;
  }
  if (type != HPS_ELEM_RFGAP_DTL && type != HPS_ELEM_RFGAP_CCL) e->SetLength(p[HPS_P_LENGTH]);
  e->SetAperture(p[HPS_P_APERTURE]);
  bl->AddElement(e);
  return 0;
}

void *ref_scheff_create(uint nr, uint nz, int adj, double interval, double remesh, double adj_w,
                        double mesh_w) {
  Scheff *s = new Scheff(nr, nz, adj);
  s->SetInterval(interval);
  s->SetRemeshThreshold(remesh);
  s->SetAdjBunchCutoffW(adj_w);
  s->SetMeshSizeCutoffW(mesh_w);
  return s;
}
void ref_scheff_free(void *s) { delete (Scheff *)s; }
void ref_scheff_mesh(double *dr, double *dz, uint *onm) { *dr = scheff_sz.dr; *dz = scheff_sz.dz; *onm = num_on_mesh; }
// mesh description of the last solve: {dr, dz, beta, freq, num_particle, current*frac/mass, adj}
void ref_scheff_mesh_params(double *m) {
  m[0] = scheff_sz.dr; m[1] = scheff_sz.dz; m[2] = sc_beta; m[3] = sc_freq;
  m[4] = sc_beam->num_particle; m[5] = sc_beam->current * sc_frac / sc_beam->mass; m[6] = sc_adj;
}

void ref_scheff_tables(double *bin, double *fld1, double *fld2) {
  std::memcpy(bin, g_bin, (size_t)sc_nr * sc_nz * sizeof(double));
  std::memcpy(fld1, g_fld1, (size_t)sc_nr * sc_nz * (sc_nr + 1) * sizeof(double2));
  std::memcpy(fld2, g_fld2, (size_t)(sc_nz + 1) * (sc_nr + 1) * sizeof(double2));
}

void *ref_sim_create(void *b, void *bl, void *sp) {
  // device globals of the kernel files start from zero for every run
  scheff_sz.dr = 0.0; scheff_sz.dz = 0.0; num_on_mesh = 0;
  SimulationEngine *e = new SimulationEngine();
  e->InitEngine((Beam *)b, (BeamLine *)bl, (SpaceCharge *)sp);
  return e;
}
void ref_sim_free(void *e) { delete (SimulationEngine *)e; }

// Simulate [start, end] one element at a time (equivalent to one
// Simulate(start, end) call: each single-element call neither resets the
// engine nor skips anything), writing the monitor record after each element.
int ref_sim_simulate(void *ep, void *bp, int start, int end, double *mon) {
  SimulationEngine *e = (SimulationEngine *)ep;
  BeamLine *bl = e_bl;
  int n = (int)bl->GetSize();
  if (start < 0) start = 0;
  if (end < 0) end = n - 1;
  try {
    for (int i = start; i <= end; ++i) {
      std::string nm = bl->GetElementName(i);
      e->Simulate(nm, nm);
      if (mon) {
        double *m = mon + (size_t)i * HPS_NMON;
        ref_beam_monitor(bp, m);
        m[HPS_MON_SC_DR] = scheff_sz.dr;
        m[HPS_MON_SC_DZ] = scheff_sz.dz;
        m[HPS_MON_SC_ONMESH] = num_on_mesh;
        m[HPS_MON_ELEM] = i;
      }
    }
  } catch (...) {
    return -1;
  }
  return 0;
}
}  // extern "C"
