// scheff_common.cuh -- the device-side body of Scheff::Start shared by the
// FP64 and FP32 solvers: mesh-size update, the remesh decision and the table
// reset (src/simulation/src/space_charge.cpp:82-139,
// src/simulation/src/space_charge.cu:88-138,
// src/simulation/inc/space_charge_kernel.cu:18-32).
#pragma once

#include "common.cuh"

namespace hps {

// Scheff::SetMeshSize (space_charge.cpp:61-73) on the device: the tables were
// reallocated and zeroed by Initialize in the reference.
__device__ inline void set_mesh_size(ScState *s, uint32_t nr, uint32_t nz) {
  if (nr != s->nx || nz != s->nz) {
    s->nx = nr;
    s->nz = nz;
    s->resized = 1;
  }
}

// UpdateScheffMeshSizeKernel, space_charge_kernel.cu:18-32
__device__ inline void mesh_size(ScState *s, double partial_r, double partial_z, double coef) {
  double bl = s->beta * CLIGHT / s->freq;
  s->dr = coef * partial_r / s->nx;
  if (coef == 1.0) s->dz = bl / s->nz;
  else {
    if (partial_z * coef > PI) s->dz = bl / s->nz;
    s->dz = coef * bl * partial_z / (s->nz * PI);
  }
}

// The host-side body of Scheff::Start after the statistics
// (space_charge.cpp:86-138) plus UpdateMeshKernelCall (space_charge.cu:122-138).
__device__ inline void scheff_decide(const DevBeam &b, ScState *s, double freq, double frac) {
  const BeamStats &st = *b.st;
  uint32_t good_cnt = st.num_good;
  double sigphi = b.n < 2 ? 0.0 : st.st[PHI_SIG_GOOD];
  double sigx = b.n < 2 ? 0.0 : st.st[X_SIG_GOOD];
  double sigy = b.n < 2 ? 0.0 : st.st[Y_SIG_GOOD];
  double ke = st.st[W_AVG_GOOD];
  double gamma = (double)ke / b.mass + 1.0;
  double beta = sqrt(1.0 - 1.0 / (gamma * gamma));
  double lmbd = 299.792458 / freq;
  double sigz = sigphi * 0.5 / 3.14159265 * beta * lmbd;
  double sigr = sqrt(sigx * sigx + sigy * sigy);
  double cratior = sigr * sigz;
  double cratioz = sigz * sigz * gamma * gamma;
  double cratior_old = s->sigr_old * s->sigz_old;
  double cratioz_old = s->sigz_old * s->sigz_old * s->gm_old * s->gm_old;
  uint32_t adj = (s->adj_bunch_w == 0.0 || ke < s->adj_bunch_w) ? s->adj_bunch : 0u;
  s->resized = 0;
  if (s->mesh_w != 0.0) {
    if (ke > s->mesh_w && (s->nx != s->nx_init / 2 || s->nz != s->nz_init / 2))
      set_mesh_size(s, s->nx_init / 2, s->nz_init / 2);
    else if (ke <= s->mesh_w && (s->nx != s->nx_init || s->nz != s->nz_init))
      set_mesh_size(s, s->nx_init, s->nz_init);
    if (ke > s->mesh_w && s->interval != s->interval_init * 4) s->interval = s->interval_init * 4;
    else if (ke <= s->mesh_w && s->interval != s->interval_init) s->interval = s->interval_init;
  }
  s->freq = freq;
  s->beta = beta;
  s->frac = frac;
  s->adj = adj;
  if (cratior_old == 0.0 || cratioz_old == 0.0 || fabs(cratior - cratior_old) / cratior_old > s->remesh_val ||
      fabs(cratioz - cratioz_old) / cratioz_old > s->remesh_val) {
    s->sigr_old = sigr;
    s->sigz_old = sigz;
    s->gm_old = gamma;
    s->good_cnt_old = good_cnt;
    s->remesh = 1;
    s->n_solves += 1;
    s->ratio_r = s->ratio_z = s->ratio_q = s->ratio_g = 1.0;
    // The reference compares the device pointers x_sig_good > y_sig_good;
    // x_sig_good is allocated first (beam.cu:51,54) so the y branch runs.
    if (adj == 0) mesh_size(s, st.st[Y_SIG_GOOD], st.st[PHI_SIG_GOOD], 3.0);
  } else {
    s->remesh = 0;
    s->ratio_r = sigr / s->sigr_old;
    s->ratio_z = sigz / s->sigz_old;
    s->ratio_q = s->good_cnt_old ? (double)(good_cnt / s->good_cnt_old) : 0.0;
    s->ratio_g = gamma / s->gm_old;
  }
}

__device__ inline void zero_mesh_tables(ScState *s, const ScTables &t, int tid, int nth) {
  if (!(s->remesh || s->resized)) return;
  uint32_t nb = s->nx * s->nz, nf = (s->nx + 1) * (s->nz + 1) * 2;
  for (uint32_t k = tid; k < nb; k += nth) t.bin_fx[k] = 0ull;
  if (t.fld2)
    for (uint32_t k = tid; k < nf; k += nth) t.fld2[k] = 0.0;
  if (t.ffld2)
    for (uint32_t k = tid; k < nf; k += nth) t.ffld2[k] = 0.0f;
  if (tid == 0 && s->remesh) s->num_on_mesh = 0u;
}
}  // namespace hps
