// surrogate.cu -- the learned SCHEFF field surrogate inside a beam's
// space-charge kick (FP64 or FP32 tables), with a spot-solve residual check
// and fallback to the plain contraction.  Launch sequence of a kick that
// remeshes (after the deposit, before the Green's table and the contraction):
//   k_sur_input   charge / total and log cell aspect as the network input
//                 (BF16), the field scale, the acceptance flag cleared;
//   the network   its 3x3 convolution layers (nn.cu) with the skip additions
//                 fused and the plane-mean broadcast, on a batch of one;
//   k_sur_spot    the plain method's field (the sum over every bin of charge
//                 times the Green's function, evaluated in FP32) at the
//                 mesh's last row and column, which the network does not
//                 predict, and at n_samples interior points drawn per solve;
//   k_sur_fit     the network's E_r and E_z corrected by gains (constant
//                 plus linear across the mesh) fitted at the sample points,
//                 and their relative residual there against the tolerance;
//   k_sur_write   when accepted, the field table gets the corrected interior
//                 and the spot-solved boundary, and the solver state says
//                 so: the FP64 Green's table and the contraction then return
//                 at once.
// Kicks that do not remesh, meshes other than the trained one and empty
// meshes leave everything to the plain path.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/hpsim_gb300.h"
#include "green32.cuh"
#include "internal.h"

namespace hps {

namespace {

constexpr int kSurBlock = 256;
constexpr int kFitBlock = 64;
constexpr int kInBlocks = 16;

struct SurDev {
  int active;          // this kick is the surrogate's to try
  double total;        // charge on the mesh (bin units)
  double scale;        // field = network output * scale
  double c1, dzg, dr;  // Green's-table scale, bunch-frame cell length, radial cell size
  double residual;     // relative residual of the last check
  double cf[6];        // field = output * (cf0 + cf1 z + cf2 r) for E_r, cf3.. for E_z
  uint32_t n_accepted, n_rejected;
  unsigned int conv_err;  // a tensor-core layer's bounded wait gave up
};

// a fixed-point charge bin as FP32 through two 32-bit conversions (a 64-bit
// integer conversion runs on the FP64 pipe)
__device__ inline float fixed_to_float(unsigned long long v) {
  const long long s = (long long)v;
  return fmaf((float)(int)(s >> 32), 4294967296.0f, (float)(unsigned)(v & 0xffffffffull));
}

__device__ inline uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}

// field point of spot index k: the last row (zp = nz, rp = 0..nr), the last
// column (rp = nr, zp = 0..nz-1), then the interior samples of this solve
__device__ inline void spot_point(uint32_t k, uint32_t nr, uint32_t nz, uint32_t solve, uint32_t &zp,
                                  uint32_t &rp) {
  if (k <= nr) { zp = nz; rp = k; return; }
  k -= nr + 1;
  if (k < nz) { zp = k; rp = nr; return; }
  k -= nz;
  const uint32_t h = mix32(solve * 0x9e3779b9u + k * 0x85ebca6bu + 0x632be5abu);
  zp = h % nz;
  rp = (h >> 16) % nr;
}

// kInBlocks blocks: each sums the whole charge table (a few microseconds of
// loads, not worth a second launch) and normalises its share; block 0
// records the kick's scalars
// fp32: the kick of an FP32 beam (mesh and Green's-table scale from the FP32
// kick constants, as the FP32 Green's table takes them)
__global__ void __launch_bounds__(kSurBlock) k_sur_input(ScState *sc, ScTables t, SurDev *sd, __nv_bfloat16 *x,
                                                         uint32_t nr, uint32_t nz, double out_scale,
                                                         uint32_t num_part, double cur_ov_mc2, int fp32) {
  __shared__ unsigned long long red[kSurBlock];
  __shared__ int go;
  __shared__ float qs;
  __shared__ __nv_bfloat16 la;
  if (threadIdx.x == 0) {
    // the trained mesh, no adjacent bunches, every source row in the table
    const uint32_t by = (512 / nz < nr) ? 512 / nz : nr;
    go = sc->remesh && sc->nx == nr && sc->nz == nz && sc->adj == 0 && by && (nr / by) * by == nr;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->sur_accepted = 0;
    if (!go) sd->active = 0;
  }
  if (!go) return;
  const uint32_t nb = nr * nz;
  unsigned long long a = 0;
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) a += t.bin_fx[k];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (fp32) {
      // FP32 arithmetic throughout (an FP64 divide costs about a microsecond)
      const Sc32Consts &k = *t.c32;
      const float dr = k.dr0, dzg = k.dzg0, c1 = k.green_c1;
      if (blockIdx.x == 0) {
        const float total = (float)(long long)red[0] * 1.4551915228366852e-11f;  // 2^-36
        sd->active = total > 0.0f;
        sd->total = total;
        sd->scale = c1 * total / ((float)out_scale * dr * dzg);
        sd->c1 = c1;
        sd->dzg = dzg;
        sd->dr = dr;
      }
      qs = red[0] ? (float)nb / (float)(long long)red[0] : 0.0f;
      la = __float2bfloat16_rn(logf(dzg / dr));
    } else {
      const double dzg = sc->dz * rsqrt(1.0 - sc->beta * sc->beta);
      if (blockIdx.x == 0) {
        const double total = (double)(long long)red[0] * kBinInvScale;
        const double c1 = 5721.67 * cur_ov_mc2 / (sc->freq * 1e6 * (double)num_part);
        sd->active = total > 0.0;
        sd->total = total;
        sd->scale = c1 * total / (out_scale * sc->dr * dzg);
        sd->c1 = c1;
        sd->dzg = dzg;
        sd->dr = sc->dr;
      }
      // charge / total * nb in bin units: the fixed-point integers times nb / sum
      qs = red[0] ? (float)((double)nb / (double)(long long)red[0]) : 0.0f;
      la = __float2bfloat16_rn((float)log(dzg / sc->dr));
    }
  }
  __syncthreads();
  if (!red[0]) return;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x) {
    x[k] = __float2bfloat16_rn(fixed_to_float(t.bin_fx[k]) * qs);
    x[nb + k] = la;
  }
}

// the plain method's field at one spot point per block: E_r += q G_r,
// E_z += +-q G_z over every bin with the contraction's pairing of bins and
// table entries, the Green's function evaluated in FP32 on the fly (the
// FP64 table is built only when the kick falls back); each thread's sum in
// FP32, the block's in FP64, in a fixed order
__global__ void __launch_bounds__(kSurBlock) k_sur_spot(const ScState *sc, const ScTables t, const SurDev *sd,
                                                        double2 *spot, uint32_t nr, uint32_t nz) {
  if (!sd->active) return;
  __shared__ double rx[kSurBlock], rz[kSurBlock];
  uint32_t zp, rp;
  spot_point(blockIdx.x, nr, nz, sc->n_solves, zp, rp);
  const uint32_t nb = nr * nz;
  const float dr = (float)sd->dr, dzg = (float)sd->dzg;
  const float rpf = (float)rp * dr;
  float ax = 0.0f, az = 0.0f;
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) {
    const unsigned long long v = t.bin_fx[k];
    if (!v) continue;
    const float q = fixed_to_float(v) * 1.4551915228366852e-11f;  // 2^-36
    const uint32_t rs = k % nr, zs = k / nr;
    const bool above = zs >= zp;
    const uint32_t dz = above ? zs - zp : zp - zs - 1;
    const float rsf = sqrtf(0.5f * (float)(rs * rs + (rs + 1) * (rs + 1))) * dr;
    const GreenTerm g = green_term(rsf, rpf, ((float)dz + 0.5f) * dzg);
    ax = fmaf(q, g.er, ax);
    az = fmaf(above ? -q : q, g.ez, az);
  }
  rx[threadIdx.x] = ax;
  rz[threadIdx.x] = az;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      rx[threadIdx.x] += rx[threadIdx.x + off];
      rz[threadIdx.x] += rz[threadIdx.x + off];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) spot[blockIdx.x] = make_double2(sd->c1 * rx[0], sd->c1 * rz[0]);
}

// each v[j] summed over the block -- a fixed shuffle tree per warp, then the
// warps in order -- and returned to every thread in v; red holds K values
// per warp
template <int K>
__device__ inline void block_sum(double *red, double (&v)[K]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < K; ++j)
    for (int off = 16; off > 0; off >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], off);
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < K; ++j) red[warp * K + j] = v[j];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < K; ++j) {
    double a = red[j];
    for (int w = 1; w < nw; ++w) a += red[w * K + j];
    v[j] = a;
  }
  __syncthreads();
}

// the solution of the symmetric 3x3 system m c = y (m packed as m00 m01 m02
// m11 m12 m22) by Cramer's rule; false when m is numerically singular
__device__ inline bool solve3(const double *m, const double *y, double *c) {
  const double a = m[0], b = m[1], d = m[2], e = m[3], f = m[4], g = m[5];
  const double c00 = e * g - f * f, c01 = d * f - b * g, c02 = b * f - d * e;
  const double det = a * c00 + b * c01 + d * c02;
  if (!(fabs(det) > 1e-12 * fabs(a * e * g) && a > 0.0)) return false;
  const double c11 = a * g - d * d, c12 = b * d - a * f, c22 = a * e - b * b;
  const double inv = 1.0 / det;  // one FP64 divide (each costs about a microsecond)
  c[0] = (c00 * y[0] + c01 * y[1] + c02 * y[2]) * inv;
  c[1] = (c01 * y[0] + c11 * y[1] + c12 * y[2]) * inv;
  c[2] = (c02 * y[0] + c12 * y[1] + c22 * y[2]) * inv;
  return true;
}

// relative mesh coordinates of the calibration's linear terms
__device__ inline float zhat(uint32_t zp, uint32_t nz) { return ((float)zp + 0.5f) / (float)nz - 0.5f; }
__device__ inline float rhat(uint32_t rp, uint32_t nr) { return ((float)rp + 0.5f) / (float)nr; }

// The acceptance test (one block).  Calibration: each component e of the
// network's field is corrected to e (c0 + c1 z + c2 r) (z, r relative mesh
// coordinates) with the least-squares coefficients that fit it to the
// spot-solved values (a global amplitude error and gains varying linearly
// across the mesh are removed; a singular fit keeps the amplitude factor
// alone).  The relative residual of the corrected field at the samples
// decides; the coefficients and the decision go to the solver state.
__global__ void __launch_bounds__(kFitBlock) k_sur_fit(ScState *sc, SurDev *sd, const __nv_bfloat16 *out,
                                                       const double2 *spot, uint32_t nr, uint32_t nz,
                                                       uint32_t n_samples, double tol) {
  if (!sd->active) return;
  __shared__ double red[18 * (kFitBlock / 32)];
  const double scale = sd->scale;
  const uint32_t nb = nr * nz, base = nr + 1 + nz;
  // per component: the normal matrix (6) and right-hand side (3)
  double fit[18];
#pragma unroll
  for (int j = 0; j < 18; ++j) fit[j] = 0.0;
  for (uint32_t k = threadIdx.x; k < n_samples; k += blockDim.x) {
    uint32_t zp, rp;
    spot_point(base + k, nr, nz, sc->n_solves, zp, rp);
    const double2 e = spot[base + k];
    const double zh = zhat(zp, nz), rh = rhat(rp, nr);
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      const double en = (double)__bfloat162float(out[comp * nb + zp * nr + rp]) * scale;
      const double bs[3] = {en, en * zh, en * rh};
      double *f = fit + 9 * comp;
      f[0] += bs[0] * bs[0]; f[1] += bs[0] * bs[1]; f[2] += bs[0] * bs[2];
      f[3] += bs[1] * bs[1]; f[4] += bs[1] * bs[2]; f[5] += bs[2] * bs[2];
      const double ex = comp ? e.y : e.x;
      f[6] += bs[0] * ex; f[7] += bs[1] * ex; f[8] += bs[2] * ex;
    }
  }
  block_sum(red, fit);
  double cf[2][3];
#pragma unroll
  for (int comp = 0; comp < 2; ++comp) {
    const double *f = fit + 9 * comp;
    if (!solve3(f, f + 6, cf[comp])) {
      cf[comp][0] = f[0] > 0.0 ? f[6] / f[0] : 1.0;
      cf[comp][1] = cf[comp][2] = 0.0;
    }
  }
  double r[2] = {0.0, 0.0};  // residual, reference
  for (uint32_t k = threadIdx.x; k < n_samples; k += blockDim.x) {
    uint32_t zp, rp;
    spot_point(base + k, nr, nz, sc->n_solves, zp, rp);
    const double2 e = spot[base + k];
    const double zh = zhat(zp, nz), rh = rhat(rp, nr);
    const double er = (double)__bfloat162float(out[zp * nr + rp]) * scale *
                      (cf[0][0] + cf[0][1] * zh + cf[0][2] * rh);
    const double ez = (double)__bfloat162float(out[nb + zp * nr + rp]) * scale *
                      (cf[1][0] + cf[1][1] * zh + cf[1][2] * rh);
    r[0] += (er - e.x) * (er - e.x) + (ez - e.y) * (ez - e.y);
    r[1] += e.x * e.x + e.y * e.y;
  }
  block_sum(red, r);
  if (threadIdx.x != 0) return;
  // the ratio in FP32 (the test needs a few digits; FP64 divide and square
  // root take microseconds on this GPU)
  const bool f32 = r[1] > 1e-30 && r[1] < 1e30 && r[0] < 1e30;
  const double res = r[1] > 0.0 ? (f32 ? (double)sqrtf((float)r[0] / (float)r[1]) : sqrt(r[0] / r[1]))
                                 : (r[0] > 0.0 ? 1.0 : 0.0);
  const bool ok = res <= tol;
  sd->residual = res;
  if (ok) sd->n_accepted += 1;
  else sd->n_rejected += 1;
  for (int j = 0; j < 6; ++j) sd->cf[j] = scale * cf[j / 3][j % 3];
  sc->sur_accepted = ok;
}

// an accepted field into the field table (the FP32 table of an FP32 beam):
// the corrected network field inside, the spot-solved values on the last row
// and column
__global__ void __launch_bounds__(kSurBlock) k_sur_write(const ScState *sc, ScTables t, const SurDev *sd,
                                                         const __nv_bfloat16 *out, const double2 *spot, uint32_t nr,
                                                         uint32_t nz, int fp32) {
  if (!sd->active || !sc->sur_accepted) return;
  const uint32_t nrow = nr + 1, nb = nr * nz;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (nz + 1) * nrow) return;
  const uint32_t zp = p / nrow, rp = p % nrow;
  double2 e;
  if (zp < nz && rp < nr) {
    const double zh = zhat(zp, nz), rh = rhat(rp, nr);
    e.x = (double)__bfloat162float(out[zp * nr + rp]) * (sd->cf[0] + sd->cf[1] * zh + sd->cf[2] * rh);
    e.y = (double)__bfloat162float(out[nb + zp * nr + rp]) * (sd->cf[3] + sd->cf[4] * zh + sd->cf[5] * rh);
  } else {
    e = spot[zp == nz ? rp : nr + 1 + zp];
  }
  if (fp32) ((float2 *)t.ffld2)[p] = make_float2((float)e.x, (float)e.y);
  else ((double2 *)t.fld2)[p] = e;
}

}  // namespace

SurNet::~SurNet() {
  for (void *p : w) cudaFree(p);
  for (void *p : wt) cudaFree(p);
  for (float *p : b) cudaFree(p);
  for (void *p : act) cudaFree(p);
  if (x) cudaFree(x);
  if (spot) cudaFree(spot);
  if (d) cudaFree(d);
}

void sur_solve(const DevBeam &bm, ScState *sc, const ScTables &t, const ScKickArgs &a, const SurNet &n,
               cudaStream_t st, int fp32) {
  SurDev *sd = (SurDev *)n.d;
  k_sur_input<<<kInBlocks, kSurBlock, 0, st>>>(sc, t, sd, (__nv_bfloat16 *)n.x, n.nr, n.nz, n.out_scale, bm.n,
                                               a.current * a.frac / bm.mass, fp32);
  const void *cur = n.x;
  for (size_t l = 0; l < n.arch.size(); ++l) {
    const int32_t *dims = n.dims.data() + 7 * l;
    const void *skip = n.skip[l] >= 0 ? n.act[n.skip[l]] : nullptr;
    if (n.use_tc && n.wt[l])
      nn_conv_forward_tc(dims, cur, n.wt[l], n.b[l], n.arch[l][4], skip, n.act[l], &sd->conv_err, st);
    else
      nn_conv_forward(dims, cur, n.w[l], n.b[l], n.arch[l][4], skip, n.act[l], st);
    if ((int)l == n.gmean_after) nn_gmean_forward(n.act[l], dims[2], n.hw[l], st);
    cur = n.act[l];
  }
  const uint32_t npts = n.nr + 1 + n.nz + n.n_samples;
  k_sur_spot<<<npts, kSurBlock, 0, st>>>(sc, t, sd, (double2 *)n.spot, n.nr, n.nz);
  const __nv_bfloat16 *out = (const __nv_bfloat16 *)n.act.back();
  k_sur_fit<<<1, kFitBlock, 0, st>>>(sc, sd, out, (const double2 *)n.spot, n.nr, n.nz, n.n_samples, n.tol);
  const uint32_t nf = (n.nz + 1) * (n.nr + 1);
  k_sur_write<<<(nf + kSurBlock - 1) / kSurBlock, kSurBlock, 0, st>>>(sc, t, sd, out, (const double2 *)n.spot,
                                                                      n.nr, n.nz, fp32);
  note_launch(4);
}

int sur_build(SurNet &n, int n_layers, const int32_t *arch, int gmean_after, const int32_t *skip,
              const uint16_t *const *weights, const float *const *biases, uint32_t nr, uint32_t nz, double out_scale,
              double tol, uint32_t n_samples, std::string &err) {
  if (n_layers < 1 || n_layers > 64 || !arch || !skip || !weights || !biases) { err = "bad arguments"; return 1; }
  if (nr < 2 || nz < 2 || nr > 256 || nz > 512 || n_samples < 1 || n_samples > 4096 || !(tol >= 0.0) ||
      !(out_scale > 0.0)) {
    err = "bad mesh, sample count, tolerance or output scale";
    return 1;
  }
  n.nr = nr; n.nz = nz; n.out_scale = out_scale; n.tol = tol; n.n_samples = n_samples;
  n.gmean_after = gmean_after;
  uint32_t h = nz, wd = nr, c = 2;
  std::vector<uint32_t> hs, ws, cs;
  for (int l = 0; l < n_layers; ++l) {
    const int32_t *a5 = arch + 5 * l;
    const int ci = a5[0], co = a5[1], s = a5[2], u = a5[3];
    if ((uint32_t)ci != c || co < 1 || (s != 1 && s != 2) || (u != 1 && u != 2) || ci > 512) {
      err = "layer " + std::to_string(l) + ": channels or stride/upsampling do not chain";
      return 1;
    }
    n.arch.push_back({a5[0], a5[1], a5[2], a5[3], a5[4]});
    n.dims.insert(n.dims.end(), {1, ci, co, (int32_t)h, (int32_t)wd, s, u});
    h = (h * u - 1) / s + 1;
    wd = (wd * u - 1) / s + 1;
    c = co;
    hs.push_back(h); ws.push_back(wd); cs.push_back(c);
    n.hw.push_back((int)(h * wd));
    if (skip[l] >= 0 && (skip[l] >= l || hs[skip[l]] != h || ws[skip[l]] != wd || cs[skip[l]] != c)) {
      err = "layer " + std::to_string(l) + ": skip source does not match";
      return 1;
    }
    n.skip.push_back(skip[l]);
  }
  if (c != 2 || h != nz || wd != nr) { err = "the last layer must give 2 channels on the nz x nr mesh"; return 1; }
  if (gmean_after >= n_layers) { err = "plane-mean layer out of range"; return 1; }
  auto dm = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess; };
  for (int l = 0; l < n_layers; ++l) {
    const size_t nw = (size_t)n.arch[l][1] * n.arch[l][0] * 9, nb = n.arch[l][1];
    void *wp = nullptr, *bp = nullptr, *ap = nullptr;
    if (!dm(&wp, nw * 2) || !dm(&bp, nb * 4) || !dm(&ap, (size_t)cs[l] * hs[l] * ws[l] * 2)) {
      if (wp) cudaFree(wp);
      if (bp) cudaFree(bp);
      err = "device allocation failed";
      return 2;
    }
    n.w.push_back(wp);
    n.b.push_back((float *)bp);
    n.act.push_back(ap);
    if (cudaMemcpy(wp, weights[l], nw * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(bp, biases[l], nb * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
      err = "weight upload failed";
      return 2;
    }
    // the tensor-core kernel's weight tiles, laid out once
    void *tp = nullptr;
    const size_t tb = conv_tc_tile_bytes(n.dims.data() + 7 * l);
    if (tb) {
      if (!dm(&tp, tb)) {
        err = "device allocation failed";
        return 2;
      }
      conv_tc_prepare(n.dims.data() + 7 * l, wp, tp, nullptr);
    }
    n.wt.push_back(tp);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    err = "weight tile layout failed";
    return 2;
  }
  if (!dm(&n.x, (size_t)2 * nr * nz * 2) || !dm(&n.spot, (size_t)(nr + 1 + nz + n_samples) * 16) ||
      !dm(&n.d, sizeof(SurDev)) || cudaMemset(n.d, 0, sizeof(SurDev)) != cudaSuccess) {
    err = "device allocation failed";
    return 2;
  }
  return 0;
}

int sur_conv_state(const SurNet &n, int *tc_layers, unsigned int *err) {
  int k = 0;
  for (void *t : n.wt) k += (n.use_tc && t) ? 1 : 0;
  if (tc_layers) *tc_layers = k;
  SurDev h;
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(&h, n.d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
    return 1;
  if (err) *err = h.conv_err;
  return 0;
}

int sur_read(const SurNet &n, double *accepted, double *rejected, double *residual) {
  SurDev h;
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(&h, n.d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
    return 1;
  if (accepted) *accepted = h.n_accepted;
  if (rejected) *rejected = h.n_rejected;
  if (residual) *residual = h.residual;
  return 0;
}

}  // namespace hps
