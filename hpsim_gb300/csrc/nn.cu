// nn.cu -- the layers of the SCHEFF field surrogate: 3x3 convolutions with
// stride 1 or 2 and an optional nearest 2x upsampling of their input, bias
// and ReLU, a global-mean broadcast, the squared-error loss and Adam, forward
// and backward.  Activations and the weights the forward pass reads are
// BF16; every sum is FP32 (one thread owns each output and sums in a fixed
// order, so results do not depend on scheduling); master weights and
// gradients are FP32.
//
// Tensors are [batch][channel][z][r] (row-major, r fastest).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cooperative_groups.h>

#include <mutex>
#include <string>

#include "../../include/hpsim_gb300.h"
#include "internal.h"
#include "tc_ptx.cuh"

namespace hps {

namespace cg = cooperative_groups;

namespace {

constexpr int kNnBlock = 256;
constexpr int kCoTile = 8;  // output channels per thread in the forward conv
constexpr int kMaxCi = 512;  // input channels of one layer (weights staged in shared memory)
constexpr int kConvSmemMax = (kMaxCi * 9 * kCoTile + 2 * kCoTile * kNnBlock) * 4;

struct ConvShape {
  int B, Ci, Co, Hi, Wi, Ho, Wo, stride, up;  // up: 1 or 2 (nearest upsampling of the input first)
};

__device__ inline float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// input value at upsampled coordinates (Y, X) of channel plane p (zero outside)
__device__ inline float in_at(const __nv_bfloat16 *p, int Y, int X, int Hi, int Wi, int up) {
  const int Hu = Hi * up, Wu = Wi * up;
  if (Y < 0 || X < 0 || Y >= Hu || X >= Wu) return 0.0f;
  return bf(p[(Y / up) * Wi + X / up]);
}

// out[b][co][oy][ox] = bias[co] + sum_ci sum_ky,kx w[co][ci][ky][kx] in_up[b][ci][oy*S+ky-1][ox*S+kx-1],
// then ReLU when relu != 0, then (skip != null) BF16-rounded and added to
// skip[b][co][oy][ox].
// A cluster of `cl` CTAs (consecutive in x) shares one (pixel tile,
// kCoTile output channels, batch) and splits the input channels into cl
// contiguous ranges; inside a CTA `split` slices of threads take the range's
// channels in turn over P = kNnBlock / split pixels, each thread kCoTile
// sums.  A CTA stages its weights (contiguous runs of [co][ci][3][3], read
// coalesced) in shared memory as FP32 [ci][tap][co], so one input channel's
// 72 weights are read as broadcasts.  Slice partials are added in slice
// order, then rank 0 adds the other CTAs' sums through distributed shared
// memory in rank order: the result depends only on the launch shape.
template <int S, int U>
__global__ void __launch_bounds__(kNnBlock) k_conv_fwd(ConvShape s, int split, int cl, const __nv_bfloat16 *x,
                                                       const __nv_bfloat16 *w, const float *bias, int relu,
                                                       const __nv_bfloat16 *skip, __nv_bfloat16 *y) {
  extern __shared__ float conv_smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int P = kNnBlock / split;
  const int co0 = blockIdx.y * kCoTile, b = blockIdx.z;
  const int nco = min(kCoTile, s.Co - co0);
  const int cpr = (s.Ci + cl - 1) / cl;                 // input channels per rank
  const int ci_lo = min(s.Ci, rank * cpr), ci_hi = min(s.Ci, ci_lo + cpr);
  const int nci = ci_hi - ci_lo;
  float *ws = conv_smem;                                // [cpr][9][kCoTile]
  float *part = conv_smem + (size_t)cpr * 9 * kCoTile;  // [split][kCoTile][P]
  float *csum = part + (size_t)split * kCoTile * P;     // [kCoTile][P]: this CTA's sums
  const int slice = threadIdx.x / P, lp = threadIdx.x % P;
  const int npix = s.Ho * s.Wo;
  const int pix = (blockIdx.x / cl) * P + lp;
  const bool live = pix < npix;
  const int Y0 = (live ? pix / s.Wo : 0) * S - 1, X0 = (live ? pix % s.Wo : 0) * S - 1;
  const int plane = s.Hi * s.Wi;
  const __nv_bfloat16 *xb = x + ((size_t)b * s.Ci + ci_lo) * plane;
  // the window's offsets in an input plane and which taps fall inside it
  // (the same for every channel)
  int off[9];
  unsigned inside = 0;
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    const int Y = Y0 + t / 3, X = X0 + t % 3;
    const bool in = live && Y >= 0 && X >= 0 && Y < s.Hi * U && X < s.Wi * U;
    off[t] = in ? (Y / U) * s.Wi + X / U : 0;
    inside |= (unsigned)in << t;
  }
  // this thread's input windows, kPre channels at a time; the first ones are
  // loaded before the weights are staged, so both global reads overlap
  constexpr int kPre = 2;
  static_assert(kCoTile == 8, "the weights of one tap are read as two float4");
  float v[kPre][9];
  auto load = [&](int c0) {
#pragma unroll
    for (int j = 0; j < kPre; ++j) {
      const int c = c0 + j * split;
      const __nv_bfloat16 *p = xb + (size_t)max(0, min(c, nci - 1)) * plane;
      const unsigned m = c < nci ? inside : 0u;
#pragma unroll
      for (int t = 0; t < 9; ++t) v[j][t] = (m >> t) & 1u ? bf(p[off[t]]) : 0.0f;
    }
  };
  load(slice);
  if (nco < kCoTile)
    for (int i = threadIdx.x; i < nci * 9 * kCoTile; i += blockDim.x) ws[i] = 0.0f;
  __syncthreads();
  const int run = nci * 9;  // each output channel's weights of this range are contiguous
  const __nv_bfloat16 *w0 = w + ((size_t)co0 * s.Ci + ci_lo) * 9;
  if ((run & 7) == 0 && ((s.Ci * 9) & 7) == 0 && ((uintptr_t)w0 & 15) == 0) {
    // 16-byte loads: thread j takes 8 weights of output channel j % nco
    const int r8 = run / 8;
    for (int j = threadIdx.x; j < nco * r8; j += blockDim.x) {
      const int k = j % nco, q = j / nco;
      const uint4 u = *(const uint4 *)(w0 + (size_t)k * s.Ci * 9 + q * 8);
      const __nv_bfloat16 *h = (const __nv_bfloat16 *)&u;
#pragma unroll
      for (int e = 0; e < 8; ++e) ws[(q * 8 + e) * kCoTile + k] = bf(h[e]);
    }
  } else {
    for (int k = 0; k < nco; ++k) {
      const __nv_bfloat16 *wk = w0 + (size_t)k * s.Ci * 9;
      for (int r = threadIdx.x; r < run; r += blockDim.x) ws[r * kCoTile + k] = bf(wk[r]);
    }
  }
  __syncthreads();
  float acc[kCoTile];
#pragma unroll
  for (int k = 0; k < kCoTile; ++k) acc[k] = 0.0f;
  if (live) {
    for (int c0 = slice; c0 < nci; c0 += kPre * split) {
      if (c0 != slice) load(c0);
#pragma unroll
      for (int j = 0; j < kPre; ++j) {
        const int c = c0 + j * split;
        if (c >= nci) break;
        const float4 *wc = (const float4 *)(ws + c * 9 * kCoTile);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
          const float4 w0 = wc[2 * t], w1 = wc[2 * t + 1];
          acc[0] = fmaf(w0.x, v[j][t], acc[0]);
          acc[1] = fmaf(w0.y, v[j][t], acc[1]);
          acc[2] = fmaf(w0.z, v[j][t], acc[2]);
          acc[3] = fmaf(w0.w, v[j][t], acc[3]);
          acc[4] = fmaf(w1.x, v[j][t], acc[4]);
          acc[5] = fmaf(w1.y, v[j][t], acc[5]);
          acc[6] = fmaf(w1.z, v[j][t], acc[6]);
          acc[7] = fmaf(w1.w, v[j][t], acc[7]);
        }
      }
    }
  }
  if (split > 1) {
#pragma unroll
    for (int k = 0; k < kCoTile; ++k) part[((size_t)slice * kCoTile + k) * P + lp] = acc[k];
    __syncthreads();
    if (slice == 0) {
#pragma unroll
      for (int k = 0; k < kCoTile; ++k) {
        float a = part[(size_t)k * P + lp];
        for (int sl = 1; sl < split; ++sl) a += part[((size_t)sl * kCoTile + k) * P + lp];
        acc[k] = a;
      }
    }
  }
  if (cl > 1) {
    if (slice == 0)
#pragma unroll
      for (int k = 0; k < kCoTile; ++k) csum[k * P + lp] = acc[k];
    cluster.sync();
    if (rank == 0 && slice == 0)
      for (int r = 1; r < cl; ++r) {
        const float *rs = cluster.map_shared_rank(csum, r);
#pragma unroll
        for (int k = 0; k < kCoTile; ++k) acc[k] += rs[k * P + lp];
      }
    cluster.sync();  // the other CTAs' sums stay until rank 0 has read them
  }
  if (rank != 0 || slice != 0 || pix >= npix) return;
  for (int k = 0; k < nco; ++k) {
    float a = acc[k] + bias[co0 + k];
    if (relu && a < 0.0f) a = 0.0f;
    const size_t o = ((size_t)b * s.Co + co0 + k) * npix + pix;
    y[o] = skip ? __float2bfloat16_rn(bf(__float2bfloat16_rn(a)) + bf(skip[o])) : __float2bfloat16_rn(a);
  }
}

// dy masked by the ReLU of the forward output (y > 0), in FP32
__global__ void k_relu_bwd(const float *dy, const __nv_bfloat16 *y, int relu, float *dz, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dz[i] = (!relu || bf(y[i]) > 0.0f) ? dy[i] : 0.0f;
}

// dx[b][ci][iy][ix] = sum over the outputs that read input (iy, ix) through
// the upsampling and the 3x3 window of w[co][ci][ky][kx] dz[b][co][oy][ox]
__global__ void __launch_bounds__(kNnBlock) k_conv_bwd_data(ConvShape s, const float *dz, const __nv_bfloat16 *w,
                                                            float *dx) {
  const long long total = (long long)s.B * s.Ci * s.Hi * s.Wi;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(g % s.Wi);
    const int iy = (int)((g / s.Wi) % s.Hi);
    const int ci = (int)((g / ((long long)s.Wi * s.Hi)) % s.Ci);
    const int b = (int)(g / ((long long)s.Wi * s.Hi * s.Ci));
    float acc = 0.0f;
    for (int uy = 0; uy < s.up; ++uy)
      for (int ux = 0; ux < s.up; ++ux) {
        const int Y = iy * s.up + uy, X = ix * s.up + ux;  // upsampled position
        for (int ky = 0; ky < 3; ++ky) {
          const int ny = Y - ky + 1;  // = oy * stride
          if (ny < 0 || ny % s.stride) continue;
          const int oy = ny / s.stride;
          if (oy >= s.Ho) continue;
          for (int kx = 0; kx < 3; ++kx) {
            const int nx = X - kx + 1;
            if (nx < 0 || nx % s.stride) continue;
            const int ox = nx / s.stride;
            if (ox >= s.Wo) continue;
            for (int co = 0; co < s.Co; ++co)
              acc = fmaf(bf(w[((size_t)co * s.Ci + ci) * 9 + ky * 3 + kx]),
                         dz[(((size_t)b * s.Co + co) * s.Ho + oy) * s.Wo + ox], acc);
          }
        }
      }
    dx[g] = acc;
  }
}

// dw[co][ci][ky][kx] = sum_b,oy,ox dz[b][co][oy][ox] in_up[b][ci][oy*s+ky-1][ox*s+kx-1];
// db[co] = sum dz.  One block per (co, ci), a fixed tree over its threads.
__global__ void __launch_bounds__(kNnBlock) k_conv_bwd_weight(ConvShape s, const float *dz, const __nv_bfloat16 *x,
                                                              float *dw, float *db) {
  __shared__ float red[10][kNnBlock];
  const int co = blockIdx.x / s.Ci, ci = blockIdx.x % s.Ci;
  float acc[10];
#pragma unroll
  for (int t = 0; t < 10; ++t) acc[t] = 0.0f;
  const int npix = s.Ho * s.Wo;
  for (int g = threadIdx.x; g < s.B * npix; g += blockDim.x) {
    const int b = g / npix, pix = g % npix;
    const int oy = pix / s.Wo, ox = pix % s.Wo;
    const float d = dz[((size_t)b * s.Co + co) * npix + pix];
    if (d == 0.0f) continue;
    const __nv_bfloat16 *p = x + ((size_t)b * s.Ci + ci) * s.Hi * s.Wi;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky)
#pragma unroll
      for (int kx = 0; kx < 3; ++kx)
        acc[ky * 3 + kx] = fmaf(d, in_at(p, oy * s.stride + ky - 1, ox * s.stride + kx - 1, s.Hi, s.Wi, s.up),
                                acc[ky * 3 + kx]);
    acc[9] += d;
  }
#pragma unroll
  for (int t = 0; t < 10; ++t) red[t][threadIdx.x] = acc[t];
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off)
#pragma unroll
      for (int t = 0; t < 10; ++t) red[t][threadIdx.x] += red[t][threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x < 9) dw[((size_t)co * s.Ci + ci) * 9 + threadIdx.x] = red[threadIdx.x][0];
  if (threadIdx.x == 9 && ci == 0) {
    // every (co, ci) block summed the same dz: the bias gradient once, from ci 0
    db[co] = red[9][0];
  }
}

// y[b][c] += mean over the plane of y[b][c] (in place, BF16): each plane by
// one block, a fixed tree
__global__ void __launch_bounds__(kNnBlock) k_gmean_fwd(__nv_bfloat16 *y, int planes, int hw) {
  __shared__ float red[kNnBlock];
  __shared__ float mean;
  __nv_bfloat16 *p = y + (size_t)blockIdx.x * hw;
  float a = 0.0f;
  for (int i = threadIdx.x; i < hw; i += blockDim.x) a += bf(p[i]);
  red[threadIdx.x] = a;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) mean = red[0] / (float)hw;
  __syncthreads();
  for (int i = threadIdx.x; i < hw; i += blockDim.x) p[i] = __float2bfloat16_rn(bf(p[i]) + mean);
}

// backward of y' = y + mean(y): dy = dy' + mean(dy') (in place, FP32)
__global__ void __launch_bounds__(kNnBlock) k_gmean_bwd(float *d, int planes, int hw) {
  __shared__ float red[kNnBlock];
  __shared__ float mean;
  float *p = d + (size_t)blockIdx.x * hw;
  float a = 0.0f;
  for (int i = threadIdx.x; i < hw; i += blockDim.x) a += p[i];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) mean = red[0] / (float)hw;
  __syncthreads();
  for (int i = threadIdx.x; i < hw; i += blockDim.x) p[i] += mean;
}

// loss partial sums of wt (pred - target)^2 per block and dpred = 2 wt (pred -
// target) / n, wt = weight[i / per_sample] (1 without weights)
__global__ void __launch_bounds__(kNnBlock) k_mse(const __nv_bfloat16 *pred, const float *target, long long n,
                                                  const float *weight, long long per_sample, float *dpred,
                                                  float *partial) {
  __shared__ float red[kNnBlock];
  float a = 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float e = bf(pred[i]) - target[i];
    const float wt = weight ? weight[i / per_sample] : 1.0f;
    a = fmaf(wt * e, e, a);
    dpred[i] = 2.0f * wt * e / (float)n;
  }
  red[threadIdx.x] = a;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Adam on FP32 master weights, then their BF16 copy for the forward pass
__global__ void k_adam(float *w, __nv_bfloat16 *wb, const float *g, float *m, float *v, long long n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
  }
}

// y = a + b elementwise (skip connections: BF16 activations, FP32 gradients)
__global__ void k_add_bf16(const __nv_bfloat16 *a, const __nv_bfloat16 *b, __nv_bfloat16 *y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(bf(a[i]) + bf(b[i]));
}
__global__ void k_add_f32(const float *a, const float *b, float *y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = a[i] + b[i];
}

__global__ void k_to_bf16(const float *a, __nv_bfloat16 *b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}
__global__ void k_to_f32(const __nv_bfloat16 *a, float *b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = bf(a[i]);
}

int nn_grid(long long n) {
  long long g = (n + kNnBlock - 1) / kNnBlock;
  if (g < 1) g = 1;
  if (g > 152 * 8) g = 152 * 8;
  return (int)g;
}

ConvShape shape(const int32_t *d) {
  ConvShape s;
  s.B = d[0]; s.Ci = d[1]; s.Co = d[2]; s.Hi = d[3]; s.Wi = d[4]; s.stride = d[5]; s.up = d[6];
  s.Ho = (s.Hi * s.up - 1) / s.stride + 1;
  s.Wo = (s.Wi * s.up - 1) / s.stride + 1;
  return s;
}

bool shape_ok(const int32_t *d) {
  return d && d[0] > 0 && d[0] <= 65535 && d[1] > 0 && d[1] <= kMaxCi && d[2] > 0 && d[3] > 0 && d[4] > 0 &&
         (d[5] == 1 || d[5] == 2) && (d[6] == 1 || d[6] == 2);
}

}  // namespace

// pixels per block: 32, or 16 for planes of at most 16 pixels (their
// blocks then split the input channels 16 ways)
int conv_pixels(int npix) { return npix <= 16 ? 16 : 32; }

int conv_split(int ci, int P) {
  int sp = 1;
  while (sp < kNnBlock / P && sp * 2 <= ci) sp *= 2;
  return sp;
}

// CTAs per cluster: up to 8, while the layer has fewer CTAs than SMs,
// keeping at least 8 input channels per CTA (a CTA's fixed costs -- weight
// staging, barriers -- make more, thinner CTAs slower)
int conv_cluster(long long blocks, int ci) {
  int cl = 1;
  while (cl < 8 && blocks * cl * 2 <= 152 && ci / (cl * 2) >= 8) cl *= 2;
  return cl;
}

size_t conv_smem(int cpr, int split) {
  return ((size_t)cpr * 9 * kCoTile + (size_t)kCoTile * kNnBlock + (size_t)kCoTile * (kNnBlock / split)) *
         sizeof(float);
}

template <int S, int U>
void conv_launch(const ConvShape &s, const __nv_bfloat16 *x, const __nv_bfloat16 *w, const float *bias, int relu,
                 const __nv_bfloat16 *skip, __nv_bfloat16 *y, cudaStream_t st) {
  static PerDevice configured;
  configured.once([] {
    cudaFuncSetAttribute(k_conv_fwd<S, U>, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmemMax);
  });
  const int npix = s.Ho * s.Wo;
  const int P0 = conv_pixels(npix);
  const int ntiles = (npix + P0 - 1) / P0, nct = (s.Co + kCoTile - 1) / kCoTile;
  const int cl = conv_cluster((long long)ntiles * nct * s.B, s.Ci);
  const int cpr = (s.Ci + cl - 1) / cl;
  const int split = conv_split(cpr, P0), P = kNnBlock / split;
  const int ptiles = (npix + P - 1) / P;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ptiles * cl, nct, s.B);
  cfg.blockDim = dim3(kNnBlock);
  cfg.dynamicSmemBytes = conv_smem(cpr, split);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_conv_fwd<S, U>, s, split, cl, x, w, bias, relu, skip, y);
}

void nn_conv_forward(const int32_t *dims, const void *x, const void *w, const float *bias, int relu,
                     const void *skip, void *y, cudaStream_t st) {
  const ConvShape s = shape(dims);
  auto xb = (const __nv_bfloat16 *)x, wb = (const __nv_bfloat16 *)w, kb = (const __nv_bfloat16 *)skip;
  auto yb = (__nv_bfloat16 *)y;
  if (s.stride == 1 && s.up == 1) conv_launch<1, 1>(s, xb, wb, bias, relu, kb, yb, st);
  else if (s.stride == 2 && s.up == 1) conv_launch<2, 1>(s, xb, wb, bias, relu, kb, yb, st);
  else if (s.stride == 1) conv_launch<1, 2>(s, xb, wb, bias, relu, kb, yb, st);
  else conv_launch<2, 2>(s, xb, wb, bias, relu, kb, yb, st);
  note_launch();
}

void nn_gmean_forward(void *y, int planes, int hw, cudaStream_t st) {
  k_gmean_fwd<<<planes, kNnBlock, 0, st>>>((__nv_bfloat16 *)y, planes, hw);
  note_launch();
}

// ---- the forward convolution on the tensor cores (inference) ---------------
// One CTA computes 128 output pixels (the MMA's M) x all output channels
// (N = c_out rounded up to 16) of one batch plane as an implicit GEMM over
// K = (tap, input channel): D[p][co] = sum_k A[p][k] W[co][k], A[p][(t, ci)]
// = the input at pixel p's tap t of channel ci.  A cluster of cl CTAs
// splits the input channels (cpr = c_in / cl each, a power of two); its CTAs
// add their accumulators through distributed shared memory in rank order.
// A CTA first copies the input rows its pixels read (its channels only) into
// shared memory, then per chunk of 64 K values four producer warps write the
// A tile (one pixel row each, 16-byte stores, 128-byte swizzle) from there
// while the chunk's weight tile arrives by bulk copy; one thread of the
// fifth warp issues the BF16 MMAs (FP32 accumulation in tensor memory).  The
// weights are laid out once per layer as those tiles (conv_tc_prepare).
// Every wait is bounded; a wait that gives up sets *err and the CTA drains
// its copies and MMAs, still takes part in both cluster barriers, and frees
// its tensor memory.
namespace {

constexpr int kCvThreads = 160;
constexpr int kCvStages = 4;
constexpr size_t kCvSlabMax = 64 * 1024;
constexpr size_t kCvSmemMax = 220 * 1024;

struct ConvTc {
  ConvShape s;
  int tiles;   // 128-pixel tiles of an output plane
  int cl;      // CTAs per cluster
  int cpr;     // input channels per CTA (power of two)
  int lg;      // log2(cpr)
  int kc;      // 64-wide K chunks per CTA (9 cpr rounded up)
  int np;      // MMA N: c_out rounded up to 16
  int cols;    // tensor-memory columns
  int rows;    // input rows a tile reads (largest over the tiles)
  uint32_t bt;    // bytes of one weight tile (np rows of 128 bytes)
  uint32_t smem;  // dynamic shared memory
};

// the source rows [r0, r1] that output pixels [128 tile, 128 tile + 127] read
__host__ __device__ inline void cv_rows(const ConvShape &s, int tile, int &r0, int &r1) {
  const int npix = s.Ho * s.Wo, p0 = tile * 128, p1 = min(npix, p0 + 128) - 1;
  const int ylo = (p0 / s.Wo) * s.stride - 1, yhi = (p1 / s.Wo) * s.stride + 1;
  r0 = ylo < 0 ? 0 : ylo / s.up;
  r1 = min(s.Hi - 1, yhi / s.up);
}

inline bool conv_tc_ok(const ConvShape &s) {
  return s.Co <= 128 && s.Ci >= 1 && s.Ci <= kMaxCi && (s.Ci & (s.Ci - 1)) == 0 && s.Wi % 2 == 0 && s.B <= 65535;
}

inline ConvTc conv_tc_plan(const ConvShape &s) {
  ConvTc p{};
  p.s = s;
  const int npix = s.Ho * s.Wo;
  p.tiles = (npix + 127) / 128;
  p.np = (s.Co + 15) / 16 * 16;
  p.cols = 32;
  while (p.cols < p.np) p.cols *= 2;
  p.rows = 0;
  for (int t = 0; t < p.tiles; ++t) {
    int r0, r1;
    cv_rows(s, t, r0, r1);
    p.rows = std::max(p.rows, r1 - r0 + 1);
  }
  // split the input channels while the layer has fewer CTAs than SMs (a
  // CTA keeps at least 8 channels), and until a CTA's input rows fit
  int cl = 1;
  while (cl < 8 && s.Ci % (2 * cl) == 0 && s.Ci / (2 * cl) >= 8 && (long long)p.tiles * 2 * cl * s.B <= 152) cl *= 2;
  while (cl < 8 && s.Ci % (2 * cl) == 0 && (size_t)(s.Ci / cl) * p.rows * s.Wi * 2 > kCvSlabMax) cl *= 2;
  p.cl = cl;
  p.cpr = s.Ci / cl;
  p.lg = 0;
  while ((1 << p.lg) < p.cpr) ++p.lg;
  p.kc = (9 * p.cpr + 63) / 64;
  p.bt = (uint32_t)p.np * 128;
  const size_t slab = ((size_t)p.cpr * p.rows * s.Wi * 2 + 15) / 16 * 16;
  p.smem = (uint32_t)(1024 + (size_t)kCvStages * (16384 + p.bt) + slab);
  return p;
}

// W[co][ci][3][3] as the kernel's weight tiles: CTA rank r, chunk c, row co,
// column j holds K value k = 64 c + j = (tap t = k / cpr, channel r cpr + k %
// cpr); zero beyond the channels, taps and output channels
__global__ void k_conv_tc_prep(const __nv_bfloat16 *w, ConvTc p, unsigned char *wt) {
  const long long total = (long long)p.cl * p.kc * p.np * 64;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e % 64), n = (int)((e / 64) % p.np), c = (int)((e / (64 * p.np)) % p.kc);
    const int r = (int)(e / (64LL * p.np * p.kc));
    const int k = 64 * c + j, t = k >> p.lg, ci = r * p.cpr + (k & (p.cpr - 1));
    const __nv_bfloat16 v =
        (n < p.s.Co && t < 9 && ci < p.s.Ci) ? w[((size_t)n * p.s.Ci + ci) * 9 + t] : __float2bfloat16_rn(0.0f);
    *(__nv_bfloat16 *)(wt + (size_t)(r * p.kc + c) * p.bt + tc_swz((uint32_t)n, (uint32_t)j)) = v;
  }
}

template <int S, int U>
__global__ void __launch_bounds__(kCvThreads, 1)
    k_conv_tc(ConvTc p, const __nv_bfloat16 *x, const unsigned char *wt, const float *bias, int relu,
              const __nv_bfloat16 *skip, __nv_bfloat16 *y, unsigned int *err) {
  extern __shared__ unsigned char cv_raw[];
  __shared__ uint64_t full[kCvStages], empty[kCvStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float sbias[128];
  cg::cluster_group cluster = cg::this_cluster();
  const ConvShape &s = p.s;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rank = (int)cluster.block_rank(), tile = blockIdx.x / p.cl, b = blockIdx.y;
  const int npix = s.Ho * s.Wo, cpr = p.cpr, kc = p.kc;
  const uint32_t bt = p.bt, stage = 16384 + bt;
  unsigned char *sm = (unsigned char *)(((uintptr_t)cv_raw + 1023) & ~(uintptr_t)1023);
  __nv_bfloat16 *slab = (__nv_bfloat16 *)(sm + kCvStages * stage);
  volatile int *abort = &abort_flag;
  int r0, r1;
  cv_rows(s, tile, r0, r1);
  const int R = r1 - r0 + 1, plane = R * s.Wi;

  if (tid < (uint32_t)s.Co) sbias[tid] = bias[tid];
  if (tid == 0) {
    for (int i = 0; i < kCvStages; ++i) {
      mbar_init(&full[i], 128 + 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // the first stages' weight tiles in flight before the input rows are read
    for (int i = 0; i < kCvStages && i < kc; ++i) {
      mbar_arrive_tx(&full[i], bt);
      bulk_g2s(sm + i * stage + 16384, wt + ((size_t)rank * kc + i) * bt, bt, &full[i]);
    }
  }
  // this CTA's input rows, two BF16 values per load (rows are even-sized)
  if (warp < 4) {
    const uint32_t half = (uint32_t)plane / 2, words = (uint32_t)cpr * half;
    const uint32_t *src0 =
        (const uint32_t *)(x + (((size_t)b * s.Ci + (size_t)rank * cpr) * s.Hi + r0) * s.Wi);
    const uint32_t cstride = (uint32_t)(s.Hi * s.Wi) / 2;  // words between channel planes
    uint32_t ci = tid / half, o = tid - ci * half;
    for (uint32_t q = tid; q < words; q += 128) {
      ((uint32_t *)slab)[q] = __ldg(src0 + (size_t)ci * cstride + o);
      o += 128;
      while (o >= half) {
        o -= half;
        ++ci;
      }
    }
  }
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_slot)),
                 "r"(p.cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  bool issued_mma = false;
  const int m = (int)tid, pix = tile * 128 + m;
  const bool live = warp < 4 && pix < npix;
  const int oy = live ? pix / s.Wo : 0, ox = live ? pix % s.Wo : 0;
  // offset of each tap's input value in a channel's rows (-1: padding or a dead pixel)
  int off[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    const int Y = oy * S + t / 3 - 1, X = ox * S + t % 3 - 1;
    off[t] = (live && Y >= 0 && X >= 0 && Y < s.Hi * U && X < s.Wi * U) ? (Y / U - r0) * s.Wi + X / U : -1;
  }

  if (warp < 4) {
    // ---- producers ----
    const unsigned char *wsrc = wt + (size_t)rank * kc * bt;
    unsigned char *arow = nullptr;
    for (int c = 0; c < kc && !*abort; ++c) {
      const int st = c % kCvStages, use = c / kCvStages;
      if (use > 0 && !mbar_wait(&empty[st], (use - 1) & 1, abort)) break;
      unsigned char *sb = sm + st * stage;
      if (tid == 0 && use > 0) {
        mbar_arrive_tx(&full[st], bt);
        bulk_g2s(sb + 16384, wsrc + (size_t)c * bt, bt, &full[st]);
      }
      arow = sb + (m >> 3) * 1024 + (m & 7) * 128;
      const unsigned short *sl = (const unsigned short *)slab;
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k0 = 64 * c + 8 * e;
        uint32_t w[4];
        if (cpr >= 8) {
          // the 8 values share one tap (uniform over the CTA): 8 channels at one offset
          const int t = k0 >> p.lg, ci0 = k0 & (cpr - 1);
          const int o = t < 9 ? off[0] : -1;
          int ot = o;
#pragma unroll
          for (int tt = 1; tt < 9; ++tt) ot = t == tt ? off[tt] : ot;
          if (t >= 9) ot = -1;
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const uint32_t lo = ot >= 0 ? sl[(ci0 + 2 * h) * plane + ot] : 0u;
            const uint32_t hi = ot >= 0 ? sl[(ci0 + 2 * h + 1) * plane + ot] : 0u;
            w[h] = lo | (hi << 16);
          }
        } else {
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            uint32_t pair[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int k = k0 + 2 * h + j, t = k >> p.lg, ci = k & (cpr - 1);
              int ot = off[0];
#pragma unroll
              for (int tt = 1; tt < 9; ++tt) ot = t == tt ? off[tt] : ot;
              pair[j] = (t < 9 && ot >= 0) ? sl[ci * plane + ot] : 0u;
            }
            w[h] = pair[0] | (pair[1] << 16);
          }
        }
        *(uint4 *)(arow + (((e ^ (m & 7)) & 7) << 4)) = make_uint4(w[0], w[1], w[2], w[3]);
      }
      fence_async_smem();
      mbar_arrive(&full[st]);
    }
  } else if (lane == 0) {
    // ---- the MMA thread ----
    const uint32_t idesc = tc_idesc((uint32_t)p.np);
    for (int c = 0; c < kc; ++c) {
      const int st = c % kCvStages, use = c / kCvStages;
      if (!mbar_wait(&full[st], use & 1, abort)) break;
      tc_fence_after();
      const uint32_t a0 = tc_smem(sm + st * stage);
      const uint64_t ad = tc_desc(a0), bd = tc_desc(a0 + 16384);
#pragma unroll
      for (uint32_t ks = 0; ks < 4; ++ks) tc_mma(tmem, ad + 2 * ks, bd + 2 * ks, idesc, (c | (int)ks) != 0);
      issued_mma = true;
      tc_commit(&empty[st]);
    }
    if (issued_mma) tc_commit(&done);
  }

  // ---- epilogue ----
  // output (co, this pixel) from its sum a, the bias, the ReLU and the skip value sk
  auto emit = [&](int co, float a, float sk) {
    a += sbias[co];
    if (relu && a < 0.0f) a = 0.0f;
    const size_t o = ((size_t)b * s.Co + co) * npix + pix;
    y[o] = skip ? __float2bfloat16_rn(__bfloat162float(__float2bfloat16_rn(a)) + sk) : __float2bfloat16_rn(a);
  };
  // the skip value of (co, this pixel), read-only (loaded ahead of the stores)
  auto skip_at = [&](int co) -> float {
    if (!skip) return 0.0f;
    const unsigned short u = __ldg((const unsigned short *)skip + ((size_t)b * s.Co + co) * npix + pix);
    return __bfloat162float(__ushort_as_bfloat16(u));
  };
  bool ok = false;
  if (warp < 4) {
    ok = !*abort && mbar_wait(&done, 0, abort);
    if (ok) {
      tc_fence_after();
      const uint32_t tl = tmem + ((32 * warp) << 16);
      float *red = (float *)sm;  // [np][128]: the stages are free once every MMA completed
      for (int c0 = 0; c0 < p.np; c0 += 16) {
        float v[16];
        tc_ld16(tl + (uint32_t)c0, v);
        if (p.cl == 1) {
          if (live) {
            float sk[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) sk[k] = c0 + k < s.Co ? skip_at(c0 + k) : 0.0f;
#pragma unroll
            for (int k = 0; k < 16; ++k)
              if (c0 + k < s.Co) emit(c0 + k, v[k], sk[k]);
          }
        } else {
#pragma unroll
          for (int k = 0; k < 16; ++k) red[(c0 + k) * 128 + m] = v[k];
        }
      }
    }
    tc_fence_before();
  }
  if (p.cl > 1) {
    cluster.sync();  // every CTA's sums are in its shared memory
    // rank r: output channels [r np / cl, (r + 1) np / cl), the CTAs' sums
    // in rank order; four channels' loads from every rank (and their skip
    // values) in flight at once
    const int per = p.np / p.cl, cend = min((rank + 1) * per, s.Co);
    if (warp < 4 && live) {
      const float *rk[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) rk[q] = cluster.map_shared_rank((float *)sm, q < p.cl ? q : 0);
      for (int co0 = rank * per; co0 < cend; co0 += 4) {
        float v[4][8], sk[4];
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          const int co = co0 + g;
          const bool valid = co < cend;
#pragma unroll
          for (int q = 0; q < 8; ++q) v[g][q] = (valid && q < p.cl) ? rk[q][co * 128 + m] : 0.0f;
          sk[g] = valid ? skip_at(co) : 0.0f;
        }
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          if (co0 + g >= cend) break;
          float a = 0.0f;
#pragma unroll
          for (int q = 0; q < 8; ++q) a += v[g][q];
          emit(co0 + g, a, sk[g]);
        }
      }
    }
    cluster.sync();  // no CTA leaves while the others read its sums
  }
  __syncthreads();
  if (*abort) {
    if (tid == 0) atomicOr(err, 1u);
    if (warp == 4 && lane == 0 && issued_mma) {
      tc_commit(&done);
      int dummy = 0;
      (void)mbar_wait(&done, 0, &dummy);
    }
    const uint64_t t0 = tc_now();
    while (tc_now() - t0 < 100000ull) {
    }
    __syncthreads();
  }
  if (warp == 4) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)p.cols)
                 : "memory");
  }
}

template <int S, int U>
void conv_tc_launch(const ConvTc &p, const __nv_bfloat16 *x, const unsigned char *wt, const float *bias, int relu,
                    const __nv_bfloat16 *skip, __nv_bfloat16 *y, unsigned int *err, cudaStream_t st) {
  static PerDevice configured;
  configured.once([] {
    cudaFuncSetAttribute(k_conv_tc<S, U>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCvSmemMax);
  });
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.tiles * p.cl, p.s.B);
  cfg.blockDim = dim3(kCvThreads);
  cfg.dynamicSmemBytes = p.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p.cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_conv_tc<S, U>, p, x, wt, bias, relu, skip, y, err);
}

}  // namespace

size_t conv_tc_tile_bytes(const int32_t *dims) {
  const ConvShape s = shape(dims);
  if (!conv_tc_ok(s)) return 0;
  const ConvTc p = conv_tc_plan(s);
  if (p.smem > kCvSmemMax) return 0;
  return (size_t)p.cl * p.kc * p.bt;
}

void conv_tc_prepare(const int32_t *dims, const void *w, void *tiles, cudaStream_t st) {
  const ConvTc p = conv_tc_plan(shape(dims));
  const long long total = (long long)p.cl * p.kc * p.np * 64;
  const int blocks = (int)std::min<long long>((total + kNnBlock - 1) / kNnBlock, 1024);
  k_conv_tc_prep<<<blocks, kNnBlock, 0, st>>>((const __nv_bfloat16 *)w, p, (unsigned char *)tiles);
  note_launch();
}

void nn_conv_forward_tc(const int32_t *dims, const void *x, const void *tiles, const float *bias, int relu,
                        const void *skip, void *y, unsigned int *err, cudaStream_t st) {
  const ConvTc p = conv_tc_plan(shape(dims));
  auto xb = (const __nv_bfloat16 *)x, kb = (const __nv_bfloat16 *)skip;
  auto wt = (const unsigned char *)tiles;
  auto yb = (__nv_bfloat16 *)y;
  if (p.s.stride == 1 && p.s.up == 1) conv_tc_launch<1, 1>(p, xb, wt, bias, relu, kb, yb, err, st);
  else if (p.s.stride == 2 && p.s.up == 1) conv_tc_launch<2, 1>(p, xb, wt, bias, relu, kb, yb, err, st);
  else if (p.s.stride == 1) conv_tc_launch<1, 2>(p, xb, wt, bias, relu, kb, yb, err, st);
  else conv_tc_launch<2, 2>(p, xb, wt, bias, relu, kb, yb, err, st);
  note_launch();
}

}  // namespace hps

extern "C" {

using namespace hps;

static hps_status nn_status(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (hps_status)set_error(HPS_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
  return HPS_OK;
}

hps_status hps_nn_conv_forward(const int32_t dims[7], const void *x, const void *w, const float *bias, int relu,
                               const void *skip, void *y, void *stream) {
  if (!shape_ok(dims) || !x || !w || !bias || !y) return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_forward: bad argument");
  nn_conv_forward(dims, x, w, bias, relu, skip, y, (cudaStream_t)stream);
  return nn_status("nn_conv_forward");
}

hps_status hps_nn_conv_tc_tile_bytes(const int32_t dims[7], uint64_t *bytes) {
  if (!shape_ok(dims) || !bytes) return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_tc_tile_bytes: bad argument");
  *bytes = conv_tc_tile_bytes(dims);
  return HPS_OK;
}

hps_status hps_nn_conv_tc_prepare(const int32_t dims[7], const void *w, void *tiles, void *stream) {
  if (!shape_ok(dims) || !w || !tiles || !conv_tc_tile_bytes(dims))
    return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_tc_prepare: bad argument or shape");
  conv_tc_prepare(dims, w, tiles, (cudaStream_t)stream);
  return nn_status("nn_conv_tc_prepare");
}

hps_status hps_nn_conv_forward_tiles(const int32_t dims[7], const void *x, const void *tiles, const float *bias,
                                     int relu, const void *skip, void *y, unsigned int *err, void *stream) {
  if (!shape_ok(dims) || !x || !tiles || !bias || !y || !err || !conv_tc_tile_bytes(dims))
    return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_forward_tiles: bad argument or shape");
  nn_conv_forward_tc(dims, x, tiles, bias, relu, skip, y, err, (cudaStream_t)stream);
  return nn_status("nn_conv_forward_tiles");
}

hps_status hps_nn_conv_forward_tc(const int32_t dims[7], const void *x, const void *w, const float *bias, int relu,
                                  const void *skip, void *y, void *stream) {
  if (!shape_ok(dims) || !x || !w || !bias || !y) return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_forward_tc: bad argument");
  const size_t tb = conv_tc_tile_bytes(dims);
  if (!tb) return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_forward_tc: layer shape not taken by the tensor-core kernel");
  cudaStream_t st = (cudaStream_t)stream;
  void *tiles = nullptr;
  unsigned int *err = nullptr;
  if (cudaMalloc(&tiles, tb) != cudaSuccess || cudaMalloc((void **)&err, sizeof(unsigned int)) != cudaSuccess) {
    cudaFree(tiles);
    return nn_status("nn_conv_forward_tc: allocation");
  }
  cudaMemsetAsync(err, 0, sizeof(unsigned int), st);
  conv_tc_prepare(dims, w, tiles, st);
  nn_conv_forward_tc(dims, x, tiles, bias, relu, skip, y, err, st);
  unsigned int h = 0;
  cudaMemcpyAsync(&h, err, sizeof(h), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(tiles);
  cudaFree(err);
  if (e != cudaSuccess) return (hps_status)set_error(HPS_ERR_CUDA, (std::string("nn_conv_forward_tc: ") + cudaGetErrorString(e)).c_str());
  if (h) return (hps_status)set_error(HPS_ERR_CUDA, "nn_conv_forward_tc: a pipeline wait timed out");
  return nn_status("nn_conv_forward_tc");
}

hps_status hps_nn_conv_backward(const int32_t dims[7], const void *x, const void *w, const void *y, int relu,
                                const float *dy, float *dz, float *dx, float *dw, float *db, void *stream) {
  if (!shape_ok(dims) || !x || !w || !y || !dy || !dz || !dw || !db)
    return (hps_status)set_error(HPS_ERR_INVALID, "nn_conv_backward: bad argument");
  const ConvShape s = shape(dims);
  cudaStream_t st = (cudaStream_t)stream;
  const long long nout = (long long)s.B * s.Co * s.Ho * s.Wo;
  k_relu_bwd<<<nn_grid(nout), kNnBlock, 0, st>>>(dy, (const __nv_bfloat16 *)y, relu, dz, nout);
  k_conv_bwd_weight<<<s.Co * s.Ci, kNnBlock, 0, st>>>(s, dz, (const __nv_bfloat16 *)x, dw, db);
  note_launch(2);
  if (dx) {
    const long long nin = (long long)s.B * s.Ci * s.Hi * s.Wi;
    k_conv_bwd_data<<<nn_grid(nin), kNnBlock, 0, st>>>(s, dz, (const __nv_bfloat16 *)w, dx);
    note_launch();
  }
  return nn_status("nn_conv_backward");
}

hps_status hps_nn_gmean_forward(void *y, int32_t planes, int32_t hw, void *stream) {
  if (!y || planes <= 0 || hw <= 0) return (hps_status)set_error(HPS_ERR_INVALID, "nn_gmean_forward: bad argument");
  nn_gmean_forward(y, planes, hw, (cudaStream_t)stream);
  return nn_status("nn_gmean_forward");
}

hps_status hps_nn_gmean_backward(float *d, int32_t planes, int32_t hw, void *stream) {
  if (!d || planes <= 0 || hw <= 0) return (hps_status)set_error(HPS_ERR_INVALID, "nn_gmean_backward: bad argument");
  k_gmean_bwd<<<planes, kNnBlock, 0, (cudaStream_t)stream>>>(d, planes, hw);
  note_launch();
  return nn_status("nn_gmean_backward");
}

hps_status hps_nn_mse(const void *pred, const float *target, int64_t n, const float *weight, int64_t per_sample,
                      float *dpred, float *partial, int32_t nblocks, void *stream) {
  if (!pred || !target || !dpred || !partial || n <= 0 || nblocks <= 0 || (weight && per_sample <= 0))
    return (hps_status)set_error(HPS_ERR_INVALID, "nn_mse: bad argument");
  k_mse<<<nblocks, kNnBlock, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)pred, target, n, weight, per_sample,
                                                        dpred, partial);
  note_launch();
  return nn_status("nn_mse");
}

hps_status hps_nn_adam(float *w, void *w_bf16, const float *g, float *m, float *v, int64_t n, float lr, float b1,
                       float b2, float eps, int32_t step, void *stream) {
  if (!w || !g || !m || !v || n <= 0 || step < 1) return (hps_status)set_error(HPS_ERR_INVALID, "nn_adam: bad argument");
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adam<<<nn_grid(n), kNnBlock, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16 *)w_bf16, g, m, v, n, lr, b1, b2, eps,
                                                             c1, c2);
  note_launch();
  return nn_status("nn_adam");
}

hps_status hps_nn_add(const void *a, const void *b, void *y, int64_t n, int bf16, void *stream) {
  if (!a || !b || !y || n <= 0) return (hps_status)set_error(HPS_ERR_INVALID, "nn_add: bad argument");
  if (bf16) k_add_bf16<<<nn_grid(n), kNnBlock, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)a,
                                                                            (const __nv_bfloat16 *)b,
                                                                            (__nv_bfloat16 *)y, n);
  else k_add_f32<<<nn_grid(n), kNnBlock, 0, (cudaStream_t)stream>>>((const float *)a, (const float *)b, (float *)y, n);
  note_launch();
  return nn_status("nn_add");
}

hps_status hps_nn_convert(const void *src, void *dst, int64_t n, int to_bf16, void *stream) {
  if (!src || !dst || n <= 0) return (hps_status)set_error(HPS_ERR_INVALID, "nn_convert: bad argument");
  if (to_bf16) k_to_bf16<<<nn_grid(n), kNnBlock, 0, (cudaStream_t)stream>>>((const float *)src, (__nv_bfloat16 *)dst, n);
  else k_to_f32<<<nn_grid(n), kNnBlock, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)src, (float *)dst, n);
  note_launch();
  return nn_status("nn_convert");
}

}  // extern "C"
