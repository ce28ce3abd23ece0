// plot.cu -- headless plot data of a beam into device buffers: the
// reference's graphics kernels (src/graphics/inc/graphics_kernel.cu,
// launchers src/graphics/src/graphics_kernel_call.cu) with the OpenGL
// vertex buffers they filled replaced by plain device memory.  Windows,
// shaders and GL interop are not built.
//
// Coordinates are read as FP64 values: FP64 beams directly, FP32 beams as
// offset + synchronous particle (the same sum the coordinate getter forms).
#include <cuda_runtime.h>

#include "internal.h"

namespace hps {

namespace {

__device__ inline double cval(const PlotCoord &c, uint32_t i) {
  return c.d ? c.d[i] : c.off + (double)c.f[i];
}

// Set2dPhaseSpaceDataKernel (graphics_kernel.cu:52-75): live particles as
// (float)(x, y), lost ones at the origin
__global__ void k_plot_points(PlotCoord x, PlotCoord y, const uint32_t *loss, uint32_t n, float2 *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = loss[i] == 0u ? make_float2((float)cval(x, i), (float)cval(y, i)) : make_float2(0.0f, 0.0f);
}

// max / min that skip NaN candidates, as BlockMaxMin2DKernel's tree
// (graphics_kernel.cu:86-165): a NaN is replaced by any number
__device__ inline double nmax(double a, double b) { return isnan(b) ? a : (isnan(a) || a < b ? b : a); }
__device__ inline double nmin(double a, double b) { return isnan(b) ? a : (isnan(a) || a > b ? b : a); }

constexpr int kPlotBlock = 256;

// FindMaxMin2D: (xmax, xmin, ymax, ymin) over the particles; with a loss
// array, a lost particle's seat holds particle 0's coordinates (the
// reference fills them with r_x[0], r_y[0]), so particle 0 always counts.
// Block partials, then the last block combines them in block order.
__global__ void __launch_bounds__(kPlotBlock) k_plot_maxmin(PlotCoord x, PlotCoord y, const uint32_t *loss,
                                                            uint32_t n, double *part, unsigned int *counter,
                                                            double *out) {
  __shared__ double s[4][kPlotBlock];
  __shared__ int last;
  const double x0 = cval(x, 0), y0 = cval(y, 0);
  double a = x0, b = x0, c = y0, d = y0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool use = !loss || loss[i] == 0u;
    const double xv = use ? cval(x, i) : x0, yv = use ? cval(y, i) : y0;
    a = nmax(a, xv); b = nmin(b, xv); c = nmax(c, yv); d = nmin(d, yv);
  }
  s[0][threadIdx.x] = a; s[1][threadIdx.x] = b; s[2][threadIdx.x] = c; s[3][threadIdx.x] = d;
  __syncthreads();
  for (int off = kPlotBlock / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      s[0][threadIdx.x] = nmax(s[0][threadIdx.x], s[0][threadIdx.x + off]);
      s[1][threadIdx.x] = nmin(s[1][threadIdx.x], s[1][threadIdx.x + off]);
      s[2][threadIdx.x] = nmax(s[2][threadIdx.x], s[2][threadIdx.x + off]);
      s[3][threadIdx.x] = nmin(s[3][threadIdx.x], s[3][threadIdx.x + off]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) part[blockIdx.x * 4 + threadIdx.x] = s[threadIdx.x][0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x < 4) {
    const int k = threadIdx.x;
    double v = __ldcg(part + k);
    for (uint32_t blk = 1; blk < gridDim.x; ++blk) {
      const double w = __ldcg(part + blk * 4 + k);
      v = (k & 1) ? nmin(v, w) : nmax(v, w);
    }
    out[k] = v;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// HistogramKernel (graphics_kernel.cu:229-252) per block in shared memory,
// added to the table as integers.  The bin is (uint)floorf((x - min) / w)
// with w = (max - min) / nbins: the quotient rounded to FP32, floored, and
// converted with the GPU's saturating float-to-unsigned conversion (below
// 0 and NaN give 0), then read as int; bins 0 .. nbins-2 count, an int
// below 0 counts in bin 0, above nbins-1 in the last bin, and exactly
// nbins-1 is not counted (the reference's range tests skip it).
__global__ void __launch_bounds__(kPlotBlock) k_plot_hist(PlotCoord x, const uint32_t *loss, uint32_t n, uint32_t nb,
                                                          double mn, double w, uint32_t *hist) {
  extern __shared__ uint32_t h[];
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x) h[k] = 0u;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (loss[i] != 0u) continue;
    const float q = (float)((cval(x, i) - mn) / w);
    const int bin = (int)__float2uint_rz(floorf(q));
    if (bin >= 0 && bin < (int)nb - 1) atomicAdd(h + bin, 1u);
    else if (bin < 0) atomicAdd(h, 1u);
    else if (bin > (int)nb - 1) atomicAdd(h + nb - 1, 1u);
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < nb; k += blockDim.x)
    if (h[k]) atomicAdd(hist + k, h[k]);
}

// Histogram2DKernel (graphics_kernel.cu:272-299): live particles inside
// [xmin, xmax] x [ymin, ymax]; bins (uint)floorf((v - min) / d), clamped to
// the last bin
__global__ void k_plot_hist2d(PlotCoord x, PlotCoord y, const uint32_t *loss, uint32_t n, double xmin, double xmax,
                              double ymin, double ymax, uint32_t nx, uint32_t ny, uint32_t *hist) {
  const double dx = (xmax - xmin) / nx, dy = (ymax - ymin) / ny;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double xv = cval(x, i), yv = cval(y, i);
    if (loss[i] != 0u || !(xv >= xmin && xv <= xmax && yv >= ymin && yv <= ymax)) continue;
    uint32_t ix = __float2uint_rz(floorf((float)((xv - xmin) / dx)));
    uint32_t iy = __float2uint_rz(floorf((float)((yv - ymin) / dy)));
    if (ix > nx - 1) ix = nx - 1;
    if (iy > ny - 1) iy = ny - 1;
    atomicAdd(hist + iy * nx + ix, 1u);
  }
}

int plot_grid(uint32_t n) {
  uint32_t g = (n + kPlotBlock - 1) / kPlotBlock;
  if (g < 1) g = 1;
  if (g > 4u * 152u) g = 4u * 152u;
  return (int)g;
}

}  // namespace

void plot_points(const PlotCoord &x, const PlotCoord &y, const uint32_t *loss, uint32_t n, float2 *out,
                 cudaStream_t st) {
  k_plot_points<<<plot_grid(n), kPlotBlock, 0, st>>>(x, y, loss, n, out);
  note_launch();
}

void plot_maxmin(const PlotCoord &x, const PlotCoord &y, const uint32_t *loss, uint32_t n, PassScratch scr,
                 double *out, cudaStream_t st) {
  k_plot_maxmin<<<plot_grid(n), kPlotBlock, 0, st>>>(x, y, loss, n, scr.part, scr.counter, out);
  note_launch();
}

void plot_hist(const PlotCoord &x, const uint32_t *loss, uint32_t n, uint32_t nb, double mn, double mx,
               uint32_t *hist, cudaStream_t st) {
  cudaMemsetAsync(hist, 0, (size_t)nb * sizeof(uint32_t), st);
  k_plot_hist<<<plot_grid(n), kPlotBlock, (size_t)nb * sizeof(uint32_t), st>>>(x, loss, n, nb, mn, (mx - mn) / nb,
                                                                               hist);
  note_launch();
}

void plot_hist2d(const PlotCoord &x, const PlotCoord &y, const uint32_t *loss, uint32_t n, const double mm[4],
                 uint32_t nx, uint32_t ny, uint32_t *hist, cudaStream_t st) {
  cudaMemsetAsync(hist, 0, (size_t)nx * ny * sizeof(uint32_t), st);
  k_plot_hist2d<<<plot_grid(n), kPlotBlock, 0, st>>>(x, y, loss, n, mm[1], mm[0], mm[3], mm[2], nx, ny, hist);
  note_launch();
}

}  // namespace hps
