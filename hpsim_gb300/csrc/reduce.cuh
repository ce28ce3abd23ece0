// reduce.cuh -- one-launch deterministic reductions over the particles.
//
// The reference reduces every moment with a Harris two-level tree: a first
// pass capped at 64 blocks, a second pass, then a <<<1,1>>> finaliser kernel
// (src/beam/src/beam.cu:411-436, 651-678); about 30 launches and 5 blocking
// scalar reads per space-charge kick.  Here one launch does all of it: every
// block reduces its grid-stride share of the particles (each thread in index
// order, warps by a fixed shuffle tree, warps in index order), writes one
// partial per block, and the last block to finish (threadfence + counter)
// sums the partials in block order and runs the finaliser.  The result is
// bitwise reproducible for a given particle count, and the per-particle
// callback may also write per-particle outputs (relative phase, loss flags)
// in the same sweep.
#pragma once

#include <algorithm>

#include <type_traits>

#include "common.cuh"
#include "lockstep.cuh"

namespace hps {

// comb() is overloaded for float so that FP32 warp trees stay on the FP32
// pipes (a float argument promoted to the double overload would run every
// shuffle step through FP64 arithmetic).
struct SumComb {
  __device__ static double ident() { return 0.0; }
  __device__ static double comb(double a, double b) { return a + b; }
  __device__ static float comb(float a, float b) { return a + b; }
};
struct MaxComb {  // MaxR2PhiReduceKernel starts from 0 (beam_kernel.cu:809-810)
  __device__ static double ident() { return 0.0; }
  __device__ static double comb(double a, double b) { return a < b ? b : a; }
  __device__ static float comb(float a, float b) { return a < b ? b : a; }
};

// Total of the per-block partials, taken by the last block: thread t combines
// blocks t, t + blockDim, ... in order (independent loads, so the sweep runs
// at memory parallelism rather than one L2 round trip per block), then the
// lanes by a fixed shuffle tree and the warps in order.
template <class C, int K>
__device__ inline void combine_partials(const double *part, uint32_t nb, double (*sm)[K], double *tot) {
  double v[K];
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = C::ident();
  for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = C::comb(v[k], __ldcg(part + (size_t)b * K + k));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = v[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x = C::comb(x, __shfl_down_sync(0xffffffffu, x, off));
    if (lane == 0) sm[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double x = C::ident();
    for (int w = 0; w < kBlock / 32; ++w) x = C::comb(x, sm[w][threadIdx.x]);
    tot[threadIdx.x] = x;
  }
  __syncthreads();
}

// Op must provide:
//   static constexpr int K;            number of accumulators (<= 32)
//   using Comb = SumComb | MaxComb;
//   __device__ bool enabled() const;   device-side predicate (false: no work)
//   __device__ void particle(uint32_t i, double (&acc)[K]) const;
//   __device__ void finalize(const double* tot, int tid, int nthreads) const;
template <class Op>
__global__ void __launch_bounds__(kBlock) pass_kernel(Op op, uint32_t n, PassScratch scr) {
  constexpr int K = Op::K;
  using C = typename Op::Comb;
  if (!op.enabled()) return;
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = C::ident();
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) op.particle(i, acc);

  __shared__ double sm[kBlock / 32][K];
  __shared__ double tot[K];
  __shared__ int is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double v = acc[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = C::comb(v, __shfl_down_sync(0xffffffffu, v, off));
    if (lane == 0) sm[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double v = C::ident();
    for (int w = 0; w < kBlock / 32; ++w) v = C::comb(v, sm[w][threadIdx.x]);
    scr.part[blockIdx.x * K + threadIdx.x] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = (atomicAdd(scr.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  combine_partials<C, K>(scr.part, gridDim.x, sm, tot);
  op.finalize(tot, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) *scr.counter = 0u;
}

template <class Op>
inline void launch_pass(const Op &op, uint32_t n, PassScratch scr, cudaStream_t s) {
  pass_kernel<Op><<<pass_blocks(n), kBlock, 0, s>>>(op, n, scr);
}

// Same scheme for FP32 particle state: each thread accumulates its particles
// in FP32 and the warp tree runs in FP32 (FP64 arithmetic on GB300 runs at
// 1/64 of the FP32 rate, so per-particle FP64 sums would dominate); warps,
// blocks and the finaliser combine in FP64.  Op::setup() returns constants
// (offsets of device-side averages from the synchronous particle), computed
// once per block.  A thread takes its particles kPassBatch at a time (2 for
// ops with many accumulators, to stay within registers): Op::load(i) reads
// particle i into an Op::P, and Op::use(i, p, acc, ctx)
// accumulates it (and may write per-particle outputs), so every load of a
// batch is in flight before the first store.
constexpr int kPassBatch = 4;
template <int K> constexpr int pass_batch() { return K > 10 ? 2 : kPassBatch; }
// an Op may set its own batch (`static constexpr int kBatch`)
template <class Op, class = void>
struct op_batch : std::integral_constant<int, pass_batch<Op::K>()> {};
template <class Op>
struct op_batch<Op, std::void_t<decltype(Op::kBatch)>> : std::integral_constant<int, Op::kBatch> {};

// An Op with `static constexpr bool kFast = true` has its block and grid
// partials combined in FP32 (counts stay exact below 2^24 particles); the
// space-charge statistics that only size the mesh and scale the kick use
// it, reported beam statistics do not.
template <class Op, class = void>
struct op_fast : std::false_type {};
template <class Op>
struct op_fast<Op, std::void_t<decltype(Op::kFast)>> : std::integral_constant<bool, Op::kFast> {};

// An Op with `static constexpr int kMaxFrom = m` (fast combine only) takes
// the maximum, not the sum, of accumulators m .. K-1; they start at -inf.
template <class Op, class = void>
struct op_max_from : std::integral_constant<int, Op::K> {};
template <class Op>
struct op_max_from<Op, std::void_t<decltype(Op::kMaxFrom)>> : std::integral_constant<int, Op::kMaxFrom> {};

template <class C, int MF>
__device__ inline float comb_k(int k, float a, float b) {
  return k >= MF ? fmaxf(a, b) : C::comb(a, b);
}

// block bid of nblk blocks of the pass over particles 0..n-1
template <class Op>
__device__ __forceinline__ void pass_body_f(const Op &op, uint32_t n, PassScratch scr, uint32_t bid, uint32_t nblk) {
  constexpr int K = Op::K;
  constexpr int B = op_batch<Op>::value;
  using C = typename Op::Comb;
  if (!op.enabled()) return;
  __shared__ double sm[kBlock / 32][K];
  __shared__ double tot[K];
  __shared__ int is_last;
  __shared__ typename Op::Ctx sctx;
  if (threadIdx.x == 0) sctx = op.setup();
  __syncthreads();
  const typename Op::Ctx ctx = sctx;
  constexpr int MF = op_max_from<Op>::value;
  static_assert(MF == K || op_fast<Op>::value, "max slots need the FP32 combine");
  float acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = k >= MF ? -INFINITY : 0.0f;
  const uint32_t stride = nblk * blockDim.x;
  for (uint32_t base = bid * blockDim.x + threadIdx.x; base < n; base += B * stride) {
    typename Op::P p[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const uint32_t i = base + u * stride;
      if (i < n) p[u] = op.load(i);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const uint32_t i = base + u * stride;
      if (i < n) op.use(i, p[u], acc, ctx);
    }
  }

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (op_fast<Op>::value) {
    // FP32 partials: warps summed in order per block, blocks by the warps of
    // the last block (slot k by warp k mod 8; lane l takes blocks l, l + 32,
    // ...; then a fixed shuffle tree).  No FP64 arithmetic on the
    // reduction's critical path.
    __shared__ float smf[kBlock / 32][K];
    float *partf = (float *)scr.part;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float v = acc[k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v = comb_k<C, MF>(k, v, __shfl_down_sync(0xffffffffu, v, off));
      if (lane == 0) smf[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
      const int k = threadIdx.x;
      float v = k >= MF ? -INFINITY : 0.0f;
      for (int w = 0; w < kBlock / 32; ++w) v = comb_k<C, MF>(k, v, smf[w][k]);
      partf[bid * K + k] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(scr.counter, 1u) == nblk - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // warp w combines slots w, w + 8, ...: the slots' chains run side by side
    for (int k = warp; k < K; k += kBlock / 32) {
      float v = k >= MF ? -INFINITY : 0.0f;
      for (uint32_t b = lane; b < nblk; b += 32) v = comb_k<C, MF>(k, v, __ldcg(partf + (size_t)b * K + k));
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v = comb_k<C, MF>(k, v, __shfl_down_sync(0xffffffffu, v, off));
      if (lane == 0) tot[k] = (double)v;
    }
    __syncthreads();
  } else {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float v = acc[k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v = C::comb(v, __shfl_down_sync(0xffffffffu, v, off));
      if (lane == 0) sm[warp][k] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
      double v = C::ident();
      for (int w = 0; w < kBlock / 32; ++w) v = C::comb(v, sm[w][threadIdx.x]);
      scr.part[bid * K + threadIdx.x] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(scr.counter, 1u) == nblk - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    combine_partials<C, K>(scr.part, nblk, sm, tot);
  }
  op.finalize(tot, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) *scr.counter = 0u;
}

template <class Op>
__global__ void __launch_bounds__(kBlock) pass_kernel_f(Op op, uint32_t n, PassScratch scr) {
  pass_body_f(op, n, scr, blockIdx.x, gridDim.x);
}

// one beam's share of a lockstep launch of pass_kernel_f
template <class Op>
struct PassSeg {
  Op op;
  uint32_t n;
  PassScratch scr;
};
template <class Op, int B>
__global__ void __launch_bounds__(kBlock) pass_kernel_f_seg(const __grid_constant__ SegArgs<PassSeg<Op>, B> a) {
  uint32_t bid, nblk;
  const PassSeg<Op> &p = a.p[seg_find(a, blockIdx.x, bid, nblk)];
  pass_body_f(p.op, p.n, p.scr, bid, nblk);
}
template <class Op>
inline void pass_merge(const std::vector<const Rec *> &recs, SegFork &, cudaStream_t st, cudaStream_t) {
  seg_chunks<PassSeg<Op>>(recs, [&](const auto &a, uint32_t blocks) {
    pass_kernel_f_seg<Op, std::decay_t<decltype(a)>::kB><<<blocks, kBlock, 0, st>>>(a);
  });
}
// a pass_kernel_f launch of `blocks` blocks, or its record under a lockstep recorder
template <class Op>
inline void launch_pass_f_grid(const Op &op, uint32_t n, PassScratch scr, cudaStream_t s, uint32_t blocks,
                               const char *site) {
  if (recorder()) {
    record(site, &pass_merge<Op>, blocks, PassSeg<Op>{op, n, scr});
    return;
  }
  launch_k(pass_kernel_f<Op>, dim3(blocks), dim3(kBlock), 0, s, op, n, scr);
}

// With the FP64 combine, at most two blocks per SM: the last block sums
// every block's partials in FP64 on one SM (1/64-rate FP64 on GB300), so
// fewer, fuller blocks keep that tail short; each thread walks more
// particles in batches instead.  With the FP32 combine, every block the SMs
// hold at once (up to the scratch's kMaxPassBlocks).
inline int pass_blocks_f(uint32_t n, int per_sm = 2) {
  uint32_t b = (n + kPassBatch * kBlock - 1) / (kPassBatch * kBlock);
  if (b < 1) b = 1;
  const uint32_t cap = std::min<uint32_t>((uint32_t)per_sm * 152u, (uint32_t)kMaxPassBlocks);
  if (b > cap) b = cap;
  return (int)b;
}

template <class Op>
inline int pass_resident() {
  static int r = 0;  // blocks of this kernel an SM holds at once
  if (!r && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, pass_kernel_f<Op>, kBlock, 0) != cudaSuccess || r < 1))
    r = 1;
  return r;
}

// cap: at most this many blocks per SM (0: no cap)
template <class Op>
inline void launch_pass_f(const Op &op, uint32_t n, PassScratch scr, cudaStream_t s, uint32_t cap = 0,
                          const char *site = "pass") {
  int per_sm = op_fast<Op>::value ? pass_resident<Op>() : 2;
  if (cap && (uint32_t)per_sm > cap) per_sm = (int)cap;
  launch_pass_f_grid(op, n, scr, s, (uint32_t)pass_blocks_f(n, per_sm), site);
}

// FP32 version of rel_phase for offsets that are already small
__device__ inline float rel_phase_f(float d) {
  const float pi = 3.14159265358979323846f, twopi = 6.28318530717958647692f;
  float tmp = d + pi;
  float sign = 1.0f;
  if (tmp < 0.0f) { sign = -1.0f; tmp = -tmp; }
  if (tmp < twopi) return sign * (tmp - pi);
  return sign * (fmodf(tmp, twopi) - pi);
}

// wrap(phi - ref) as UpdateRelativePhiKernel, beam_kernel.cu:1507-1525
__device__ inline double rel_phase(double phi, double ref) {
  double tmp = phi - ref + PI;
  double sign = 1.0;
  if (tmp < 0) { sign = -1.0; tmp = -tmp; }
  return sign * (fmod(tmp, TWOPI) - PI);
}

}  // namespace hps
