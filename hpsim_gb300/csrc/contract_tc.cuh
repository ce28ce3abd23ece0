// contract_tc.cuh -- the SCHEFF ring-to-mesh field sum of FP32 beams on the
// tensor cores (UpdateFldTbl2KernelDouble, src/simulation/inc/
// space_charge_kernel.cu:472-568, launched by UpdateFinalFldTblKernelCall,
// src/simulation/src/space_charge.cu:189-218).
//
// The sum E[zp][rp] = sum over bins (zs, rs) of q(zs, rs) g(rp, rs, zp - zs)
// (g the sign-folded Green's table of contract.cuh) is, for the field rows
// zp < nz, a matrix product
//   D[zp][n] = sum over (rs, k) of A[zp][(rs, k)] B[(rs, k)][n],
//   A[zp][(rs, k)] = q(zp - k, rs)   (zero outside the mesh),
//   B[(rs, k)][n]  = g(rp, rs, k)    (n = 2 rp + component, rp = 0 .. nr),
// with k = zp - zs running over the folded range -(nz - 1) .. nz.  Each CTA
// takes one 128-row tile of zp (the MMA's M) and one source radius rs: K =
// the 127 + nz offsets that tile needs, in chunks of 64, N = 2 (nr + 1)
// rounded up to a multiple of 16 (the padding rows of B are zero).  The
// last field row zp = nz needs offsets k = 1 .. nz only, which are all in
// the last tile's chunks: that tile's producer threads sum it from the B
// tiles while they are staged, one row of B (one (rp, component)) each.
//
// Precision: split BF16.  Both operands are written as hi = bf16(x), lo =
// bf16(x - hi); the three products hi*hi + hi*lo + lo*hi are accumulated in
// FP32 in tensor memory (relative error of a product ~2^-17; measured on the
// test meshes ~4e-6 of the largest field component against FP64).
//
// Data movement: the Green's kernel writes B directly as the MMA's shared-
// memory image (K-major, 128-byte swizzle, tiles of N rows x 64 offsets,
// hi and lo), so a 1D bulk copy (cp.async.bulk, completion on an mbarrier)
// stages each tile.  A is a Toeplitz expansion of one charge column: row zp
// of a chunk is a window of 64 consecutive values of the reversed,
// zero-padded column, which the producer warps copy with 16-byte shared-
// memory loads from 8 shifted copies of it and store swizzled.
//
// Warp roles (160 threads): warps 0-3 build the A tiles and issue the bulk
// copies, then read the accumulator back (warp w owns TMEM lanes 32w..);
// warp 4 allocates the tensor memory and one of its threads issues the MMAs
// and commits them to the stage's "empty" barrier.  Every wait is bounded
// (about a second); a wait that gives up sets the solver's error word, and
// the CTA drains its copies and MMAs before it frees the tensor memory.
//
// The per-radius partial tiles (and last-row partials) are summed in a
// fixed order by k_tc_reduce: results are deterministic.
#pragma once

#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "contract.cuh"
#include "tc_ptx.cuh"

namespace hps {
namespace {

constexpr int kTcM = 128;           // field rows per tile (MMA M)
constexpr int kTcKC = 64;           // offsets per chunk (one 128-byte swizzle row of BF16)
constexpr int kTcThreads = 160;     // 4 producer / epilogue warps + 1 MMA warp
constexpr int kTcProducers = 128;
constexpr size_t kTcSmemMax = 227 * 1024;

// meshes the tensor-core path takes: nz a multiple of the tile height, N
// (below) at most 256 (one MMA), powers of two as every SCHEFF mesh
__host__ __device__ inline bool tc_mesh_ok(uint32_t nr, uint32_t nz) {
  return nz >= 128 && nz <= 512 && (nz & (nz - 1)) == 0 && nr >= 16 && nr <= 64 && (nr & (nr - 1)) == 0;
}
// MMA columns: (E_r, E_z) of the nr + 1 field radii, rounded up to 16
__host__ __device__ inline uint32_t tc_n(uint32_t nr) { return (2 * (nr + 1) + 15) / 16 * 16; }
// tensor-memory columns: the power of two >= N (at least 32)
__host__ __device__ inline uint32_t tc_tmem_cols(uint32_t N) {
  uint32_t c = 32;
  while (c < N) c *= 2;
  return c;
}

// launch shape of one mesh
struct TcDims {
  uint32_t nr, nz;
  uint32_t N;        // MMA columns, tc_n(nr)
  uint32_t cols;     // tensor-memory columns allocated
  uint32_t NC;       // chunks of the folded range (2 nz / 64)
  uint32_t CPT;      // chunks a tile needs (nz / 64 + 2)
  uint32_t BT;       // bytes of one B tile (N rows x 128 B)
  uint32_t S;        // pipeline stages
  uint32_t L;        // elements of one shifted copy of the padded charge column
  uint32_t tiles;    // nz / 128
  size_t smem;       // dynamic shared memory of k_contract_tc
};

__host__ __device__ inline size_t tc_stage_bytes(uint32_t BT) { return 2 * 16384 + 2 * (size_t)BT; }

inline TcDims tc_dims(uint32_t nr, uint32_t nz) {
  TcDims d{};
  d.nr = nr; d.nz = nz; d.N = tc_n(nr); d.cols = tc_tmem_cols(d.N); d.NC = 2 * nz / kTcKC; d.CPT = nz / kTcKC + 2;
  d.BT = d.N * 128; d.L = nz + 264; d.tiles = nz / kTcM;
  // 256 bytes are left for the kernel's static shared memory (barriers)
  const size_t fixed = 1024 + (size_t)16 * d.L * 2 + (size_t)nz * 4 + 256;
  d.S = fixed + 3 * tc_stage_bytes(d.BT) <= kTcSmemMax ? 3 : 2;
  d.smem = fixed + d.S * tc_stage_bytes(d.BT);
  return d;
}

// bytes of the folded split-BF16 table and of the partials (tiles, then the
// last row's per-radius partials)
inline size_t tc_table_bytes(uint32_t nr, uint32_t nz) { return (size_t)nr * (2 * nz / kTcKC) * 2 * tc_n(nr) * 128; }
inline size_t tc_partial_bytes(uint32_t nr, uint32_t nz) {
  return ((size_t)(nz / kTcM) * nr * tc_n(nr) * kTcM + (size_t)nr * tc_n(nr)) * 4;
}

// the tensor-core path runs this kick: FP32 tables sized for this mesh
__device__ inline bool tc_go(const ScState *sc, const ScTables &t) {
  return t.tcg != nullptr && sc->remesh && !sc->sur_accepted && sc->nx == t.tc_nr && sc->nz == t.tc_nz;
}

// the Green's kernel's share: entry (rp <= nr, rs, dz) of component comp
// (value v, E_z already carrying its sign for k >= 1) at both folded
// offsets k = dz + 1 and k = -dz (E_z negated there), hi and lo
__device__ inline void tc_put_green(const ScTables &t, uint32_t nr, uint32_t nz, uint32_t rp, uint32_t rs,
                                    uint32_t dz, float er, float ez) {
  unsigned char *base = (unsigned char *)t.tcg;
  const uint32_t NC = 2 * nz / kTcKC, BT = tc_n(nr) * 128;
  const uint32_t kid[2] = {dz + nz, nz - 1 - dz};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const uint32_t c = kid[side] / kTcKC, j = kid[side] % kTcKC;
    unsigned char *tile = base + ((size_t)(rs * NC + c) * 2) * BT;
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
      const float v = comp == 0 ? er : (side == 0 ? ez : -ez);
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
      const uint32_t off = tc_swz(2 * rp + comp, j);
      *(__nv_bfloat16 *)(tile + off) = hi;
      *(__nv_bfloat16 *)(tile + BT + off) = lo;
    }
  }
}

// 2^-36 fixed-point charge as FP32 (two 32-bit conversions)
__device__ __forceinline__ float tc_charge(unsigned long long v) {
  const long long s = (long long)v;
  return fmaf((float)(int)(s >> 32), 4294967296.0f, (float)(unsigned)(v & 0xffffffffull)) *
         1.4551915228366852e-11f;
}

// ---- the product ------------------------------------------------------------
// the CTA of field-row tile `tile` and source radius `rs`
__device__ __forceinline__ void contract_tc_body(const ScState *sc, const ScTables &t, const TcDims &d,
                                                 uint32_t tile, uint32_t rs) {
  if (!tc_go(sc, t)) return;
  extern __shared__ unsigned char tc_raw[];
  __shared__ uint64_t full[3], empty[3], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t N = d.N, nz = d.nz, nr = d.nr, S = d.S, BT = d.BT, L = d.L;
  // 1024-byte aligned stage buffers, then the shifted charge copies and the column
  unsigned char *sm = (unsigned char *)(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
  const size_t stage = tc_stage_bytes(BT);
  __nv_bfloat16 *cp = (__nv_bfloat16 *)(sm + S * stage);  // [h][s][L]
  float *qc = (float *)(sm + S * stage + (size_t)16 * L * 2);
  volatile int *abort = &abort_flag;

  // the charge column first: its loads overlap the set-up below
  if (warp < 4)
    for (uint32_t zs = tid; zs < nz; zs += kTcProducers) qc[zs] = tc_charge(__ldg(t.bin_fx + zs * nr + rs));
  if (tid == 0) {
    for (uint32_t s = 0; s < S; ++s) {
      mbar_init(&full[s], kTcProducers + 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_slot)),
                 "r"(d.cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t c0 = 2 * tile, nch = d.CPT;  // this tile's chunks of the folded range
  bool issued_mma = false;

  if (warp < 4) {
    // ---- producers: the B tiles of the first stages in flight, the charge
    // column's shifted copies, then per chunk the A tile (and the B tile of
    // the chunks after the first S) ----
    const unsigned char *gsrc = (const unsigned char *)t.tcg + (size_t)rs * d.NC * 2 * BT;
    if (tid == 0) {
      for (uint32_t i = 0; i < S && i < nch; ++i) {
        unsigned char *st = sm + i * stage;
        mbar_arrive_tx(&full[i], 2 * BT);
        const unsigned char *src = gsrc + (size_t)(c0 + i) * 2 * BT;
        bulk_g2s(st + 2 * 16384, src, BT, &full[i]);
        bulk_g2s(st + 2 * 16384 + BT, src + BT, BT, &full[i]);
      }
    }
    // copy s, element x holds R(x + s - 128), R(v) = q(nz - 1 - v) inside the
    // mesh; eight elements per 16-byte store (L is a multiple of 8)
    const uint32_t groups = L / 8;
    for (uint32_t e = tid; e < 8 * groups; e += kTcProducers) {
      const uint32_t s = e / groups, x0 = (e % groups) * 8;
      __align__(16) __nv_bfloat16 hv[8], lv[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int v = (int)(x0 + j) + (int)s - 128;
        const float q = (v >= 0 && v < (int)nz) ? qc[nz - 1 - v] : 0.0f;
        hv[j] = __float2bfloat16_rn(q);
        lv[j] = __float2bfloat16_rn(q - __bfloat162float(hv[j]));
      }
      *(uint4 *)(cp + s * L + x0) = *(const uint4 *)hv;
      *(uint4 *)(cp + (8 + s) * L + x0) = *(const uint4 *)lv;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const uint32_t m = tid;  // the A row this thread writes
    // the last tile's threads also sum the last field row from B rows tid
    // and tid + 128 (n < N) of the chunks of offsets 1 .. nz
    const bool last_row = tile + 1 == d.tiles;
    float lr0 = 0.0f, lr1 = 0.0f;
    for (uint32_t i = 0; i < nch && !*abort; ++i) {
      const uint32_t s = i % S, use = i / S;
      if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1, abort)) break;
      unsigned char *st = sm + s * stage;
      if (tid == 0 && use > 0) {
        mbar_arrive_tx(&full[s], 2 * BT);
        const unsigned char *src = gsrc + (size_t)(c0 + i) * 2 * BT;
        bulk_g2s(st + 2 * 16384, src, BT, &full[s]);
        bulk_g2s(st + 2 * 16384 + BT, src + BT, BT, &full[s]);
      }
      // row m of the chunk: R(W .. W + 63), W = 64 i - m (+128 into the copies)
      const int wp = 64 * (int)i - (int)m + 128;
      const int sh = wp & 7, base = wp - sh;
      const uint4 *hi = (const uint4 *)(cp + sh * L + base);
      const uint4 *lo = (const uint4 *)(cp + (8 + sh) * L + base);
      unsigned char *ah = st + (m >> 3) * 1024 + (m & 7) * 128;
      unsigned char *al = ah + 16384;
#pragma unroll
      for (uint32_t jj = 0; jj < 8; ++jj) {
        const uint32_t off = ((jj ^ (m & 7)) & 7) << 4;
        *(uint4 *)(ah + off) = hi[jj];
        *(uint4 *)(al + off) = lo[jj];
      }
      fence_async_smem();
      mbar_arrive(&full[s]);
      const uint32_t c = c0 + i;  // this chunk's offsets: kidx = 64 c + j
      if (last_row && c * kTcKC >= nz) {
        // B landed (the phase also needs the tile's bytes); offset kidx
        // k = kidx - (nz - 1) takes the charge of row zs = 2 nz - 1 - kidx
        if (!mbar_wait(&full[s], use & 1, abort)) break;
        const unsigned char *bh = st + 2 * 16384, *bl = bh + BT;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const uint32_t n = tid + 128 * half;
          if (n >= N) continue;
          const uint32_t row = (n >> 3) * 1024 + (n & 7) * 128;
          float acc = 0.0f;
#pragma unroll
          for (uint32_t jj = 0; jj < 8; ++jj) {
            const uint32_t off = row + (((jj ^ (n & 7)) & 7) << 4);
            const uint4 vh = *(const uint4 *)(bh + off), vl = *(const uint4 *)(bl + off);
            const __nv_bfloat16 *h8 = (const __nv_bfloat16 *)&vh, *l8 = (const __nv_bfloat16 *)&vl;
#pragma unroll
            for (uint32_t u = 0; u < 8; ++u) {
              const uint32_t zs = 2 * nz - 1 - (c * kTcKC + 8 * jj + u);
              acc = fmaf(qc[zs], __bfloat162float(h8[u]) + __bfloat162float(l8[u]), acc);
            }
          }
          if (half == 0) lr0 += acc;
          else lr1 += acc;
        }
      }
    }
    if (last_row && !*abort) {
      // rows n < N only: a thread beyond them would write into the next
      // radius's partials
      float *pl = t.tcp + (size_t)d.tiles * nr * N * kTcM + (size_t)rs * N;
      if (tid < N) pl[tid] = lr0;
      if (tid + 128 < N) pl[tid + 128] = lr1;
    }
  } else if (lane == 0) {
    // ---- the MMA thread ----
    const uint32_t idesc = tc_idesc(N);
    for (uint32_t i = 0; i < nch; ++i) {
      const uint32_t s = i % S, use = i / S;
      if (!mbar_wait(&full[s], use & 1, abort)) break;
      tc_fence_after();
      const uint32_t a0 = tc_smem(sm + s * stage), b0 = a0 + 2 * 16384;
      const uint64_t ah = tc_desc(a0), al = tc_desc(a0 + 16384), bh = tc_desc(b0), bl = tc_desc(b0 + BT);
#pragma unroll
      for (uint32_t ks = 0; ks < kTcKC / 16; ++ks) {
        const uint64_t adv = 2 * ks;  // 32 bytes along K, in 16-byte units
        tc_mma(tmem, ah + adv, bh + adv, idesc, (i | ks) != 0);
        tc_mma(tmem, ah + adv, bl + adv, idesc, 1);
        tc_mma(tmem, al + adv, bh + adv, idesc, 1);
      }
      issued_mma = true;
      tc_commit(&empty[s]);
    }
    if (issued_mma) tc_commit(&done);
  }

  // ---- epilogue: the accumulator to this (tile, radius) partial ----
  if (warp < 4) {
    const bool ok = !*abort && mbar_wait(&done, 0, abort);
    if (ok) {
      tc_fence_after();
      float *out = t.tcp + ((size_t)(tile * nr + rs) * N) * kTcM + 32 * warp + lane;
      const uint32_t tl = tmem + ((32 * warp) << 16);
      for (uint32_t c = 0; c < N; c += 16) {
        float v[16];
        tc_ld16(tl + c, v);
#pragma unroll
        for (int k = 0; k < 16; ++k) out[(size_t)(c + k) * kTcM] = v[k];
      }
    }
    tc_fence_before();
  }
  __syncthreads();
  if (*abort) {
    // a wait gave up: record it, let the bulk copies and MMAs already issued
    // land (both finish on their own within microseconds), then free the
    // tensor memory
    if (tid == 0) atomicOr((unsigned int *)&((ScState *)sc)->tc_error, 1u);
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(d.cols) : "memory");
  }
}

// grid (tiles, nr): tile blockIdx.x of field rows, source radius blockIdx.y
__global__ void __launch_bounds__(kTcThreads, 1) k_contract_tc(const ScState *sc, ScTables t, TcDims d) {
  contract_tc_body(sc, t, d, blockIdx.x, blockIdx.y);
}
// the lockstep form: grid z over the beams, one solver's tables each
template <int B>
__global__ void __launch_bounds__(kTcThreads, 1) k_contract_tc_seg(const __grid_constant__ SegArgs<MeshSeg, B> a,
                                                                 TcDims d) {
  const MeshSeg &p = a.p[blockIdx.z];
  contract_tc_body(p.sc, p.t, d, blockIdx.x, blockIdx.y);
}

// The partials summed over the source radii: a block takes 64 consecutive
// field rows of one field radius (blockIdx.y), its four thread quarters a
// quarter of the source radii each (rows adjacent in memory, so every load
// of a warp is coalesced), summed in radius order within a quarter and the
// quarters in order: deterministic.  Tile partials for the rows zp < nz, the
// last tile's last-row partials for zp = nz.
__device__ __forceinline__ void tc_reduce_body(const ScState *sc, const ScTables &t, const TcDims &d, uint32_t bx,
                                               uint32_t by) {
  if (!tc_go(sc, t)) return;
  __shared__ float red[2][4][64];
  const uint32_t nr = d.nr, nz = d.nz, N = d.N, nrow = nr + 1;
  const uint32_t q = threadIdx.x / 64, ml = threadIdx.x % 64;
  const uint32_t zp = bx * 64 + ml, rp = by;
  float ex = 0.0f, ez = 0.0f;
  if (zp <= nz) {
    const float *p;
    size_t stride, comp;
    if (zp < nz) {
      p = t.tcp + ((size_t)(zp / kTcM) * nr * N + 2 * rp) * kTcM + zp % kTcM;
      stride = (size_t)N * kTcM;
      comp = kTcM;
    } else {
      p = t.tcp + (size_t)d.tiles * nr * N * kTcM + 2 * rp;
      stride = N;
      comp = 1;
    }
    const uint32_t per = nr / 4, g0 = q * per;  // nr >= 16: a multiple of 4 radii per quarter
    for (uint32_t g = g0; g < g0 + per; g += 4) {
      float vx[4], vz[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        vx[u] = __ldcg(p + (g + u) * stride);
        vz[u] = __ldcg(p + (g + u) * stride + comp);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        ex += vx[u];
        ez += vz[u];
      }
    }
  }
  red[0][q][ml] = ex;
  red[1][q][ml] = ez;
  __syncthreads();
  if (q != 0 || zp > nz) return;
  const size_t pt = (size_t)zp * nrow + rp;
  t.ffld2[2 * pt] = ((red[0][0][ml] + red[0][1][ml]) + red[0][2][ml]) + red[0][3][ml];
  t.ffld2[2 * pt + 1] = ((red[1][0][ml] + red[1][1][ml]) + red[1][2][ml]) + red[1][3][ml];
}

__global__ void __launch_bounds__(256) k_tc_reduce(const ScState *sc, ScTables t, TcDims d) {
  tc_reduce_body(sc, t, d, blockIdx.x, blockIdx.y);
}
template <int B>
__global__ void __launch_bounds__(256) k_tc_reduce_seg(const __grid_constant__ SegArgs<MeshSeg, B> a, TcDims d) {
  const MeshSeg &p = a.p[blockIdx.z];
  tc_reduce_body(p.sc, p.t, d, blockIdx.x, blockIdx.y);
}

// the dynamic shared-memory limit of the largest mesh the path takes (static
// and dynamic shared memory together stay within the 227 KB a CTA may have)
inline cudaError_t contract_tc_configure() {
  size_t most = 0;
  for (uint32_t nr = 16; nr <= 64; nr *= 2)
    for (uint32_t nz = 128; nz <= 512; nz *= 2) most = std::max(most, tc_dims(nr, nz).smem);
  cudaError_t e = cudaFuncSetAttribute(k_contract_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_contract_tc_seg<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_contract_tc_seg<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_contract_tc_seg<SegCap<MeshSeg>::value>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)most);
  return e;
}

inline void contract_tc_merge(const std::vector<const Rec *> &recs, SegFork &, cudaStream_t st, cudaStream_t) {
  uint32_t dims[2];
  std::memcpy(dims, recs[0]->p.data() + sizeof(MeshSeg), sizeof(dims));
  const uint32_t nr = dims[0], nz = dims[1];
  const TcDims d = tc_dims(nr, nz);
  std::vector<Rec> heads(recs.size());  // the MeshSeg heads of the records
  std::vector<const Rec *> hp(recs.size());
  for (size_t k = 0; k < recs.size(); ++k) {
    heads[k].p.assign(recs[k]->p.begin(), recs[k]->p.begin() + sizeof(MeshSeg));
    hp[k] = &heads[k];
  }
  seg_chunks<MeshSeg>(hp, [&](const auto &a, uint32_t) {
    constexpr int B = std::decay_t<decltype(a)>::kB;
    k_contract_tc_seg<B><<<dim3(d.tiles, nr, a.nb), kTcThreads, d.smem, st>>>(a, d);
    k_tc_reduce_seg<B><<<dim3((nz + 1 + 63) / 64, nr + 1, a.nb), 256, 0, st>>>(a, d);
  });
}

// both launches of a tensor-core solve on a mesh of nr x nz
inline void contract_tc_launch(const ScState *sc, const ScTables &t, uint32_t nr, uint32_t nz, cudaStream_t st) {
  if (recorder()) {
    struct { MeshSeg m; uint32_t dims[2]; } p{{sc, t}, {nr, nz}};
    record("contract_tc", &contract_tc_merge, 0, p, (uint64_t)p.dims[0] << 32 | p.dims[1]);
    return;
  }
  const TcDims d = tc_dims(nr, nz);
  k_contract_tc<<<dim3(d.tiles, nr), kTcThreads, d.smem, st>>>(sc, t, d);
  k_tc_reduce<<<dim3((nz + 1 + 63) / 64, nr + 1), 256, 0, st>>>(sc, t, d);
}

}  // namespace
}  // namespace hps
