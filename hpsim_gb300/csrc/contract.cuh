// contract.cuh -- the SCHEFF ring-to-mesh field sum (UpdateFldTbl2KernelDouble,
// src/simulation/inc/space_charge_kernel.cu:472-568) for FP32 tables (FP32
// beams) and FP64 tables (FP64 beams), one kernel template:
//   E[zp][rp] = sum over bins (zs, rs) of q(zs, rs) g(zp - zs),
// g(k) = G[rp][k - 1][rs] for sources below the point (k >= 1) and
// G[rp][-k][rs] with E_z negated for sources at or above it (k <= 0).
// For each source radius this is a convolution along z.  A block stages its
// rp's g(k) (mirrored with the sign included, or the table rows alone with
// the E_z sign flipped on reading when the mirror does not fit) and the
// charges (2^-36 fixed point converted to T) in shared memory, a tile of
// source radii at a time.  A warp computes kCP consecutive field points over half the source
// rows (two warps per point group, summed in a fixed order): the lanes run
// over source radii, and as the warp walks the rows the kCP values of g it
// needs slide by one, kept in a ring of kCP + 1 registers that takes one new
// shared-memory load per row (one charge and one table load per 2 kCP FMAs).
// Each point's sum ends with a fixed shuffle tree.  The set of bins each
// point sums is the reference's (its integer partition of the table): bins
// zs * nr + rs at or above a limit are left out, which only happens when the
// mesh has fewer than 1024 bins or a row count that does not divide them.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "lockstep.cuh"

namespace hps {
namespace {

constexpr int kCP = 4;                     // field points per warp
constexpr int kCH = 2;                     // warps sharing the source rows of a point group
constexpr int kCG = 4;                     // point groups per block
constexpr int kCZ = kCP * kCG;             // field points per block
constexpr int kContractThreads = kCG * kCH * 32;
// largest table + charge tile: 32 source radii of an FP32 256-row mesh or of
// an FP64 128-row mesh (two CTAs per SM; lanes run over source radii)
constexpr int kContractSmem = 96 * 1024;

// the FP32 and FP64 tables: pair type, table layout, charge conversion
template <class T> struct CTab;
template <> struct CTab<float> {
  using V = float2;
  // FP32 Green's table [rp][dz][rs] (ScTables::ffld1)
  static __device__ const V *slice(const ScTables &t, uint32_t rp, uint32_t fld) {
    return (const V *)t.ffld1 + (size_t)rp * fld;
  }
  static __device__ size_t at(uint32_t z, uint32_t rs, uint32_t nx, uint32_t) { return (size_t)z * nx + rs; }
  static constexpr bool kZFast = false;  // consecutive table entries run over rs
  // 2^-36 fixed-point charge through two 32-bit conversions (a 64-bit
  // integer conversion runs on the FP64 pipe)
  static __device__ float charge(unsigned long long v) {
    const long long s = (long long)v;
    const int hi = (int)(s >> 32);
    const unsigned lo = (unsigned)(v & 0xffffffffull);
    return fmaf((float)hi, 4294967296.0f, (float)lo) * 1.4551915228366852e-11f;  // 2^-36
  }
  static __device__ float *out(const ScTables &t) { return t.ffld2; }
};
template <> struct CTab<double> {
  using V = double2;
  // FP64 Green's table [rp][rs][dz] (ScTables::fld1)
  static __device__ const V *slice(const ScTables &t, uint32_t rp, uint32_t fld) {
    return (const V *)t.fld1 + (size_t)rp * fld;
  }
  static __device__ size_t at(uint32_t z, uint32_t rs, uint32_t, uint32_t nz) { return (size_t)rs * nz + z; }
  static constexpr bool kZFast = true;   // consecutive table entries run over dz
  static __device__ double charge(unsigned long long v) { return (double)(long long)v * kBinInvScale; }
  static __device__ double *out(const ScTables &t) { return t.fld2; }
};

// Two layouts of the staged table.  Mirrored (M): g(k) for k = -(nz - 1)
// .. nz stored with its sign, 2 nz pairs per radius, read with no select;
// single: the nz table rows, g(k) formed on reading (E_z negated for k <=
// 0).  With the charges, 5 or 3 values of T per row and radius.  The
// mirrored layout is used when a 32-radius tile of it fits.
template <class T, bool M>
__host__ __device__ inline uint32_t contract_tile(uint32_t nx, uint32_t nz) {
  const uint32_t t = (uint32_t)(kContractSmem / ((M ? 5 : 3) * sizeof(T) * nz));
  return t < nx ? t : nx;
}
template <class T>
inline bool contract_mirrored(uint32_t nx_max, uint32_t nz_max) {
  return (size_t)5 * sizeof(T) * nz_max * std::min<uint32_t>(32u, nx_max) <= (size_t)kContractSmem;
}
// (bounds the tile of every mesh up to nx_max x nz_max)
template <class T>
inline size_t contract_smem(uint32_t nx_max, uint32_t nz_max) {
  const size_t per = contract_mirrored<T>(nx_max, nz_max) ? 5 : 3;
  return std::min<size_t>(kContractSmem, per * sizeof(T) * nx_max * nz_max);
}

// g(k) of the staged tile (h: the tile's column of this lane's radius)
template <bool M, class V>
__device__ __forceinline__ V gk(const V *h, int k, int tr, int nz) {
  if (M) return h[(nz - 1 + k) * tr];
  const bool below = k >= 1;
  const V v = h[(below ? k - 1 : -k) * tr];
  return below ? v : V{v.x, -v.y};
}

// the bin limit of field row zp (the reference's partition of the table)
__device__ inline uint32_t contract_lim(uint32_t zp, uint32_t rp, uint32_t nx, uint32_t nz) {
  const uint32_t fld_sz = nx * nz;
  if (zp < nz) {
    const uint32_t gnum = 1024 / nz;
    return gnum ? gnum * (fld_sz / gnum) : 0;
  }
  if (rp < nx) {
    const uint32_t gnum = 1024 / nx;
    return gnum ? gnum * (fld_sz / gnum) : 0;
  }
  return (fld_sz / 1024) * 1024;
}

template <class T, class V>
__device__ inline V cpair(T x, T y) { return V{x, y}; }

// One block's work: S slabs of kCZ field rows of one field radius from
// each staged tile (S > 1 stages the table once for more rows); TR > 0 is
// the tile width known at compile time (nr == TR, one tile: every
// shared-memory offset of the row walk is an immediate), TR == 0 the general
// tiled form.
template <class T, int TR, bool M, int S>
__device__ __forceinline__ void contract_block(const ScState *sc, const ScTables &t, T *sm,
                                               typename CTab<T>::V (*upper)[kCG][kCP], uint32_t bx, uint32_t by) {
  using V = typename CTab<T>::V;
  const uint32_t nx = sc->nx, nz = sc->nz, fld_sz = nx * nz, nrow = nx + 1;
  const uint32_t rp = bx, zb0 = by * kCZ * S;
  const uint32_t tr = TR > 0 ? (uint32_t)TR : contract_tile<T, M>(nx, nz);
  V *gz = (V *)sm;                     // M: [k + nz - 1][tr]; else [dz][tr] holding g(dz + 1)
  T *qs = sm + (M ? 4 : 2) * nz * tr;  // [zs][tr]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp / kCH, half = warp % kCH;
  const uint32_t za = half * nz / kCH, zb = (half + 1) * nz / kCH;  // this warp's source rows
  const V *G = CTab<T>::slice(t, rp, fld_sz);
  T axs[S][kCP], azs[S][kCP];
#pragma unroll
  for (int sl = 0; sl < S; ++sl)
#pragma unroll
    for (int j = 0; j < kCP; ++j) axs[sl][j] = azs[sl][j] = T(0);
  for (uint32_t rs0 = 0; rs0 < nx; rs0 += tr) {
    const uint32_t ntr = TR > 0 ? (uint32_t)TR : min(tr, nx - rs0), ntile = nz * ntr;
    __syncthreads();
    // every load of a thread's share is issued before its first store: one
    // memory round trip per kStage elements, not per element; thread order
    // follows the table's fast index
    constexpr int kStage = 8;
    for (uint32_t e0 = threadIdx.x; e0 < ntile; e0 += kStage * blockDim.x) {
      V gv[kStage];
      unsigned long long bv[kStage];
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const uint32_t e = e0 + u * blockDim.x;
        if (e < ntile) {
          const uint32_t z = CTab<T>::kZFast ? e % nz : e / ntr, r = CTab<T>::kZFast ? e / nz : e % ntr;
          gv[u] = __ldg(G + CTab<T>::at(z, rs0 + r, nx, nz));
          bv[u] = __ldg(t.bin_fx + z * nx + rs0 + r);
        }
      }
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const uint32_t e = e0 + u * blockDim.x;
        if (e < ntile) {
          const uint32_t z = CTab<T>::kZFast ? e % nz : e / ntr, r = CTab<T>::kZFast ? e / nz : e % ntr;
          if (M) {
            gz[(nz + z) * tr + r] = gv[u];                               // k = z + 1
            gz[(nz - 1 - z) * tr + r] = cpair<T, V>(gv[u].x, -gv[u].y);  // k = -z
          } else {
            gz[z * tr + r] = gv[u];  // g(z + 1), and g(-z) with E_z negated
          }
          qs[z * tr + r] = CTab<T>::charge(bv[u]);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int sl = 0; sl < S; ++sl) {
    const uint32_t zp0 = zb0 + sl * kCZ + grp * kCP;  // points zp0 .. zp0 + kCP - 1
    if (zp0 > nz) continue;
    uint32_t lim[kCP];
    bool cut = false;
#pragma unroll
    for (int j = 0; j < kCP; ++j) {
      lim[j] = contract_lim(zp0 + j, rp, nx, nz);
      cut |= zp0 + j <= nz && lim[j] < fld_sz;
    }
    T (&ax)[kCP] = axs[sl];
    T (&az)[kCP] = azs[sl];
    for (uint32_t r = lane; r < ntr; r += 32) {
      if (!cut) {
        // ring slot (j - u) mod R holds g(zp0 + j - zs), u = zs - zs0; the
        // slot (-u - 1) mod R is free at row zs and takes g(zp0 - zs - 1).
        // gp walks g(zp0 - zs - 1) down the rows, qp the charges up.
        constexpr int R = kCP + 1;
        V ring[R];
        const V *h = gz + r;
#pragma unroll
        for (int j = 0; j < kCP; ++j) ring[j] = gk<M>(h, min((int)(zp0 + j) - (int)za, (int)nz), (int)tr, (int)nz);
        const T *qp = qs + za * tr + r;
        for (uint32_t zs0 = za; zs0 < zb; zs0 += R, qp += R * tr) {
#pragma unroll
          for (int u = 0; u < R; ++u) {
            if (zs0 + u >= zb) break;
            // g(zp0 - zs - 1) for the next row
            if (zs0 + u + 1 < zb) ring[(R - 1 - u) % R] = gk<M>(h, (int)zp0 - (int)(zs0 + u) - 1, (int)tr, (int)nz);
            const T qv = qp[u * tr];
#pragma unroll
            for (int j = 0; j < kCP; ++j) {
              const V gv = ring[(j - u + R) % R];
              ax[j] = fma(qv, gv.x, ax[j]);
              az[j] = fma(qv, gv.y, az[j]);
            }
          }
        }
      } else {
        // small meshes: each point sums the source rows below its own limit
        const T *q = qs + r;
        const V *h = gz + r;
        const uint32_t rs = rs0 + r;
        for (int j = 0; j < kCP; ++j) {
          if (zp0 + j > nz) continue;
          const uint32_t zend = lim[j] > rs ? min(zb, (lim[j] - rs + nx - 1) / nx) : 0u;
          for (uint32_t zs = za; zs < zend; ++zs) {
            const T qv = q[zs * tr];
            const V gv = gk<M>(h, (int)(zp0 + j) - (int)zs, (int)tr, (int)nz);
            ax[j] = fma(qv, gv.x, ax[j]);
            az[j] = fma(qv, gv.y, az[j]);
          }
        }
      }
    }
    }  // slabs
  }
#pragma unroll
  for (int sl = 0; sl < S; ++sl)
#pragma unroll
    for (int j = 0; j < kCP; ++j) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        axs[sl][j] += __shfl_down_sync(0xffffffffu, axs[sl][j], off);
        azs[sl][j] += __shfl_down_sync(0xffffffffu, azs[sl][j], off);
      }
    }
  if (half == 1 && lane == 0)
    for (int sl = 0; sl < S; ++sl)
      for (int j = 0; j < kCP; ++j) upper[sl][grp][j] = cpair<T, V>(axs[sl][j], azs[sl][j]);
  __syncthreads();
  if (half != 0 || lane != 0) return;
  T *out = CTab<T>::out(t);
  for (int sl = 0; sl < S; ++sl) {
    const uint32_t zp0 = zb0 + sl * kCZ + grp * kCP;
    for (int j = 0; j < kCP; ++j) {
      if (zp0 + j > nz) break;
      const size_t pt = (size_t)(zp0 + j) * nrow + rp;
      out[2 * pt] = axs[sl][j] + upper[sl][grp][j].x;
      out[2 * pt + 1] = azs[sl][j] + upper[sl][grp][j].y;
    }
  }
}

// grid (nr_max + 1, ceil((nz_max + 1) / (kCZ S))), kContractThreads threads,
// contract_smem<T>(nr_max, nz_max) bytes, M = contract_mirrored<T>(nr_max,
// nz_max), S = contract_slabs<T>(nz_max)
template <class T, bool M, int S>
__device__ __forceinline__ void contract_m_body(const ScState *sc, const ScTables &t, uint32_t bx, uint32_t by) {
  if (!sc->remesh || sc->sur_accepted) return;
  // FP32 tables of a tensor-core mesh: contract_tc.cuh's kernels take the solve
  if (sizeof(T) == 4 && t.tcg && sc->nx == t.tc_nr && sc->nz == t.tc_nz) return;
  const uint32_t nx = sc->nx, nz = sc->nz;
  if (bx > nx || by * kCZ * S > nz) return;
  extern __shared__ __align__(16) unsigned char contract_raw[];
  __shared__ typename CTab<T>::V upper[S][kCG][kCP];  // second halves' sums
  T *sm = (T *)contract_raw;
  if (nx == 32 && contract_tile<T, M>(nx, nz) == 32) contract_block<T, 32, M, S>(sc, t, sm, upper, bx, by);
  else contract_block<T, 0, M, S>(sc, t, sm, upper, bx, by);
}

template <class T, bool M, int S>
__global__ void __launch_bounds__(kContractThreads) k_contract_m(const ScState *sc, ScTables t) {
  contract_m_body<T, M, S>(sc, t, blockIdx.x, blockIdx.y);
}

// a solver's tables, one per beam of a lockstep launch (grid z: the beam)
struct MeshSeg {
  const ScState *sc;
  ScTables t;
};
template <class T, bool M, int S, int B>
__global__ void __launch_bounds__(kContractThreads) k_contract_m_seg(const __grid_constant__ SegArgs<MeshSeg, B> a) {
  const MeshSeg &p = a.p[blockIdx.z];
  contract_m_body<T, M, S>(p.sc, p.t, blockIdx.x, blockIdx.y);
}

// slabs per block: FP32 meshes of 256 rows and more have blocks enough to
// stage the table for 4 slabs at once (4x less table traffic from L2)
template <class T>
inline int contract_slabs(uint32_t nz_max) { return sizeof(T) == 4 && nz_max >= 256 ? 4 : 1; }

// the launch: the layout and slab count for the largest mesh the solver takes
template <class T>
inline void contract_m_merge(const std::vector<const Rec *> &recs, SegFork &, cudaStream_t st, cudaStream_t) {
  uint32_t dims[2];
  std::memcpy(dims, recs[0]->p.data() + sizeof(MeshSeg), sizeof(dims));
  const uint32_t nx_max = dims[0], nz_max = dims[1];
  const int S = contract_slabs<T>(nz_max);
  const size_t smem = contract_smem<T>(nx_max, nz_max);
  const bool mir = contract_mirrored<T>(nx_max, nz_max);
  std::vector<Rec> heads(recs.size());  // the MeshSeg heads of the records
  std::vector<const Rec *> hp(recs.size());
  for (size_t k = 0; k < recs.size(); ++k) {
    heads[k].p.assign(recs[k]->p.begin(), recs[k]->p.begin() + sizeof(MeshSeg));
    hp[k] = &heads[k];
  }
  seg_chunks<MeshSeg>(hp, [&](const auto &a, uint32_t) {
    constexpr int B = std::decay_t<decltype(a)>::kB;
    const dim3 cg(nx_max + 1, (nz_max + 1 + kCZ * S - 1) / (kCZ * S), a.nb);
    if (S == 4) {
      if (mir) k_contract_m_seg<T, true, 4, B><<<cg, kContractThreads, smem, st>>>(a);
      else k_contract_m_seg<T, false, 4, B><<<cg, kContractThreads, smem, st>>>(a);
    } else {
      if (mir) k_contract_m_seg<T, true, 1, B><<<cg, kContractThreads, smem, st>>>(a);
      else k_contract_m_seg<T, false, 1, B><<<cg, kContractThreads, smem, st>>>(a);
    }
  });
}

template <class T>
inline void contract_launch(const ScState *sc, const ScTables &t, uint32_t nx_max, uint32_t nz_max,
                            cudaStream_t st) {
  if (recorder()) {  // a lockstep range: the solver's tables and the mesh
    struct { MeshSeg m; uint32_t dims[2]; } p{{sc, t}, {nx_max, nz_max}};
    static_assert(sizeof(p) >= sizeof(MeshSeg) + 2 * sizeof(uint32_t), "layout");
    record("contract_m", &contract_m_merge<T>, 0, p, (uint64_t)p.dims[0] << 32 | p.dims[1]);
    return;
  }
  const int S = contract_slabs<T>(nz_max);
  const dim3 cg(nx_max + 1, (nz_max + 1 + kCZ * S - 1) / (kCZ * S));
  const size_t smem = contract_smem<T>(nx_max, nz_max);
  const bool mir = contract_mirrored<T>(nx_max, nz_max);
  if (S == 4) {
    if (mir) k_contract_m<T, true, 4><<<cg, kContractThreads, smem, st>>>(sc, t);
    else k_contract_m<T, false, 4><<<cg, kContractThreads, smem, st>>>(sc, t);
  } else {
    if (mir) k_contract_m<T, true, 1><<<cg, kContractThreads, smem, st>>>(sc, t);
    else k_contract_m<T, false, 1><<<cg, kContractThreads, smem, st>>>(sc, t);
  }
}

template <class T, int B>
inline void contract_seg_configure() {
  cudaFuncSetAttribute(k_contract_m_seg<T, true, 1, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  cudaFuncSetAttribute(k_contract_m_seg<T, false, 1, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  cudaFuncSetAttribute(k_contract_m_seg<T, true, 4, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  cudaFuncSetAttribute(k_contract_m_seg<T, false, 4, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
}
template <class T>
inline void contract_configure() {
  cudaFuncSetAttribute(k_contract_m<T, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  cudaFuncSetAttribute(k_contract_m<T, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  cudaFuncSetAttribute(k_contract_m<T, true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  cudaFuncSetAttribute(k_contract_m<T, false, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kContractSmem);
  contract_seg_configure<T, 4>();
  contract_seg_configure<T, 16>();
  contract_seg_configure<T, SegCap<MeshSeg>::value>();
}

}  // namespace
}  // namespace hps
