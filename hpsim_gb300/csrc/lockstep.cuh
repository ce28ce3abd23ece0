// lockstep.cuh -- batches of beams advanced in lockstep: one launch per
// kernel of an element for every beam of the batch.
//
// A batch whose simulators share a lattice topology (same element kinds in
// the same order; set points may differ) runs each element's launches once
// for all beams.  The runtime first records, per beam, the launches that
// visiting the range would issue (the host state advances as it does during
// a graph capture; the launch sites hand their per-beam parameters to the
// recorder instead of launching), then merges launch j of every beam into
// one segmented launch: particle kernels get a flat grid of every beam's
// blocks with a block -> beam table, mesh kernels a grid dimension over the
// beams.  Every beam keeps the block count, reduction scratch and counters
// it has alone, so each beam's sums run in the order they have when the beam
// is simulated by itself (the merged kernels are separate compilations of the
// same source: the compiler may fuse a few multiply-adds differently, so the
// results agree with the beam alone to FP32 rounding).  The per-beam
// parameters live in the merged kernels' own parameters (SegArgs).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace hps {

struct SegFork;

// one recorded launch of one beam
struct Rec {
  const char *site = nullptr;   // launch site: merged launches need equal sites
  // issue the merged launch of recs (one per beam, same site) on st
  void (*merge)(const std::vector<const Rec *> &recs, SegFork &a, cudaStream_t main, cudaStream_t side) = nullptr;
  uint32_t blocks = 0;          // this beam's grid blocks (flat launches)
  uint64_t shape = 0;           // launch shape every beam of a merged launch must share
  std::vector<unsigned char> p; // the launch's parameters (trivially copyable bytes)
};

// Collects the launches of one beam while a lockstep range is recorded.
// `unsupported` names a launch site that cannot be merged (the batch then
// runs as a graph of per-simulator child graphs).
struct Recorder {
  std::vector<Rec> recs;
  std::string unsupported;
};
// the recorder of the calling thread (null: launch normally)
Recorder *&recorder();

template <class P>
inline void record(const char *site, void (*merge)(const std::vector<const Rec *> &, SegFork &, cudaStream_t, cudaStream_t),
                   uint32_t blocks, const P &p, uint64_t shape = 0) {
  Rec r;
  r.site = site;
  r.merge = merge;
  r.blocks = blocks;
  r.shape = shape;
  r.p.resize(sizeof(P));
  std::memcpy(r.p.data(), &p, sizeof(P));
  recorder()->recs.push_back(std::move(r));
}

// The events of a merged range's side-stream branch (the Green's tables):
// it forks from the main stream and joins it again.
struct SegFork {
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

// The per-beam parameters of one merged launch, passed as the kernel's own
// parameters: they live in the constant bank, and a block's beam is a value
// uniform over the block (its block index against the beams' first blocks,
// or a grid index), so a beam's parameters are read as uniform constants, as
// a single-beam launch reads its own, instead of occupying registers.
// Kernel parameters may take up to 32,764 bytes: a launch takes at most
// SegCap<P> beams and a batch with more runs in several launches.
constexpr size_t kSegParamBytes = 32000;
template <class P>
struct SegCap {
  static constexpr size_t fit = (kSegParamBytes - 8 - 4 * 65) / sizeof(P);
  static constexpr int value = fit < 64 ? (int)fit : 64;
  static_assert(value >= 16, "per-beam parameters too large for a merged launch");
};
template <class P, int B>
struct SegArgs {
  static constexpr int kB = B;
  uint32_t nb;            // beams in this launch
  uint32_t first[B + 1];  // per beam: its first block (flat launches); first[nb]: the launch's blocks
  P p[B];
};

// Launch recs (one per beam) in chunks of at most SegCap<P> beams, each with
// the smallest argument block that holds it: f(args, blocks) per chunk, with
// args a SegArgs<P, 4 | 16 | SegCap<P>> and blocks the chunk's flat grid.
template <class P, int B, class F>
inline void seg_chunk(const std::vector<const Rec *> &recs, size_t k0, size_t k1, F &f) {
  static_assert(sizeof(SegArgs<P, B>) <= 32764, "a merged launch's parameters exceed the kernel parameter limit");
  std::vector<unsigned char> buf(sizeof(SegArgs<P, B>), 0);  // up to 32 KB: not on the stack
  SegArgs<P, B> &a = *reinterpret_cast<SegArgs<P, B> *>(buf.data());
  a.nb = (uint32_t)(k1 - k0);
  uint32_t acc = 0;
  for (size_t k = k0; k < k1; ++k) {
    a.first[k - k0] = acc;
    acc += recs[k]->blocks;
    std::memcpy(&a.p[k - k0], recs[k]->p.data(), sizeof(P));
  }
  a.first[a.nb] = acc;
  f(a, acc);
}
template <class P, class F>
inline void seg_chunks(const std::vector<const Rec *> &recs, F &&f) {
  constexpr int cap = SegCap<P>::value;
  for (size_t k0 = 0; k0 < recs.size(); k0 += cap) {
    const size_t k1 = std::min(recs.size(), k0 + (size_t)cap), m = k1 - k0;
    if (m <= 4) seg_chunk<P, 4>(recs, k0, k1, f);
    else if (m <= 16) seg_chunk<P, 16>(recs, k0, k1, f);
    else seg_chunk<P, cap>(recs, k0, k1, f);
  }
}

#ifdef __CUDACC__
#define HPS_SEG_FN __host__ __device__ __forceinline__
#else
#define HPS_SEG_FN inline
#endif
// the beam of flat block blk, its block index within the beam and the beam's
// block count (uniform over the block: a binary search of the constant-bank
// table with the block index)
template <class P, int B>
HPS_SEG_FN uint32_t seg_find(const SegArgs<P, B> &a, uint32_t blk, uint32_t &bid, uint32_t &nblk) {
  uint32_t lo = 0, hi = a.nb;  // first[lo] <= blk < first[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (blk >= a.first[mid]) lo = mid;
    else hi = mid;
  }
  bid = blk - a.first[lo];
  nblk = a.first[lo + 1] - a.first[lo];
  return lo;
}
#undef HPS_SEG_FN

}  // namespace hps
