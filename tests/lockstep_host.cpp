// Host check of the lockstep batch helpers in hpsim_gb300/csrc/lockstep.cuh
// (compiled with g++ by tests/test_lockstep_host.py; no GPU): the chunking
// of per-beam launch records into merged launches (seg_chunks) and the
// block -> beam search the merged kernels run (seg_find), against a linear
// scan, for parameter blocks of several sizes and ragged per-beam grids.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "lockstep.cuh"

namespace hps {
Recorder *&recorder() {
  static Recorder *r = nullptr;
  return r;
}
}  // namespace hps

using namespace hps;

static int failures = 0;
#define EXPECT(c)                                                         \
  do {                                                                    \
    if (!(c)) {                                                           \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);           \
      ++failures;                                                         \
    }                                                                     \
  } while (0)

template <size_t N>
struct Par {
  unsigned char b[N];
};

static uint32_t lcg(uint32_t &s) {
  s = s * 1664525u + 1013904223u;
  return s >> 8;
}

// m beams with ragged grids (0..max_blocks blocks each); every chunk must hold
// the next beams in order, with the smallest argument block that fits them,
// a prefix-sum table whose last entry is the chunk's grid, each beam's own
// parameter bytes, and a block search that agrees with a linear scan
template <size_t N>
static void check(size_t m, uint32_t max_blocks, uint32_t seed) {
  using P = Par<N>;
  constexpr int cap = SegCap<P>::value;
  std::vector<Rec> recs(m);
  for (size_t k = 0; k < m; ++k) {
    recs[k].blocks = max_blocks ? lcg(seed) % (max_blocks + 1) : 0;
    P p;
    for (size_t i = 0; i < N; ++i) p.b[i] = (unsigned char)(k * 131 + i * 7);
    recs[k].p.resize(sizeof(P));
    std::memcpy(recs[k].p.data(), &p, sizeof(P));
  }
  std::vector<const Rec *> v(m);
  for (size_t k = 0; k < m; ++k) v[k] = &recs[k];
  size_t next = 0, chunks = 0;
  auto f = [&](const auto &a, uint32_t blocks) {
    constexpr int B = std::remove_reference_t<decltype(a)>::kB;
    const size_t nb = a.nb;
    ++chunks;
    EXPECT(nb >= 1 && nb <= (size_t)B && (int)nb <= cap);
    // the smallest of 4, 16 and the cap that holds the chunk
    EXPECT(B == (nb <= 4 ? 4 : nb <= 16 ? 16 : cap));
    EXPECT(a.first[nb] == blocks);
    uint32_t acc = 0;
    for (size_t k = 0; k < nb; ++k) {
      EXPECT(a.first[k] == acc);
      acc += recs[next + k].blocks;
      EXPECT(std::memcmp(&a.p[k], recs[next + k].p.data(), sizeof(P)) == 0);
    }
    EXPECT(acc == blocks);
    for (uint32_t blk = 0; blk < blocks; ++blk) {
      uint32_t lin = 0;
      while (!(blk >= a.first[lin] && blk < a.first[lin + 1])) ++lin;
      uint32_t bid = 0, nblk = 0;
      const uint32_t beam = seg_find(a, blk, bid, nblk);
      EXPECT(beam == lin);
      EXPECT(bid == blk - a.first[lin]);
      EXPECT(nblk == a.first[lin + 1] - a.first[lin]);
      EXPECT(nblk > 0);
    }
    next += nb;
  };
  seg_chunks<P>(v, f);
  EXPECT(next == m);
  EXPECT(chunks == (m + cap - 1) / cap);
}

int main() {
  // the cap: as many beams as the parameter space holds, at most 64
  EXPECT(SegCap<Par<8>>::value == 64);
  EXPECT(SegCap<Par<1000>>::value == 31);
  EXPECT(SegCap<Par<1960>>::value == 16);
  EXPECT(sizeof(SegArgs<Par<1960>, SegCap<Par<1960>>::value>) <= 32764);
  EXPECT(sizeof(SegArgs<Par<8>, 64>) <= 32764);
  const size_t beams[] = {1, 2, 3, 4, 5, 15, 16, 17, 31, 32, 33, 63, 64, 65, 200, 256};
  uint32_t seed = 12345;
  for (size_t m : beams) {
    check<8>(m, 9, seed++);
    check<200>(m, 300, seed++);
    check<1000>(m, 40, seed++);
    check<1960>(m, 3, seed++);
  }
  // beams without blocks (an empty beam's launch) between beams with blocks
  check<64>(40, 1, 99);
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
