// cpu_playouts.cpp -- the stronger CPU baseline (measurement only).
//
// The project's own bitboard ply (gpu_ai_gb300/csrc/rules.cuh built for the
// host) with per-playout Philox streams, on every host core: the best CPU
// form of the random playout path, timed beside the reference's
// HostPlayoutDriver (src/playout.cpp:17-32), which generates its move list
// twice per ply over a byte board and draws from glibc rand().  Playout j uses
// stream (seed, stream_base + j, tag 0) exactly as the GPU kernel does, so its
// outcomes equal the GPU's; bench.py's CPU-baseline leg and the CPU tests are
// its only users.
#include "../gpu_ai_gb300/csrc/rules.cuh"

#include <atomic>
#include <cstdint>
#include <thread>
#include <vector>

using namespace ga;

namespace {

int8_t playout(Board b, uint64_t seed, uint64_t id, uint32_t *plies) {
  Stream rs;
  rs.init(seed, id, 0);
  uint32_t p = 0;
  for (;;) {
    if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) break;
    const int n = ply<0>(b, rs);
    if (n == 0) {
      *plies += p;
      return (b.meta & 1u) ? 1 : -1;  // the side to move cannot move: it loses
    }
    if (n < 0) break;
    p++;
  }
  *plies += p;
  return 0;
}

}  // namespace

extern "C" {

// reps[p] playouts of board pos[p] (4 words each), outcomes in order into out;
// nthreads <= 0 uses every hardware thread.  Returns the plies played.
uint64_t cp_playouts(const uint32_t *pos, const uint32_t *reps, uint32_t npos, uint64_t seed, uint64_t stream_base,
                     int8_t *out, int nthreads) {
  std::vector<uint64_t> first(npos + 1, 0);
  for (uint32_t p = 0; p < npos; p++) first[p + 1] = first[p] + reps[p];
  const uint64_t total = first[npos];
  if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
  if (nthreads < 1) nthreads = 1;
  constexpr uint64_t kChunk = 256;
  std::atomic<uint64_t> next{0};
  std::vector<uint64_t> plies(nthreads, 0);
  auto work = [&](int t) {
    uint32_t my = 0;
    uint64_t acc = 0;
    uint32_t p = 0;
    for (;;) {
      const uint64_t lo = next.fetch_add(kChunk);
      if (lo >= total) break;
      const uint64_t hi = lo + kChunk < total ? lo + kChunk : total;
      for (uint64_t j = lo; j < hi; j++) {  // chunks are claimed in increasing order: p only grows
        while (first[p + 1] <= j) p++;
        const uint32_t *w = pos + 4 * (size_t)p;
        my = 0;
        out[j] = playout(Board{w[0], w[1], w[2], w[3]}, seed, stream_base + j, &my);
        acc += my;
      }
    }
    plies[t] = acc;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &x : th) x.join();
  uint64_t sum = 0;
  for (uint64_t v : plies) sum += v;
  return sum;
}

}  // extern "C"
