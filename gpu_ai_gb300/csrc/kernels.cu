// kernels.cu -- playout, move-list and position kernels for sm_103a.
//
// Thread-per-playout: each thread keeps its board as four 32-bit words in
// registers and plays one ply per loop iteration.  The loop is warp-uniform:
// a lane whose game ends writes its int8 outcome and, in the same iteration,
// takes the next playout index from a warp-aggregated claim on a global work
// counter, so the warp never waits for its longest game (the reference's
// coarsePlayoutKernel work queue, src/coarsePlayout.cu:73-86, done with one
// atomicAdd per warp claim instead of a per-thread atomicCAS spin).
#include "launch.h"
#include "rules.cuh"

namespace ga {

constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ uint32_t position_of(const PlayoutArgs &a, uint32_t j) {
  if (a.offsets == nullptr) return j / a.uniform_reps;
  uint32_t lo = 0, hi = a.npos;  // largest p < npos with offsets[p] <= j
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&a.offsets[mid]) <= j) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ Board load_board(const Board *p) {
  uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
  Board b;
  b.p1 = v.x; b.p2 = v.y; b.kings = v.z; b.meta = v.w;
  return b;
}

// ---- the playout kernel

template <int POLICY>
__global__ void __launch_bounds__(kPlayoutBlock) playout_kernel(PlayoutArgs a) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  Board b = {0, 0, 0, 0};
  Stream rs;
  rs.init(0, 0, 0);
  uint32_t j = 0, plies_here = 0, game_plies = 0;
  bool have = false, exhausted = false;
  unsigned long long my_plies = 0;

  for (;;) {
    // lanes without a game take the next playout indices (one atomic per warp)
    const uint32_t need = __ballot_sync(kFull, !have);
    if (need && !exhausted) {
      const uint32_t cnt = __popc(need);
      const uint32_t leader = __ffs(need) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(a.counter, cnt);
      base = __shfl_sync(kFull, base, leader);
      if (base + cnt >= a.total) exhausted = true;
      if (!have) {
        j = base + __popc(need & lt_mask);
        if (j < a.total) {
          have = true;
          b = load_board(a.pos + position_of(a, j));
          rs.init(a.seed, a.stream_base + j, 0);
          game_plies = 0;
        }
      }
    }
    if (!__any_sync(kFull, have)) break;
    if (have) {
      int outcome = 0;
      bool fin = false;
      if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) {
        fin = true;
      } else {
        const int n = ply<POLICY>(b, rs);
        if (n == 0) {
          fin = true;
          outcome = (b.meta & 1u) ? 1 : -1;  // side to move cannot move and loses
        } else if (n < 0) {
          fin = true;
          atomicOr(a.status, kStatusDepth);
        } else if (++game_plies > kMaxPlies) {
          fin = true;
          atomicOr(a.status, kStatusPlyCap);
        } else {
          plies_here++;
        }
      }
      if (fin) {
        a.out[j] = (int8_t)outcome;
        have = false;
      }
    }
  }
  if (a.plies != nullptr) {
    my_plies = plies_here;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_plies += __shfl_xor_sync(kFull, my_plies, o);
    if (lane == 0) atomicAdd(a.plies, my_plies);
  }
}

// ---- move lists (thread per board)

__global__ void genmoves_kernel(const Board *pos, uint32_t n, uint8_t *out, uint32_t max_moves,
                                uint8_t *counts, uint32_t *status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Board b = load_board(pos + i);
  Side s;
  make_side(b, s);
  const uint32_t J = jumpers(s);
  uint32_t k = 0;
  const int c = for_each_move(s, J, [&](int from, int to, uint32_t removed, int jumps,
                                        uint32_t dirs) {
    if (k < max_moves) {
      uint32_t w[8];
      pack_move(b, from, to, jumps, dirs, w);
      uint4 *dst = reinterpret_cast<uint4 *>(out + 32 * ((size_t)i * max_moves + k));
      dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
      dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
    k++;
    return false;
  });
  if (c < 0) atomicOr(status, kStatusDepth);
  if (k > max_moves) atomicOr(status, kStatusOverflow);
  counts[i] = (uint8_t)(k > 255u ? 255u : k);
}

// ---- seeded positions (thread per position, stream tag 1)

__global__ void random_positions_kernel(uint64_t seed, uint32_t n, uint32_t min_plies,
                                        uint32_t max_plies, Board *out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  Stream rs;
  rs.init(seed, p, 1);
  Board b = {0x00000FFFu, 0xFFF00000u, 0u, 0u};
  const uint32_t np = min_plies + mulhi_index(rs.next(), max_plies - min_plies + 1u);
  for (uint32_t q = 0; q < np; q++) {
    if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) break;
    if (ply_random(b, rs) <= 0) break;
  }
  uint4 *dst = reinterpret_cast<uint4 *>(out + p);
  *dst = make_uint4(b.p1, b.p2, b.kings, b.meta);
}

// ---- launchers

cudaError_t playout_occupancy(int policy, int *blocks_per_sm) {
  if (policy == 1)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, playout_kernel<1>, kPlayoutBlock, 0);
  if (policy == 2)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, playout_kernel<2>, kPlayoutBlock, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, playout_kernel<0>, kPlayoutBlock, 0);
}

cudaError_t launch_playouts(const PlayoutArgs &a, int policy, int grid, cudaStream_t s) {
  if (policy == 1) playout_kernel<1><<<grid, kPlayoutBlock, 0, s>>>(a);
  else if (policy == 2) playout_kernel<2><<<grid, kPlayoutBlock, 0, s>>>(a);
  else playout_kernel<0><<<grid, kPlayoutBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_genmoves(const Board *pos, uint32_t n, void *out, uint32_t max_moves,
                            uint8_t *counts, uint32_t *status, cudaStream_t s) {
  const int block = 128;
  genmoves_kernel<<<(n + block - 1) / block, block, 0, s>>>(pos, n, (uint8_t *)out, max_moves,
                                                           counts, status);
  return cudaGetLastError();
}

cudaError_t launch_random_positions(uint64_t seed, uint32_t n, uint32_t min_plies,
                                    uint32_t max_plies, Board *out, cudaStream_t s) {
  const int block = 128;
  random_positions_kernel<<<(n + block - 1) / block, block, 0, s>>>(seed, n, min_plies, max_plies,
                                                                   out);
  return cudaGetLastError();
}

}  // namespace ga
