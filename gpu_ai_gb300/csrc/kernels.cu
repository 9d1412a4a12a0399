// kernels.cu -- playout, move-list and position kernels for sm_103a.
//
// Thread-per-playout: each thread keeps its board as four 32-bit words in
// registers and plays one ply per loop iteration.  The loop is warp-uniform:
// a lane whose game ends writes its int8 outcome and, at the next refill
// iteration (every fourth), takes the next playout index from a
// warp-aggregated claim on a global work counter, so the warp never waits for
// its longest game (the reference's coarsePlayoutKernel work queue,
// src/coarsePlayout.cu:73-86, done with one atomicAdd per warp claim instead
// of a per-thread atomicCAS spin).
#include "detmath.cuh"
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

// Random-stream id of playout j, which plays position p.
__device__ __forceinline__ uint64_t stream_of(const PlayoutArgs &a, uint32_t p, uint32_t j) {
  if (a.pos_stream == nullptr) return a.stream_base + j;
  const uint32_t first = a.offsets ? __ldg(&a.offsets[p]) : p * a.uniform_reps;
  return __ldg(&a.pos_stream[p]) + (j - first);
}

__device__ __forceinline__ Board load_board(const Board *p) {
  uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
  Board b;
  b.p1 = v.x; b.p2 = v.y; b.kings = v.z; b.meta = v.w;
  return b;
}

// ---- the playout kernel

// Lanes without a game take the next playout indices: one atomicAdd per warp.
// Returns true for lanes that got a playout (index in j).
__device__ __forceinline__ bool claim(const PlayoutArgs &a, bool have, uint32_t &j, bool &exhausted,
                                      uint32_t lane) {
  if (exhausted) return false;  // warp-uniform
  const uint32_t need = __ballot_sync(kFull, !have);
  if (!need) return false;
  const uint32_t cnt = __popc(need);
  const uint32_t leader = __ffs(need) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(a.counter, cnt);
  base = __shfl_sync(kFull, base, leader);
  if (base + cnt >= a.total) exhausted = true;
  if (have) return false;
  j = base + __popc(need & ((1u << lane) - 1u));
  return j < a.total;
}

// Resident blocks per SM that the register budget is sized for: 64 registers
// a thread for blocks of 256 or more threads (80 for the reference heuristic
// at 256: 3 blocks), 72 (96 for the reference heuristic) for smaller blocks.
template <int POLICY, int BLOCK>
constexpr int playout_min_blocks() {
  constexpr int regs = BLOCK >= 256 ? (POLICY == 1 && BLOCK == 256 ? 80 : 64) : (POLICY == 1 ? 96 : 72);
  return 65536 / (regs * BLOCK);
}

// Block pool of the pooled layout: a shared-memory lock that lane 0 tries to
// take once (a warp that does not get it carries on as the unpooled kernel
// does and tries again on a later iteration: nothing ever waits for it), and
// the two pools' capacity.
constexpr uint32_t kPoolCap = 64;

__device__ __forceinline__ bool pool_lock(uint32_t *lock, uint32_t lane) {
  uint32_t got = 0;
  if (lane == 0) got = atomicCAS(lock, 0u, 1u) == 0u ? 1u : 0u;
  got = __shfl_sync(kFull, got, 0);
  __threadfence_block();
  __syncwarp();
  return got != 0;
}

__device__ __forceinline__ void pool_unlock(uint32_t *lock, uint32_t lane) {
  __threadfence_block();
  __syncwarp();
  if (lane == 0) atomicExch(lock, 0u);
}

__device__ __forceinline__ uint32_t vload(const uint32_t *p) { return *reinterpret_cast<const volatile uint32_t *>(p); }

template <int POLICY, int BLOCK, bool POOL>
__global__ void __launch_bounds__(BLOCK, (playout_min_blocks<POLICY, BLOCK>())) playout_kernel(PlayoutArgs a) {
  if (a.dev_sizes != nullptr) {
    a.npos = __ldg(&a.dev_sizes[0]);
    a.total = __ldg(&a.dev_sizes[1]);
  }
  const uint32_t lane = threadIdx.x & 31u;
  Board b = {0, 0, 0, 0};
  uint32_t j = 0, plies_here = 0, game_plies = 0;
  bool have = false, exhausted = false;

  static_assert(POLICY >= 0 && POLICY <= 2, "policies: 0 random, 1 reference heuristic, 2 eps-greedy");
  {
    // Uniform random policy: at most one draw per ply, so Philox blocks are
    // generated for the whole warp every fourth iteration (DrawRing keeps four
    // or more draws buffered) and new games start on those iterations too.
    // eps-greedy (policy 2, play_ply_eps_sched) takes at most two draws per
    // ply and refills every second iteration.  The reference heuristic
    // (policy 1, play_ply_heur_sched) takes two draws per legal move: its ply
    // loops over the moves for the warp's longest move list and refills the
    // ring every second step, so Philox still runs for the whole warp at once.
    // Plies whose capture can be extended take longer code.  Those with one
    // legal move (about two thirds) follow their chain at once; the others,
    // men's multi-jumps (about 1% of plies) and plies where a king's capture
    // can continue (about 0.2%, the costlier depth-first search), are deferred
    // to every kMenPeriod-th (eps-greedy and reference heuristic only:
    // defer_men) and every king_period(POLICY)-th iteration, so that the lanes
    // needing that code run it together and the other iterations stay
    // branch-free.
    // Once the work counter is exhausted, a warp with sparse_lanes(POLICY) or fewer
    // games defers nothing: its few games are latency-bound.
    //
    // Once the work counter is exhausted, every compact_period(POLICY)-th iteration the
    // block packs its unfinished games (board, random-stream state, counters)
    // into its lowest threads through shared memory; warps left without games
    // wait at the next barrier instead of issuing empty iterations.  The loop
    // ends for the whole block when it has no game left.
    //
    // Pooled layout (POOL): while work remains, a lane whose ply must wait for
    // a men's multi-jump or king capture search hands its game to the block's
    // pending pool and takes a new one; once the pool holds 32 such games, the
    // warp that sees it moves its own games to the block's ready pool, takes
    // the 32 and plays their deferred plies at once with every lane busy.
    // Free lanes take ready games before new ones (and pending ones once the
    // work ran out); compaction packs the pools' games too.  A game keeps its
    // whole state (board, stream, ring of draws) wherever it is played, so
    // the outcomes are the same as without the pools.
    constexpr int kWords = 17;
    constexpr uint32_t kCap = POOL ? kPoolCap : 1u;
    __shared__ uint32_t s_slot[kWords][BLOCK];
    __shared__ uint32_t s_cnt[BLOCK / 32];
    __shared__ uint32_t s_pend[kWords][kCap];   // games waiting for a deferred ply
    __shared__ uint32_t s_ready[kWords][kCap];  // games a swap moved out of their lane
    __shared__ uint32_t s_pool[4];              // lock, pending games, ready games
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    if constexpr (POOL) {
      if (threadIdx.x < 4) s_pool[threadIdx.x] = 0;
      __syncthreads();
    }
    DrawRing rs;
    rs.start(0, 0, 0);
    uint32_t pend = 0;    // deferred ply: 0 none, 1 men's multi-jump, 2 king capture search
    bool sparse = false;  // warp-uniform: the work ran out and the warp holds sparse_lanes(POLICY) games or fewer
    constexpr uint32_t kCompactPeriod = compact_period(POLICY);
    constexpr uint32_t kSparseLanes = sparse_lanes(POLICY);
    auto pick = [&](uint32_t n) { return rs.pick(n); };
    // a game's state in word q of column idx of a [kWords][stride] area
    auto put = [&](uint32_t *area, uint32_t stride, uint32_t idx) {
      const uint32_t v[kWords] = {b.p1, b.p2, b.kings, b.meta, j, game_plies, pend,
                                  rs.a0, rs.a1, rs.a2, rs.a3, rs.b0, rs.b1, rs.b2, rs.b3, rs.k, rs.avail};
#pragma unroll
      for (int q = 0; q < kWords; q++) area[q * stride + idx] = v[q];
    };
    auto take = [&](const uint32_t *area, uint32_t stride, uint32_t idx) {
      b.p1 = area[idx]; b.p2 = area[stride + idx]; b.kings = area[2 * stride + idx]; b.meta = area[3 * stride + idx];
      j = area[4 * stride + idx];
      game_plies = area[5 * stride + idx];
      pend = area[6 * stride + idx];
      rs.start(a.seed, stream_of(a, position_of(a, j), j), 0);  // then the buffered draws and counter
      rs.a0 = area[7 * stride + idx]; rs.a1 = area[8 * stride + idx]; rs.a2 = area[9 * stride + idx];
      rs.a3 = area[10 * stride + idx]; rs.b0 = area[11 * stride + idx]; rs.b1 = area[12 * stride + idx];
      rs.b2 = area[13 * stride + idx]; rs.b3 = area[14 * stride + idx];
      rs.k = area[15 * stride + idx];
      rs.avail = area[16 * stride + idx];
    };
    // Claim order (equal repetitions, at most BLOCK positions): lanes take
    // the playouts of positions with more pieces first.  Their games are
    // longer on average, so the last claims of the batch are the shorter
    // games and less of the batch tail waits on a game that started late.
    // Playout j keeps its index (its outcome slot and random stream); only the
    // order in which lanes take the playouts changes.
    __shared__ uint16_t s_order[BLOCK];
    __shared__ uint8_t s_key[BLOCK];
    const bool ordered = a.offsets == nullptr && a.npos > 1 && a.npos <= (uint32_t)BLOCK;
    if (ordered) {  // uniform over the block
      const uint32_t t = threadIdx.x;
      if (t < a.npos) {
        const Board pb = load_board(a.pos + t);
        s_key[t] = (uint8_t)popc(pb.p1 | pb.p2);
      }
      __syncthreads();
      if (t < a.npos) {
        const uint32_t kt = s_key[t];
        uint32_t rank = 0;
        for (uint32_t u = 0; u < a.npos; u++) {
          const uint32_t ku = s_key[u];
          rank += (ku > kt || (ku == kt && u < t)) ? 1u : 0u;
        }
        s_order[rank] = (uint16_t)t;
      }
      __syncthreads();
    }
    constexpr uint32_t kRefillMask = POLICY == 2 ? 1u : 3u;
    for (uint32_t it = 0;; ++it) {
      bool swapped = false;  // warp-uniform: this iteration's games came from the pending pool
      if constexpr (POOL) {
        // 32 games wait for their deferred ply and the ready pool has room for
        // this warp's games: play the 32 in this warp now (checked on the men's
        // phase iterations only)
        if (!exhausted && (it & (kMenPeriod - 1u)) == kMenPhase) {
          uint32_t ok = 0;
          if (lane == 0) ok = vload(&s_pool[1]) >= 32u && vload(&s_pool[2]) + 32u <= kCap;
          if (__shfl_sync(kFull, ok, 0) && pool_lock(&s_pool[0], lane)) {
            const uint32_t npend = vload(&s_pool[1]), nready = vload(&s_pool[2]);
            const uint32_t hm = __ballot_sync(kFull, have);
            if (npend >= 32u && nready + (uint32_t)__popc(hm) <= kCap) {
              if (have) put(&s_ready[0][0], kCap, nready + __popc(hm & lt));
              take(&s_pend[0][0], kCap, npend - 32u + lane);
              have = true;
              if (lane == 0) {
                s_pool[1] = npend - 32u;
                s_pool[2] = nready + __popc(hm);
              }
              swapped = true;
            }
            pool_unlock(&s_pool[0], lane);
            if (swapped) rs.refill();
          }
        }
      }
      if ((it & kRefillMask) == 0) {
        if constexpr (POOL) {
          // free lanes take ready games (and, once the work ran out, pending ones)
          const uint32_t fm = __ballot_sync(kFull, !have);
          if (fm) {
            uint32_t avail = 0;
            if (lane == 0) avail = vload(&s_pool[2]) + (exhausted ? vload(&s_pool[1]) : 0u);
            if (__shfl_sync(kFull, avail, 0) && pool_lock(&s_pool[0], lane)) {
              const uint32_t nr = vload(&s_pool[2]), np = exhausted ? vload(&s_pool[1]) : 0u;
              const uint32_t rank = __popc(fm & lt), k = min((uint32_t)__popc(fm), nr + np);
              if (!have && rank < k) {
                if (rank < nr) take(&s_ready[0][0], kCap, nr - 1u - rank);
                else take(&s_pend[0][0], kCap, np - 1u - (rank - nr));
                have = true;
              }
              if (lane == 0) {
                const uint32_t from_r = min(k, nr);
                s_pool[2] = nr - from_r;
                if (exhausted) s_pool[1] = np - (k - from_r);
              }
              pool_unlock(&s_pool[0], lane);
            }
          }
        }
        if (claim(a, have, j, exhausted, lane)) {
          have = true;
          if (ordered) {  // claim index -> playout index
            const uint32_t k = j / a.uniform_reps;
            j = (uint32_t)s_order[k] * a.uniform_reps + (j - k * a.uniform_reps);
          }
          const uint32_t p = position_of(a, j);
          if (GA_IN_BOUNDS(p < a.npos, a.status)) b = load_board(a.pos + p);
          rs.start(a.seed, stream_of(a, p, j), 0);
          game_plies = 0;
        }
        if (have) rs.refill();
      }
      const bool men_ok = !defer_men(POLICY) || sparse || swapped || (it & (kMenPeriod - 1u)) == kMenPhase;
      const bool king_ok = sparse || swapped || (it & (king_period(POLICY) - 1u)) == kKingPhase;
      bool deferred_now = false;  // this iteration's ply was deferred (a candidate for the pending pool)
      do {
        if (!have) break;
        if ((pend == 1u && !men_ok) || (pend == 2u && !king_ok)) break;  // still deferred
        if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) {
          if (GA_IN_BOUNDS(j < a.total, a.status)) a.out[j] = 0;
          have = false;
          break;
        }
        int n;
        if constexpr (POLICY == 2) {
          n = play_ply_eps_sched(b, rs, men_ok, king_ok);
        } else if constexpr (POLICY == 1) {
          RingOnDemand more{rs};
          n = play_ply_heur_sched(
              b, rs, more, men_ok, king_ok, [](uint32_t m) { return __reduce_max_sync(__activemask(), m); },
              [&] { rs.refill(); });
        } else {
          n = play_ply_sched(b, pick, men_ok, king_ok);
        }
        if (n == kNeedMen || n == kNeedKing) {
          pend = n == kNeedMen ? 1u : 2u;
          deferred_now = true;
          break;
        }
        pend = 0;
        if (n > 0 && ++game_plies <= kMaxPlies) {
          plies_here++;
          break;
        }
        if (n < 0) atomicOr(a.status, kStatusDepth);
        else if (n > 0) atomicOr(a.status, kStatusPlyCap);
        if (GA_IN_BOUNDS(j < a.total, a.status))
          a.out[j] = (int8_t)(n == 0 ? ((b.meta & 1u) ? 1 : -1) : 0);  // side to move cannot move: loses
        have = false;
      } while (false);
      if constexpr (POOL) {
        // hand deferred games to the pending pool while work remains
        if (!exhausted && !sparse) {
          const uint32_t pm = __ballot_sync(kFull, deferred_now);
          uint32_t room = 0;
          if (pm && lane == 0) room = vload(&s_pool[1]) < kCap;
          if (pm && __shfl_sync(kFull, room, 0) && pool_lock(&s_pool[0], lane)) {
            const uint32_t np = vload(&s_pool[1]);
            const uint32_t k = min((uint32_t)__popc(pm), kCap - np), rank = __popc(pm & lt);
            if (deferred_now && rank < k) {
              put(&s_pend[0][0], kCap, np + rank);
              have = false;
              pend = 0;
            }
            if (lane == 0) s_pool[1] = np + k;
            pool_unlock(&s_pool[0], lane);
          }
        }
      }

      if ((it & (kCompactPeriod - 1u)) != kCompactPeriod - 1u) {
        if (exhausted) {
          const uint32_t live = __ballot_sync(kFull, have);
          sparse = __popc(live) <= kSparseLanes;
          // a warp with no game left skips ahead to the block's next compaction point
          if (!live) it = (it | (kCompactPeriod - 1u)) - 1u;
        }
        continue;
      }
      if (!exhausted) {
        // A warp whose lanes are all busy makes no claims: it reads the work
        // counter itself.  Counter values only grow, and a warp waits at the
        // barrier below only after it saw the counter at or past the total, so
        // every other warp of the block sees that too at its next compaction
        // point and joins it: no barrier is needed while work remains.
        uint32_t c = 0;
        if (lane == 0) c = *reinterpret_cast<volatile const uint32_t *>(a.counter);
        if (__shfl_sync(kFull, c, 0) < a.total) continue;  // warp-uniform
        exhausted = true;
      }
      // Only warps that know the work is exhausted get here; they all pass the
      // same sequence of compaction points (it % compact_period equal, absolute
      // iteration counts may differ).  This barrier also keeps a fast warp from
      // writing s_cnt for the next point while a slow one still reads it.
      __syncthreads();
      const uint32_t m = __ballot_sync(kFull, have);
      if (lane == 0) s_cnt[warp] = __popc(m);
      __syncthreads();
      uint32_t total = 0, before = 0, busy_warps = 0;
#pragma unroll
      for (uint32_t w = 0; w < BLOCK / 32; w++) {
        const uint32_t c = s_cnt[w];
        before += w < warp ? c : 0u;
        total += c;
        busy_warps += c ? 1u : 0u;
      }
      // games still in the pools (stable here: every warp knows the work ran
      // out, so none pushes, and all are between the two barriers)
      const uint32_t nr = POOL ? vload(&s_pool[2]) : 0u, np = POOL ? vload(&s_pool[1]) : 0u;
      if (total + nr + np == 0) break;
      sparse = __popc(m) <= kSparseLanes;
      if (nr + np == 0 && (total + 31u) / 32u >= busy_warps) continue;  // packing would free no warp
      const uint32_t n_all = min((uint32_t)BLOCK, total + nr + np);  // games the block's lanes hold after packing
      if (have) put(&s_slot[0][0], BLOCK, before + __popc(m & lt));
      if constexpr (POOL) {
        // pool games fill the lanes after the live ones: ready games first
        const uint32_t t = threadIdx.x;
        if (t >= total && t < n_all) {
          const uint32_t e = t - total;
          uint32_t v[kWords];
          if (e < nr) {
#pragma unroll
            for (int q = 0; q < kWords; q++) v[q] = s_ready[q][nr - 1u - e];
          } else {
#pragma unroll
            for (int q = 0; q < kWords; q++) v[q] = s_pend[q][np - 1u - (e - nr)];
          }
#pragma unroll
          for (int q = 0; q < kWords; q++) s_slot[q][t] = v[q];
        }
      }
      __syncthreads();
      if constexpr (POOL) {
        // every thread has read the counts (before the barrier above); a
        // second barrier publishes the new ones before any lane pops again
        if (threadIdx.x == 0) {
          const uint32_t moved = n_all - total, from_r = min(moved, nr);
          s_pool[2] = nr - from_r;
          s_pool[1] = np - (moved - from_r);
        }
        __syncthreads();
      }
      have = threadIdx.x < n_all;
      sparse = n_all <= warp * 32u + kSparseLanes;  // this warp now holds min(32, n_all - 32 * warp) games
      if (have) take(&s_slot[0][0], BLOCK, threadIdx.x);
    }
  }
  if (a.plies != nullptr) {
    unsigned long long my_plies = plies_here;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_plies += __shfl_xor_sync(kFull, my_plies, o);
    if (lane == 0) atomicAdd(a.plies, my_plies);
  }
}

// ---- warp per playout (uniform random policy)

// Warp-cooperative layout, the shape of the reference's playoutKernel
// (src/multiplePlayout.cu:14-52: one block of threads per playout, one thread
// per square), kept as the alternative the autotuner measures against thread
// per playout.  Lane s owns dark square s.  Each ply every lane counts the
// legal moves that start on its square (only captures when the side to move
// has one); a warp prefix sum over the lanes puts them in the reference's
// move-list order (squares ascending, each square's moves in its DFS /
// direction order).  Lane 0 draws the move index from the playout's stream
// exactly as the thread-per-playout kernel does (one draw per ply with two or
// more moves), the lane owning that index applies its move, and the board is
// broadcast.  Outcomes equal the thread-per-playout kernel's bit for bit.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) warp_playout_kernel(PlayoutArgs a) {
  if (a.dev_sizes != nullptr) {
    a.npos = __ldg(&a.dev_sizes[0]);
    a.total = __ldg(&a.dev_sizes[1]);
  }
  const uint32_t lane = threadIdx.x & 31u;
  const int sq = (int)lane;
  unsigned long long plies_here = 0;
  for (;;) {
    uint32_t j = 0;
    if (lane == 0) j = atomicAdd(a.counter, 1u);
    j = __shfl_sync(kFull, j, 0);
    if (j >= a.total) break;
    const uint32_t p = position_of(a, j);
    Board b = load_board(a.pos + p);
    Stream rs;  // drawn by lane 0 only
    rs.init(a.seed, stream_of(a, p, j), 0);
    uint32_t game_plies = 0;
    int outcome = 0;
    for (;;) {
      if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) break;  // draw
      Side s;
      make_side(b, s);
      const uint32_t J = jumpers(s);
      uint32_t md[4];
      direct_masks(s, md);
      int cnt = 0;
      if (J) {
        if ((J >> sq) & 1u) cnt = capture_walk(s, sq, [](int, uint32_t, int, uint32_t) { return false; });
      } else {
        cnt = (int)(((md[0] >> sq) & 1u) + ((md[1] >> sq) & 1u) + ((md[2] >> sq) & 1u) + ((md[3] >> sq) & 1u));
      }
      if (__any_sync(kFull, cnt < 0)) {  // capture deeper than kMaxDepth
        if (lane == 0) atomicOr(a.status, kStatusDepth);
        outcome = 0;
        break;
      }
      uint32_t incl = (uint32_t)cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= (uint32_t)o) incl += t;
      }
      const uint32_t n = __shfl_sync(kFull, incl, 31);
      if (n == 0) {
        outcome = (b.meta & 1u) ? 1 : -1;  // side to move cannot move: loses
        break;
      }
      uint32_t idx = 0;
      if (lane == 0 && n >= 2) idx = mulhi_index(rs.next(), n);
      idx = __shfl_sync(kFull, idx, 0);
      const uint32_t excl = incl - (uint32_t)cnt;
      const bool mine = idx >= excl && idx < incl;
      const int owner = __ffs(__ballot_sync(kFull, mine)) - 1;
      if (mine) {
        uint32_t want = idx - excl;
        if (J) {
          capture_walk(s, sq, [&](int t, uint32_t removed, int, uint32_t) {
            if (want-- != 0) return false;
            apply_move(b, sq, t, removed);
            return true;
          });
        } else {
          for (int d = 0; d < 4; d++)
            if ((md[d] >> sq) & 1u) {
              if (want == 0) {
                apply_move(b, sq, sq + step_off(sq, d), 0u);
                break;
              }
              want--;
            }
        }
      }
      b.p1 = __shfl_sync(kFull, b.p1, owner);
      b.p2 = __shfl_sync(kFull, b.p2, owner);
      b.kings = __shfl_sync(kFull, b.kings, owner);
      b.meta = __shfl_sync(kFull, b.meta, owner);
      if (++game_plies > kMaxPlies) {
        if (lane == 0) atomicOr(a.status, kStatusPlyCap);
        outcome = 0;
        break;
      }
      plies_here++;
    }
    if (lane == 0) a.out[j] = (int8_t)outcome;
  }
  if (a.plies != nullptr && lane == 0) atomicAdd(a.plies, plies_here);
}

// ---- learned-proposal plies (thread per playout)

// One guided ply: the legal moves of playout j's board are weighted by the
// network's policy -- the softmax at temperature T of each move's (from, to)
// logit over the legal pairs, a pair's share split equally among the moves
// that have it -- as integers w = max(1, floor(2^24 e^((l - lmax) / T)) / mult),
// and the move taken is the first whose running weight sum exceeds
// mulhi(draw, sum of w).  The draw is draw number `ply` of the playout's
// stream under tag kTagProposal (the playout's own random moves use tag 0).
// The float steps are detmath.cuh's, so a CPU replay fed the same logits and
// draws picks the same move.  A finished game keeps its board.
__global__ void __launch_bounds__(128) proposal_ply_kernel(ProposalArgs a) {
  if (a.dev_sizes != nullptr) {
    a.npos = __ldg(&a.dev_sizes[0]);
    a.total = __ldg(&a.dev_sizes[1]);
  }
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0 && a.out_sizes != nullptr) {
    a.out_sizes[0] = a.total;
    a.out_sizes[1] = a.total;
  }
  if (j >= a.total) return;
  uint32_t row = j;
  uint64_t sid = a.stream_base + j;
  if (a.per_position) {
    PlayoutArgs pa{};
    pa.offsets = a.offsets;
    pa.npos = a.npos;
    pa.uniform_reps = a.uniform_reps;
    pa.stream_base = a.stream_base;
    pa.pos_stream = a.pos_stream;
    row = position_of(pa, j);
    sid = stream_of(pa, row, j);
  } else if (a.play_stream != nullptr) {
    sid = a.play_stream[j];
  }
  Board b = load_board(a.in + row);
  const uint16_t *lg = a.logits + (size_t)row * 1024u;
  if (a.trace_boards) a.trace_boards[j] = b;
  if (a.trace_logits) {
    const uint4 *src = reinterpret_cast<const uint4 *>(lg);
    uint4 *dst = reinterpret_cast<uint4 *>(a.trace_logits + (size_t)j * 1024u);
    for (int q = 0; q < 128; q++) dst[q] = src[q];
  }
  if (a.out_stream) a.out_stream[j] = sid;
  if (((b.meta >> 8) & 0xffu) < (uint32_t)kDrawPlies) {
    Side sd;
    make_side(b, sd);
    const uint32_t J = jumpers(sd);
    uint32_t c[4] = {a.ply >> 2, (uint32_t)sid, (uint32_t)(sid >> 32), kTagProposal};
    philox4x32_10(c, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
    const uint32_t w = a.ply & 3u;
    const uint32_t draw = w == 0 ? c[0] : (w == 1 ? c[1] : (w == 2 ? c[2] : c[3]));
    uint16_t pair[kProposalMaxMoves];
    int k = 0;
    float lmax = -3.0e38f;
    const int n = for_each_move(sd, J, [&](int from, int to, uint32_t, int, uint32_t) {
      if (k < kProposalMaxMoves) {
        pair[k] = (uint16_t)(from * 32 + to);
        lmax = fmaxf(lmax, __uint_as_float((uint32_t)lg[pair[k]] << 16));
      }
      k++;
      return false;
    });
    if (n > 0) {
      uint32_t pick = 0;
      if (n > kProposalMaxMoves) {
        pick = mulhi_index(draw, (uint32_t)n);
      } else if (n >= 2) {
        uint32_t wt[kProposalMaxMoves];
        uint32_t sum = 0;
        for (int m = 0; m < n; m++) {
          uint32_t mult = 0;
          for (int q = 0; q < n; q++) mult += pair[q] == pair[m];
          const float l = __uint_as_float((uint32_t)lg[pair[m]] << 16);
          const float e = dm::det_exp(dm::mul(dm::sub(l, lmax), a.inv_temperature));
          const uint32_t v = __float2uint_rz(dm::mul(e, 16777216.0f)) / mult;
          wt[m] = v > 0u ? v : 1u;
          sum += wt[m];
        }
        const uint32_t r = mulhi_index(draw, sum);
        uint32_t acc = 0;
        for (int m = 0; m < n; m++) {
          acc += wt[m];
          if (acc > r) {
            pick = (uint32_t)m;
            break;
          }
        }
      }
      uint32_t at = 0;
      const Board before = b;
      for_each_move(sd, J, [&](int from, int to, uint32_t removed, int, uint32_t) {
        if (at++ != pick) return false;
        b = before;
        apply_move(b, from, to, removed);
        return true;
      });
    }
  }
  uint4 *dst = reinterpret_cast<uint4 *>(a.out + j);
  *dst = make_uint4(b.p1, b.p2, b.kings, b.meta);
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

// Position p: U{min_plies..max_plies} plies of POLICY from the standard
// start (random stream (seed, p, 1)), stopping early at a finished game.
template <int POLICY>
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
    if (ply<POLICY>(b, rs) <= 0) break;
  }
  uint4 *dst = reinterpret_cast<uint4 *>(out + p);
  *dst = make_uint4(b.p1, b.p2, b.kings, b.meta);
}

// ---- launchers

template <int POLICY, bool POOL>
static const void *kernel_for(int block) {
  switch (block) {
    case 64: return (const void *)playout_kernel<POLICY, 64, POOL>;
    case 128: return (const void *)playout_kernel<POLICY, 128, POOL>;
    case 512: return (const void *)playout_kernel<POLICY, 512, POOL>;
    default: return (const void *)playout_kernel<POLICY, 256, POOL>;
  }
}

static const void *warp_kernel_for(int block) {
  switch (block) {
    case 64: return (const void *)warp_playout_kernel<64>;
    case 128: return (const void *)warp_playout_kernel<128>;
    case 512: return (const void *)warp_playout_kernel<512>;
    default: return (const void *)warp_playout_kernel<256>;
  }
}

static const void *playout_fn(int policy, int block, int layout) {
  if (layout == kLayoutWarp) return warp_kernel_for(block);
  if (layout == kLayoutPooled) {
    if (policy == 1) return kernel_for<1, true>(block);
    if (policy == 2) return kernel_for<2, true>(block);
    return kernel_for<0, true>(block);
  }
  if (policy == 1) return kernel_for<1, false>(block);
  if (policy == 2) return kernel_for<2, false>(block);
  return kernel_for<0, false>(block);
}

bool valid_block(int block) { return block == 64 || block == 128 || block == 256 || block == 512; }

cudaError_t playout_occupancy(int policy, int block, int *blocks_per_sm, int layout) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, playout_fn(policy, block, layout), block, 0);
}

cudaError_t launch_playouts(const PlayoutArgs &a, int policy, int block, int grid, cudaStream_t s, int layout) {
  if (layout == kLayoutWarp && policy != 0) return cudaErrorInvalidValue;
  void *args[] = {const_cast<PlayoutArgs *>(&a)};
  return cudaLaunchKernel(playout_fn(policy, block, layout), dim3(grid), dim3(block), args, 0, s);
}

cudaError_t launch_proposal_ply(const ProposalArgs &a, cudaStream_t s) {
  const uint32_t grid = (a.total + 127u) / 128u;  // a.total: upper bound when dev_sizes is set
  if (grid == 0) return cudaSuccess;
  proposal_ply_kernel<<<grid, 128, 0, s>>>(a);
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
                                    uint32_t max_plies, Board *out, cudaStream_t s, int policy) {
  const int block = 128;
  const uint32_t grid = (n + block - 1) / block;
  if (policy == 1) random_positions_kernel<1><<<grid, block, 0, s>>>(seed, n, min_plies, max_plies, out);
  else if (policy == 2) random_positions_kernel<2><<<grid, block, 0, s>>>(seed, n, min_plies, max_plies, out);
  else random_positions_kernel<0><<<grid, block, 0, s>>>(seed, n, min_plies, max_plies, out);
  return cudaGetLastError();
}

}  // namespace ga
