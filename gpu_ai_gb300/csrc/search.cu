// search.cu -- many MCTS searches at once, with their trees in device memory.
//
// The reference runs one search per MCTSPlayer on the host and sends each leaf
// batch to the GPU (src/player.cpp:134-150, src/mcts.cpp:63-191).  Here all
// searches' trees live in one node pool in HBM (structure of arrays, one
// contiguous node range per search) and one step advances every active
// search:
//
//   quota_kernel     leaf slots per search this step (min(Q, remaining
//                    budget)), prefix sums, total leaves / playouts
//   select_kernel    a warp per search (a block for steps of 128 leaves or
//                    more): the step's Q leaf slots are split
//                    over the tree level by level the way the reference's
//                    GameTree::select splits a batch (src/mcts.cpp:63-157):
//                    untried children share the slots equally, otherwise in
//                    proportion to UCB1, remainders to the heaviest children;
//                    a leaf given more than one slot is expanded; the lanes
//                    of the warp take one frontier node each
//   playout_kernel   the playout kernel on the leaf boards (sizes and stream
//                    ids read from device memory)
//   backprop_kernel  one thread per leaf: visits and score up the path
//
// Learned searches (a policy/value network attached) add, between the
// playouts and the backpropagation, the network's forward pass on the leaf
// boards (net.cu) and leaf_eval_kernel, which turns a leaf's move logits into
// priors of its moves and its value head into the leaf value.  Their selection
// splits a node's slots by PUCT with virtual visits (split_puct) and expands a
// node once it has been evaluated; backprop blends the network value with the
// playout results.
//
// The launches of a step are replayed as one CUDA graph.  Because each
// search is selected by a single warp in a fixed order and its playouts use
// its own stream ids, a search's tree and result do not depend on which other
// searches share the steps.
//
// Node record (one uint4 per node, read with one load): x = first child (-1
// before expansion), y = number of children | state << 16, z = playouts through
// the node, w = score in half points of the player who moved into the node.
#include "../../include/gpuai.h"
#include "host/state.hpp"
#include "detmath.cuh"
#include "launch.h"
#include "net.h"
#include "rules.cuh"

#include <cuda_fp16.h>

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace ga {
namespace {

constexpr uint32_t kExpanded = 1u, kTerminal = 2u, kEvaluated = 4u;  // node state bits (info.y >> 16)
constexpr int kMaxSelectDepth = 512;
constexpr uint32_t kStatusSelectDepth = 8u;
constexpr int kSelectThreads = 128;   // threads per narrow select block: 4 searches of a warp each
constexpr uint32_t kWideLeaves = 128;  // steps of this many leaves per search or more select with a block per search
// Team size of a step with Q leaves per search: a warp below kWideLeaves,
// else a block of 128, 256 or 512 threads (the largest power of two <= Q).
inline int select_team(uint32_t Q) { return Q < kWideLeaves ? 32 : (Q < 256 ? 128 : (Q < 512 ? 256 : 512)); }
constexpr uint32_t kMaxLeavesPerStep = 512;  // frontier capacity per search (4 KB of shared memory each)
constexpr float kUcbC = 1.41421356f;
constexpr int kMaxChildren = 64;  // moves per position handled by split_slots
constexpr uint32_t kUnits = 64;   // learned searches: visit units per leaf slot (score2 = units * (1 + value))
constexpr uint32_t kPriors = 32;  // stored priors per node (more moves: uniform priors)
constexpr float kFpuReduction = 0.1f;  // unvisited child's Q = parent's Q - this
constexpr float kTerminalLeaf = 2.0f;  // leaf value marking a finished game

struct Pool {  // one entry per node
  uint32_t nodes;  // capacity (bounds checks of the checked build)
  uint4 *info;   // {first child, nchild | state << 16, visits, score2}
  uint4 *board;
  int32_t *parent;
  uint32_t *move, *removed;
  __half *prior;  // learned searches: kPriors per node, the node's moves' priors
};

struct Table {  // one entry per search slot
  int32_t *root, *node_next, *node_end;
  unsigned long long *stream_next, *budget, *done;
  uint32_t *quota_off;  // slots + 1
};

struct Leaves {
  uint4 *board;
  int32_t *node, *search;
  unsigned long long *stream;
  int8_t *out;
  uint32_t *sizes;  // {leaves, playouts}
  float *value;     // learned searches: network value for the side to move at the leaf
};

struct Learned {
  float c_puct;
  float value_weight;
  uint32_t max_leaves;  // leaf slots per search and step at most (bounds checks of the checked build)
};

__device__ __forceinline__ bool board_terminal(const Board &b) {
  if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) return true;
  Side s;
  make_side(b, s);
  return count_moves(s, jumpers(s)) == 0;
}

// Leaf slots per search and their prefix sums (one block).
__global__ void __launch_bounds__(1024) quota_kernel(Table t, uint32_t slots, uint32_t Q, uint32_t ppl, Leaves l) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t carry;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < slots; base += 1024) {
    const uint32_t s = base + tid;
    uint32_t q = 0;
    if (s < slots && t.root[s] >= 0) {
      const unsigned long long b = t.budget[s], d = t.done[s];
      if (d < b) {
        const unsigned long long need = (b - d + ppl - 1) / ppl;
        q = need < Q ? (uint32_t)need : Q;
      }
    }
    uint32_t v = q;
    for (uint32_t o = 1; o < 32; o <<= 1) {
      const uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += n;
    }
    if (lane == 31) warp_sum[warp] = v;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = warp_sum[lane];
      for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t n = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += n;
      }
      warp_sum[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = v - q + (warp ? warp_sum[warp - 1] : 0u);
    if (s < slots) t.quota_off[s] = carry + excl;
    __syncthreads();
    if (tid == 0) carry += warp_sum[31];
    __syncthreads();
  }
  if (tid == 0) {
    t.quota_off[slots] = carry;
    l.sizes[0] = carry;
    l.sizes[1] = carry * ppl;
  }
}

// Number of children node n would get (its legal moves), 0 for none or when
// the game is over (a node's terminal flag is set only for roots; a finished
// game below the root is found here, when it is first to be expanded).
__device__ int child_count(const Pool &p, int32_t n) {
  const uint4 bv = p.board[n];
  const Board b{bv.x, bv.y, bv.z, bv.w};
  if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) return 0;
  Side sd;
  make_side(b, sd);
  const int k = count_moves(sd, jumpers(sd));
  return (k > 0 && k <= kMaxChildren) ? k : 0;
}

// Writes the k children of node n at node indices base.. (called by one lane).
__device__ void expand_at(const Pool &p, int32_t n, int32_t base, int k) {
  const uint4 bv = p.board[n];
  const Board b{bv.x, bv.y, bv.z, bv.w};
  Side sd;
  make_side(b, sd);
  int32_t c = base;
  for_each_move(sd, jumpers(sd), [&](int from, int to, uint32_t removed, int jumps, uint32_t) {
    Board cb = b;
    apply_move(cb, from, to, removed);
    p.board[c] = make_uint4(cb.p1, cb.p2, cb.kings, cb.meta);
    p.parent[c] = n;
    p.info[c] = make_uint4(0xffffffffu, 0u, 0u, 0u);
    p.move[c] = (uint32_t)from | ((uint32_t)to << 8) | ((uint32_t)jumps << 16) |
                ((promotes(b, from, to) ? 1u : 0u) << 24);
    p.removed[c] = removed;
    c++;
    return false;
  });
  const uint4 inf = p.info[n];
  p.info[n] = make_uint4((uint32_t)base, (uint32_t)k | (((inf.y >> 16) | kExpanded) << 16), inf.z, inf.w);
}

// Splits T slots over the children of node n (the reference's rule,
// src/mcts.cpp:95-136): untried children share them equally; otherwise in
// proportion to UCB1 weights rounded down; the remainder goes one each to the
// heaviest children (first on ties).  Weights that sum to zero count as
// equal.  Fills give[0..k) and returns the number of children given slots.
// The weights use the correctly rounded operations of detmath.cuh in a fixed
// order, so the CPU restatement (oracle/search.py) reproduces every split.
__device__ __forceinline__ float ucb_weight(uint4 ci, float lnN) {
  const float mean = dm::div(dm::mul(0.5f, (float)ci.w), (float)ci.z);
  return dm::add(mean, dm::mul(kUcbC, dm::sqrt_(dm::div(lnN, (float)ci.z))));
}

__device__ int split_slots(const Pool &p, int32_t first, int k, uint32_t parent_visits, uint32_t T,
                           uint32_t *give) {
  const float lnN = dm::det_log((float)(parent_visits > 0 ? parent_visits : 1u));
  float wsum = 0.0f;
  int untried = 0;
  for (int c = 0; c < k; c++) {
    const uint4 ci = p.info[first + c];
    if (ci.z == 0) untried++;
    else wsum = dm::add(wsum, ucb_weight(ci, lnN));
  }
  const bool equal = untried == 0 && !(wsum > 0.0f);
  uint32_t assigned = 0;
  float w[kMaxChildren];
  for (int c = 0; c < k; c++) {
    const uint4 ci = p.info[first + c];
    w[c] = ci.z == 0 ? 3.0e38f : (equal ? 1.0f : ucb_weight(ci, lnN));
    if (untried > 0) give[c] = ci.z == 0 ? T / (uint32_t)untried : 0u;
    else give[c] = (uint32_t)dm::mul((float)T, dm::div(w[c], equal ? (float)k : wsum));
    assigned += give[c];
  }
  uint64_t extra = 0;  // children that already took one of the remaining slots
  while (assigned < T) {
    float mw = -1.0f;
    int opt = -1;
    for (int c = 0; c < k; c++)
      if (!((extra >> c) & 1ull) && w[c] > mw) {
        mw = w[c];
        opt = c;
      }
    if (opt < 0) break;  // cannot happen: fewer than k slots remain
    extra |= 1ull << opt;
    give[opt]++;
    assigned++;
  }
  int kids = 0;
  for (int c = 0; c < k; c++) kids += give[c] != 0;
  return kids;
}

// Learned searches: splits T slots over the k children of node n one slot at
// a time, each to the child with the largest Q + c_puct * P * sqrt(N + t + 1)
// / (1 + n + slots already given) (first on ties), where Q is the child's mean
// score for the player to move at n (an unvisited child: n's own Q minus
// kFpuReduction), P its prior (uniform when n has more than kPriors moves or
// has not been evaluated), N = n's visits and n the child's, in leaf slots.
// Fills give[0..k) and returns the number of children given slots.
__device__ int split_puct(const Pool &p, int32_t n, int32_t first, int k, uint32_t parent_visits,
                          uint32_t parent_score2, uint32_t st, uint32_t T, float c_puct, uint32_t *give) {
  float q[kMaxChildren], u[kMaxChildren], pr[kMaxChildren], nv[kMaxChildren];
  const bool priors = (st & kEvaluated) && k <= (int)kPriors;
  const float fpu =
      parent_visits
          ? fmaxf(0.0f, dm::sub(dm::sub(1.0f, dm::div(dm::mul(0.5f, (float)parent_score2), (float)parent_visits)),
                                kFpuReduction))
          : 0.5f;
  const float uniform = dm::div(1.0f, (float)k);
  for (int c = 0; c < k; c++) {
    const uint4 ci = p.info[first + c];
    q[c] = ci.z ? dm::div(dm::mul(0.5f, (float)ci.w), (float)ci.z) : fpu;
    nv[c] = dm::add(1.0f, (float)(ci.z / kUnits));
    pr[c] = dm::mul(c_puct, priors ? __half2float(p.prior[(size_t)n * kPriors + c]) : uniform);
    u[c] = dm::div(pr[c], nv[c]);  // exploration term without the sqrt(N) factor
    give[c] = 0;
  }
  const float N = (float)(parent_visits / kUnits);
  for (uint32_t t = 0; t < T; t++) {
    const float sq = dm::sqrt_(dm::add(dm::add(N, (float)t), 1.0f));
    int best = 0;
    float bs = -3.0e38f;
    for (int c = 0; c < k; c++) {
      const float sc = dm::add(dm::mul(sq, u[c]), q[c]);
      if (sc > bs) {
        bs = sc;
        best = c;
      }
    }
    give[best]++;
    nv[best] = dm::add(nv[best], 1.0f);
    u[best] = dm::div(pr[best], nv[best]);
  }
  int kids = 0;
  for (int c = 0; c < k; c++) kids += give[c] != 0;
  return kids;
}

// A team of TEAM threads per search (a warp, or the whole 128-thread block
// for wide steps).  The frontier holds (node, slots) pairs; each round the
// team takes TEAM frontier entries at a time, expands or splits them, and
// compacts the children it produced into the next frontier and the leaf slots
// it produced into the search's output range, in entry order.
template <bool LEARNED, int TEAM>
__global__ void __launch_bounds__(TEAM == 32 ? kSelectThreads : TEAM)
    select_kernel(Pool p, Table t, Leaves l, uint32_t slots, uint32_t ppl, Learned lrn, uint32_t *status) {
  static_assert(TEAM == 32 || TEAM == 128 || TEAM == 256 || TEAM == 512, "a team is a warp or a whole block");
  constexpr int kTeams = TEAM == 32 ? kSelectThreads / 32 : 1, kWarps = TEAM / 32;
  __shared__ int32_t f_node[kTeams][2][kMaxLeavesPerStep];
  __shared__ uint32_t f_cnt[kTeams][2][kMaxLeavesPerStep];
  __shared__ uint32_t s_scan[kTeams][2][kWarps];
  const uint32_t lane = threadIdx.x & 31u, tl = threadIdx.x % TEAM, wt = tl >> 5, ti = threadIdx.x / TEAM;
  const uint32_t s = blockIdx.x * kTeams + ti;
  if (s >= slots) return;  // uniform over the team
  const int32_t root = t.root[s];
  if (root < 0) return;
  const uint32_t off = t.quota_off[s], q = t.quota_off[s + 1] - off;
  if (q == 0) return;
  auto team_sync = [&]() {
    if (TEAM == 32) __syncwarp();
    else __syncthreads();
  };
  // inclusive prefix sums of a and b over the team's threads, and their totals
  auto scan2 = [&](uint32_t &a, uint32_t &b, uint32_t &ta, uint32_t &tb) {
    for (uint32_t o = 1; o < 32; o <<= 1) {
      const uint32_t x = __shfl_up_sync(0xffffffffu, a, o), y = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += x;
        b += y;
      }
    }
    if (TEAM == 32) {
      ta = __shfl_sync(0xffffffffu, a, 31);
      tb = __shfl_sync(0xffffffffu, b, 31);
      return;
    }
    if (lane == 31) {
      s_scan[ti][0][wt] = a;
      s_scan[ti][1][wt] = b;
    }
    __syncthreads();
    uint32_t pa = 0, pb = 0;
    ta = 0;
    tb = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      const uint32_t va = s_scan[ti][0][w], vb = s_scan[ti][1][w];
      if ((uint32_t)w < wt) {
        pa += va;
        pb += vb;
      }
      ta += va;
      tb += vb;
    }
    a += pa;
    b += pb;
    __syncthreads();  // s_scan is reused by the next scan
  };
  auto team_max = [&](uint32_t x) -> uint32_t {
    x = __reduce_max_sync(0xffffffffu, x);
    if (TEAM == 32) return x;
    if (lane == 0) s_scan[ti][0][wt] = x;
    __syncthreads();
    uint32_t m = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) m = max(m, s_scan[ti][0][w]);
    __syncthreads();
    return m;
  };
  int cur = 0;
  uint32_t nf = 1, emitted = 0;
  int32_t node_next = t.node_next[s];
  const int32_t node_end = t.node_end[s];
  if (tl == 0) {
    f_node[ti][0][0] = root;
    f_cnt[ti][0][0] = q;
  }
  team_sync();
  for (int depth = 0; nf > 0; depth++) {
    if (depth >= kMaxSelectDepth) {
      if (tl == 0) atomicOr(status, kStatusSelectDepth);
      break;
    }
    uint32_t next_n = 0;
    for (uint32_t base = 0; base < nf; base += TEAM) {
      const uint32_t e = base + tl;
      // pass 1: what each thread's entry produces (children entries or leaf slots)
      int32_t n = -1, first = 0, k = 0;
      uint32_t T = 0, leaf = 0, kids = 0, visits = 0, score2 = 0, st = 0;
      int grow = 0;  // children this thread's node gets if it is expanded now
      if (e < nf) {
        n = f_node[ti][cur][e];
        T = f_cnt[ti][cur][e];
        const uint4 inf = p.info[n];
        st = inf.y >> 16;
        visits = inf.z;
        score2 = inf.w;
        first = (int32_t)inf.x;
        k = (int32_t)(inf.y & 0xffffu);
        if (st & kTerminal) leaf = T;
        else if (!(st & kExpanded)) {
          if (LEARNED) {
            // a node is expanded once the network has evaluated it
            if (st & kEvaluated) grow = child_count(p, n);
            if (grow == 0) leaf = T;
          } else {
            if (T == 1) leaf = 1;
            else grow = child_count(p, n);
            if (T > 1 && grow == 0) leaf = T;
          }
        }
      }
      // node indices for this round's expansions, in entry order; an
      // expansion that does not fit the search's node range plays out
      // instead (fitting is a prefix of the entries: the inclusive sums grow)
      uint32_t gx = (uint32_t)grow, unused = 0, gtot = 0, utot = 0;
      scan2(gx, unused, gtot, utot);
      const bool fits = grow > 0 && node_next + (int32_t)gx <= node_end;
      const uint32_t fit_end = team_max(fits ? gx : 0u);
      if (fits && GA_IN_BOUNDS(node_next + (int32_t)gx <= node_end && (uint32_t)node_end <= p.nodes, status)) {
        first = node_next + (int32_t)gx - grow;
        k = grow;
        expand_at(p, n, first, k);
      } else if (grow > 0) {
        leaf = T;
      }
      node_next += (int32_t)fit_end;
      uint32_t give[kMaxChildren];  // this thread's split, written to the next frontier in pass 2
      if (e < nf && !leaf) {
        if (LEARNED)
          kids = (uint32_t)split_puct(p, n, first, k, visits, score2, st, T, lrn.c_puct, give);
        else
          kids = (uint32_t)split_slots(p, first, k, visits, T, give);
      }
      team_sync();
      // team prefix sums of children entries and leaf slots
      uint32_t kx = kids, lx = leaf, ktot = 0, ltot = 0;
      scan2(kx, lx, ktot, ltot);
      const uint32_t kid_at = next_n + kx - kids, leaf_at = emitted + lx - leaf;
      next_n += ktot;
      emitted += ltot;
      // pass 2: write children entries and leaf slots
      if (e < nf) {
        if (leaf) {
          const uint4 bv = p.board[n];
          for (uint32_t r = 0; r < leaf; r++) {
            const uint32_t o = off + leaf_at + r;
            if (!GA_IN_BOUNDS(o < slots * lrn.max_leaves && leaf_at + r < q, status)) break;
            l.board[o] = bv;
            l.node[o] = n;
            l.search[o] = (int32_t)s;
          }
        } else {
          uint32_t w = kid_at;
          for (int c = 0; c < k; c++)
            if (give[c]) {
              if (!GA_IN_BOUNDS(w < kMaxLeavesPerStep && (uint32_t)(first + c) < p.nodes, status)) break;
              f_node[ti][cur ^ 1][w] = first + c;
              f_cnt[ti][cur ^ 1][w] = give[c];
              w++;
            }
        }
      }
      team_sync();
    }
    cur ^= 1;
    nf = next_n;
  }
  if (tl == 0) t.node_next[s] = node_next;
  // per-slot random streams, in slot order
  const unsigned long long sbase = t.stream_next[s];
  for (uint32_t i = tl; i < q; i += TEAM) l.stream[off + i] = sbase + (unsigned long long)i * ppl;
  team_sync();
  if (tl == 0) t.stream_next[s] = sbase + (unsigned long long)q * ppl;
}

// One thread per leaf: outcomes up the path (score in half points for the
// player who made the move into each node).
__global__ void backprop_kernel(Pool p, Table t, Leaves l, uint32_t ppl, uint32_t max_leaves, uint32_t *status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= max_leaves || i >= l.sizes[0]) return;
  const int32_t s = l.search[i];
  const int32_t root = t.root[s];
  uint32_t w1 = 0, w2 = 0, dr = 0;
  for (uint32_t k = 0; k < ppl; k++) {
    const int8_t o = l.out[(size_t)i * ppl + k];
    w1 += o > 0;
    w2 += o < 0;
    dr += o == 0;
  }
  for (int32_t n = l.node[i]; n >= 0; n = p.parent[n]) {
    if (!GA_IN_BOUNDS((uint32_t)n < p.nodes, status)) break;
    const uint32_t mover = (p.board[n].w & 1u) ^ 1u;  // 0: PLAYER_1 moved into n
    atomicAdd(&p.info[n].z, ppl);
    atomicAdd(&p.info[n].w, 2u * (mover == 0 ? w1 : w2) + dr);
  }
  (void)root;
  atomicAdd(&t.done[s], (unsigned long long)ppl);
}

// Learned searches: one thread per leaf; the leaf's result for PLAYER_1 is
// value_weight * network value + (1 - value_weight) * playout mean (terminal
// leaves: the playouts, which end at once with the exact result), added as
// kUnits visits.
__global__ void backprop_learned_kernel(Pool p, Table t, Leaves l, uint32_t ppl, uint32_t max_leaves,
                                        Learned lrn, uint32_t *status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= max_leaves || i >= l.sizes[0]) return;
  const int32_t s = l.search[i];
  const int32_t leaf = l.node[i];
  int sum = 0;  // outcomes for PLAYER_1
  for (uint32_t k = 0; k < ppl; k++) sum += l.out[(size_t)i * ppl + k];
  const float pm = dm::div((float)sum, (float)ppl);
  float x1 = pm;
  const float v = l.value[i];
  if (v <= 1.0f) {  // kTerminalLeaf (> 1): a finished game, whose playouts give the exact result
    const float v1 = (p.board[leaf].w & 1u) ? -v : v;  // the value is for the side to move
    x1 = dm::add(dm::mul(lrn.value_weight, v1), dm::mul(dm::sub(1.0f, lrn.value_weight), pm));
  }
  x1 = fminf(1.0f, fmaxf(-1.0f, x1));
  const uint32_t s1 = (uint32_t)__float2int_rn(dm::mul((float)kUnits, dm::add(1.0f, x1)));  // half points of PLAYER_1
  const uint32_t s2 = 2u * kUnits - s1;
  for (int32_t n = leaf; n >= 0; n = p.parent[n]) {
    if (!GA_IN_BOUNDS((uint32_t)n < p.nodes, status)) break;
    const uint32_t mover = (p.board[n].w & 1u) ^ 1u;  // 0: PLAYER_1 moved into n
    atomicAdd(&p.info[n].z, kUnits);
    atomicAdd(&p.info[n].w, mover == 0 ? s1 : s2);
  }
  atomicAdd(&t.done[s], (unsigned long long)ppl);
}

// Learned searches: one thread per leaf.  The leaf value (tanh of the value
// head, for the side to move; kTerminalLeaf for a finished game) and, the
// first time a node is a leaf, its moves' priors: the softmax of the move
// logits over its legal (from, to) pairs, a pair's probability shared equally
// by the moves that have it.
__global__ void leaf_eval_kernel(Pool p, Leaves l, const __nv_bfloat16 *logits, const float *vraw,
                                 uint32_t max_leaves) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= max_leaves || i >= l.sizes[0]) return;
  const uint4 bv = l.board[i];
  const Board b{bv.x, bv.y, bv.z, bv.w};
  Side sd;
  make_side(b, sd);
  const uint32_t J = jumpers(sd);
  const int k = count_moves(sd, J);
  const bool over = k == 0 || ((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies;
  l.value[i] = over ? kTerminalLeaf : dm::det_tanh(vraw[i]);
  const int32_t n = l.node[i];
  const uint32_t st = p.info[n].y >> 16;
  if (over || (st & (kEvaluated | kTerminal))) return;
  if (k >= 1 && k <= (int)kPriors) {
    uint16_t pair[kPriors] = {};
    uint8_t of[kPriors];
    uint8_t mult[kPriors];
    int np = 0, m = 0;
    for_each_move(sd, J, [&](int from, int to, uint32_t, int, uint32_t) {
      const uint16_t pi = (uint16_t)(from * 32 + to);
      int u = 0;
      while (u < np && pair[u] != pi) u++;
      if (u == np) {
        pair[np] = pi;
        mult[np] = 0;
        np++;
      }
      mult[u]++;
      of[m++] = (uint8_t)u;
      return false;
    });
    const __nv_bfloat16 *lr = logits + (size_t)i * net::kOut;
    float lg[kPriors];
    float lmax = -3.0e38f;
    for (int u = 0; u < np; u++) {
      lg[u] = __bfloat162float(lr[pair[u]]);
      lmax = fmaxf(lmax, lg[u]);
    }
    float sum = 0.0f;
    for (int u = 0; u < np; u++) sum = dm::add(sum, dm::det_exp(dm::sub(lg[u], lmax)));
    for (int j = 0; j < k; j++) {
      const int u = of[j];
      p.prior[(size_t)n * kPriors + j] =
          __float2half_rn(dm::div(dm::div(dm::det_exp(dm::sub(lg[u], lmax)), sum), (float)mult[u]));
    }
  }
  atomicOr(&p.info[n].y, kEvaluated << 16);
}

__global__ void init_search_kernel(Pool p, Table t, int32_t slot, int32_t start, int32_t cap, uint4 board,
                                   unsigned long long budget, unsigned long long stream_base) {
  p.board[start] = board;
  p.parent[start] = -1;
  const Board b{board.x, board.y, board.z, board.w};
  p.info[start] = make_uint4(0xffffffffu, (board_terminal(b) ? kTerminal : 0u) << 16, 0u, 0u);
  p.move[start] = 0;
  p.removed[start] = 0;
  t.root[slot] = start;
  t.node_next[slot] = start + 1;
  t.node_end[slot] = start + cap;
  t.stream_next[slot] = stream_base;
  t.budget[slot] = budget;
  t.done[slot] = 0;
}

__global__ void remove_search_kernel(Table t, int32_t slot) { t.root[slot] = -1; }

}  // namespace
}  // namespace ga

using namespace ga;

struct gpuai_searches {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t slots = 0, pool_nodes = 0, qmax = 0, ppl = 1;
  int32_t policy = 0;
  uint64_t seed = 0;
  int sms = 0, blocks_per_sm = 1;
  Pool pool{};
  Table tab{};
  Leaves leaves{};
  uint32_t *ctl = nullptr;  // counter, status, plies (2 words)
  std::map<uint32_t, uint32_t> free_ranges;  // start -> length
  std::vector<int32_t> start, cap;           // per slot; start -1 = free slot
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_q = 0;
  std::mutex mu;
  std::vector<void *> allocations;
  // learned searches
  gpuai_net *net = nullptr;
  Learned lrn{1.5f, 1.0f, 0u};
  ga::net::Fwd fw;
  cudaStream_t side = nullptr;  // the network's branch of a learned step
  cudaEvent_t fork = nullptr, join = nullptr;
  // learned-proposal playouts: the first `guided` plies of each playout are
  // drawn from the network's policy
  uint32_t guided = 0;
  float inv_temperature = 1.0f;
  ga::net::Fwd pfw;               // forward on the playouts' boards (later guided plies)
  ga::Board *pcur = nullptr;      // each playout's board
  unsigned long long *pstream = nullptr;  // each playout's stream id
  uint32_t *psizes = nullptr;     // {playouts, playouts}
};

namespace {

int err(int code, const std::string &m) { return ga::record_error(code, m.c_str()); }
int cuda_err(cudaError_t e, const char *what) {
  return err(e == cudaErrorMemoryAllocation ? GPUAI_ERR_OOM : GPUAI_ERR_CUDA,
             std::string("searches: ") + what + ": " + cudaGetErrorString(e));
}

#define SCK(call, what)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_err(e_, what);     \
  } while (0)

template <class T>
cudaError_t dalloc(gpuai_searches *s, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T) + 16);
  if (e == cudaSuccess) {
    s->allocations.push_back(q);
    *p = static_cast<T *>(q);
  }
  return e;
}

int enqueue_step(gpuai_searches *s, uint32_t q) {
  const cudaStream_t st = s->stream;
  // work counter and ply count restart every step; status bits accumulate
  // until poll reads them
  SCK(cudaMemsetAsync(s->ctl, 0, sizeof(uint32_t), st), "reset work counter");
  quota_kernel<<<1, 1024, 0, st>>>(s->tab, s->slots, q, s->ppl, s->leaves);
  // narrow steps: a warp per search, four per block; wide steps (>= 128
  // leaves per search): a block of 128-512 threads per search, as many
  // frontier entries per round
  const int team = select_team(q);
  const uint32_t per_block = team == 32 ? (uint32_t)(kSelectThreads / 32) : 1u;
  const uint32_t sel_blocks = (s->slots + per_block - 1) / per_block;
  const int threads = team == 32 ? kSelectThreads : team;
  auto sel = [&](auto kernel) {
    kernel<<<sel_blocks, threads, 0, st>>>(s->pool, s->tab, s->leaves, s->slots, s->ppl, s->lrn, s->ctl + 1);
  };
  if (s->net) {
    switch (team) {
      case 32: sel(select_kernel<true, 32>); break;
      case 128: sel(select_kernel<true, 128>); break;
      case 256: sel(select_kernel<true, 256>); break;
      default: sel(select_kernel<true, 512>); break;
    }
  } else {
    switch (team) {
      case 32: sel(select_kernel<false, 32>); break;
      case 128: sel(select_kernel<false, 128>); break;
      case 256: sel(select_kernel<false, 256>); break;
      default: sel(select_kernel<false, 512>); break;
    }
  }
  PlayoutArgs a;
  a.pos = reinterpret_cast<const Board *>(s->leaves.board);
  a.offsets = nullptr;
  a.npos = 0;
  a.uniform_reps = s->ppl;
  a.total = 0;
  a.seed = s->seed;
  a.stream_base = 0;
  a.out = s->leaves.out;
  a.counter = s->ctl;
  a.status = s->ctl + 1;
  a.plies = nullptr;
  a.pos_stream = reinterpret_cast<const uint64_t *>(s->leaves.stream);
  a.dev_sizes = s->leaves.sizes;
  const uint32_t max_leaves = s->slots * s->qmax;
  if (s->net && s->guided > 0) {
    // learned-proposal step: the network's forward on the leaves gives the
    // priors, the leaf values and the first guided ply of every playout;
    // later guided plies run the network on the playouts' boards; then the
    // uniformly random rest of each game
    SCK(ga::net::forward(s->net, s->fw, reinterpret_cast<const gpuai_board *>(s->leaves.board), 0, s->leaves.sizes,
                         s->ctl + 1, st),
        "network forward on the leaves");
    leaf_eval_kernel<<<(max_leaves + 255) / 256, 256, 0, st>>>(s->pool, s->leaves, s->fw.logits_b, s->fw.vraw,
                                                               max_leaves);
    SCK(cudaGetLastError(), "leaf evaluation launch");
    ProposalArgs pa{};
    pa.in = reinterpret_cast<const Board *>(s->leaves.board);
    pa.uniform_reps = s->ppl;
    pa.total = max_leaves * s->ppl;  // grid bound; the sizes come from device memory
    pa.dev_sizes = s->leaves.sizes;
    pa.per_position = true;
    pa.logits = reinterpret_cast<const uint16_t *>(s->fw.logits_b);
    pa.seed = s->seed;
    pa.pos_stream = reinterpret_cast<const uint64_t *>(s->leaves.stream);
    pa.inv_temperature = s->inv_temperature;
    pa.out = s->pcur;
    pa.out_stream = reinterpret_cast<uint64_t *>(s->pstream);
    pa.out_sizes = s->psizes;
    for (uint32_t g = 0; g < s->guided; g++) {
      if (g > 0) {
        SCK(ga::net::forward(s->net, s->pfw, reinterpret_cast<const gpuai_board *>(s->pcur), 0, s->psizes,
                             s->ctl + 1, st),
            "network forward on the playouts");
        pa.in = s->pcur;
        pa.per_position = false;
        pa.dev_sizes = s->psizes;
        pa.logits = reinterpret_cast<const uint16_t *>(s->pfw.logits_b);
        pa.pos_stream = nullptr;
        pa.play_stream = reinterpret_cast<const uint64_t *>(s->pstream);
        pa.out_stream = nullptr;
        pa.out_sizes = nullptr;
      }
      pa.ply = g;
      SCK(ga::launch_proposal_ply(pa, st), "guided ply launch");
    }
    PlayoutArgs b = a;
    b.pos = s->pcur;
    b.uniform_reps = 1;
    b.pos_stream = reinterpret_cast<const uint64_t *>(s->pstream);
    b.dev_sizes = s->psizes;
    SCK(launch_playouts(b, s->policy, kPlayoutBlock, s->sms * s->blocks_per_sm, st), "playout kernel launch");
    backprop_learned_kernel<<<(max_leaves + 255) / 256, 256, 0, st>>>(s->pool, s->tab, s->leaves, s->ppl,
                                                                      max_leaves, s->lrn, s->ctl + 1);
    SCK(cudaGetLastError(), "search kernel launch");
    return GPUAI_OK;
  }
  if (s->net) {
    // the network's forward pass and the leaf evaluation do not depend on the
    // playouts: they run on a second stream and fill the SMs that the playout
    // kernel's last games leave idle; backprop waits for both
    SCK(cudaEventRecord(s->fork, st), "fork");
    SCK(cudaStreamWaitEvent(s->side, s->fork, 0), "fork");
    SCK(ga::net::forward(s->net, s->fw, reinterpret_cast<const gpuai_board *>(s->leaves.board), 0, s->leaves.sizes,
                         s->ctl + 1, s->side),
        "network forward on the leaves");
    leaf_eval_kernel<<<(max_leaves + 255) / 256, 256, 0, s->side>>>(s->pool, s->leaves, s->fw.logits_b,
                                                                    s->fw.vraw, max_leaves);
    SCK(cudaGetLastError(), "leaf evaluation launch");
    SCK(cudaEventRecord(s->join, s->side), "join");
  }
  SCK(launch_playouts(a, s->policy, kPlayoutBlock, s->sms * s->blocks_per_sm, st), "playout kernel launch");
  if (s->net) {
    SCK(cudaStreamWaitEvent(st, s->join, 0), "join");
    backprop_learned_kernel<<<(max_leaves + 255) / 256, 256, 0, st>>>(s->pool, s->tab, s->leaves, s->ppl,
                                                                      max_leaves, s->lrn, s->ctl + 1);
  } else {
    backprop_kernel<<<(max_leaves + 255) / 256, 256, 0, st>>>(s->pool, s->tab, s->leaves, s->ppl, max_leaves,
                                                              s->ctl + 1);
  }
  SCK(cudaGetLastError(), "search kernel launch");
  return GPUAI_OK;
}

}  // namespace

extern "C" {

int gpuai_searches_create(int device, uint32_t max_searches, uint32_t pool_nodes, uint32_t max_leaves_per_step,
                          uint32_t playouts_per_leaf, int32_t policy, uint64_t seed, gpuai_searches **out) {
  if (!out) return err(GPUAI_ERR_INVALID, "gpuai_searches_create: out is NULL");
  *out = nullptr;
  if (max_searches == 0 || pool_nodes == 0 || max_leaves_per_step == 0 || playouts_per_leaf == 0)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_create: zero size");
  if (policy < 0 || policy > 2) return err(GPUAI_ERR_INVALID, "gpuai_searches_create: unknown policy");
  if (max_leaves_per_step > kMaxLeavesPerStep)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_create: max_leaves_per_step above 512");
  if ((uint64_t)max_searches * max_leaves_per_step * playouts_per_leaf > 0x7fffffffull || pool_nodes > 0x7fffffffu)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_create: sizes exceed 2^31");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    return err(GPUAI_ERR_NO_DEVICE, "gpuai_searches_create: no such CUDA device");
  gpuai_searches *s = new gpuai_searches;
  s->device = device;
  s->slots = max_searches;
  s->pool_nodes = pool_nodes;
  s->qmax = max_leaves_per_step;
  s->ppl = playouts_per_leaf;
  s->policy = policy;
  s->seed = seed;
  s->pool.nodes = pool_nodes;
  s->lrn.max_leaves = max_leaves_per_step;
  auto fail = [&](int rc) {
    gpuai_searches_destroy(s);
    return rc;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(err(GPUAI_ERR_CUDA, "cudaSetDevice failed"));
  cudaError_t e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = playout_occupancy(policy, kPlayoutBlock, &s->blocks_per_sm);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  const size_t P = pool_nodes, S = max_searches, L = (size_t)max_searches * max_leaves_per_step;
  if (e == cudaSuccess) e = dalloc(s, &s->pool.info, P);
  if (e == cudaSuccess) e = dalloc(s, &s->pool.board, P);
  if (e == cudaSuccess) e = dalloc(s, &s->pool.parent, P);
  if (e == cudaSuccess) e = dalloc(s, &s->pool.move, P);
  if (e == cudaSuccess) e = dalloc(s, &s->pool.removed, P);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.root, S);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.node_next, S);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.node_end, S);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.stream_next, S);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.budget, S);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.done, S);
  if (e == cudaSuccess) e = dalloc(s, &s->tab.quota_off, S + 1);
  if (e == cudaSuccess) e = dalloc(s, &s->leaves.board, L);
  if (e == cudaSuccess) e = dalloc(s, &s->leaves.node, L);
  if (e == cudaSuccess) e = dalloc(s, &s->leaves.search, L);
  if (e == cudaSuccess) e = dalloc(s, &s->leaves.stream, L);
  if (e == cudaSuccess) e = dalloc(s, &s->leaves.out, L * playouts_per_leaf);
  if (e == cudaSuccess) e = dalloc(s, &s->leaves.sizes, 2);
  if (e == cudaSuccess) e = dalloc(s, &s->ctl, 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->tab.root, 0xff, S * sizeof(int32_t), s->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->leaves.sizes, 0, 2 * sizeof(uint32_t), s->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->ctl, 0, 4 * sizeof(uint32_t), s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return fail(cuda_err(e, "gpuai_searches_create"));
  s->free_ranges[0] = pool_nodes;
  s->start.assign(S, -1);
  s->cap.assign(S, 0);
  *out = s;
  return GPUAI_OK;
}

void gpuai_searches_destroy(gpuai_searches *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->side) cudaStreamSynchronize(s->side);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  for (void *p : s->allocations) cudaFree(p);
  if (s->fork) cudaEventDestroy(s->fork);
  if (s->join) cudaEventDestroy(s->join);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

int gpuai_searches_add(gpuai_searches *s, const gpuai_board *root, uint64_t playout_budget, uint32_t node_capacity,
                       uint64_t stream_base, int32_t *slot) {
  if (!s || !root || !slot) return err(GPUAI_ERR_INVALID, "gpuai_searches_add: NULL argument");
  if (node_capacity < 1) return err(GPUAI_ERR_INVALID, "gpuai_searches_add: node_capacity must be >= 1");
  if ((root->p1 & root->p2) || (root->kings & ~(root->p1 | root->p2)) || (root->meta & ~0xff01u))
    return err(GPUAI_ERR_INVALID, "gpuai_searches_add: malformed board");
  std::lock_guard<std::mutex> lock(s->mu);
  int32_t free_slot = -1;
  for (uint32_t i = 0; i < s->slots; i++)
    if (s->start[i] < 0) {
      free_slot = (int32_t)i;
      break;
    }
  if (free_slot < 0) return err(GPUAI_ERR_OOM, "gpuai_searches_add: admission refused: all search slots busy");
  auto it = s->free_ranges.begin();
  for (; it != s->free_ranges.end(); ++it)
    if (it->second >= node_capacity) break;
  if (it == s->free_ranges.end())
    return err(GPUAI_ERR_OOM, "gpuai_searches_add: admission refused: no free node range of that size");
  const uint32_t start = it->first, len = it->second;
  s->free_ranges.erase(it);
  if (len > node_capacity) s->free_ranges[start + node_capacity] = len - node_capacity;
  s->start[free_slot] = (int32_t)start;
  s->cap[free_slot] = (int32_t)node_capacity;
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  init_search_kernel<<<1, 1, 0, s->stream>>>(s->pool, s->tab, free_slot, (int32_t)start, (int32_t)node_capacity,
                                              make_uint4(root->p1, root->p2, root->kings, root->meta),
                                              playout_budget, stream_base);
  SCK(cudaGetLastError(), "init_search_kernel");
  *slot = free_slot;
  return GPUAI_OK;
}

int gpuai_searches_remove(gpuai_searches *s, int32_t slot) {
  if (!s) return err(GPUAI_ERR_INVALID, "gpuai_searches_remove: NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  if (slot < 0 || (uint32_t)slot >= s->slots || s->start[slot] < 0)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_remove: no such search");
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  remove_search_kernel<<<1, 1, 0, s->stream>>>(s->tab, slot);
  SCK(cudaGetLastError(), "remove_search_kernel");
  // return the node range, merging with free neighbours
  uint32_t start = (uint32_t)s->start[slot], len = (uint32_t)s->cap[slot];
  auto next = s->free_ranges.lower_bound(start);
  if (next != s->free_ranges.end() && next->first == start + len) {
    len += next->second;
    next = s->free_ranges.erase(next);
  }
  if (next != s->free_ranges.begin()) {
    auto prev = std::prev(next);
    if (prev->first + prev->second == start) {
      start = prev->first;
      len += prev->second;
      s->free_ranges.erase(prev);
    }
  }
  s->free_ranges[start] = len;
  s->start[slot] = -1;
  s->cap[slot] = 0;
  return GPUAI_OK;
}

int gpuai_searches_step(gpuai_searches *s, uint32_t steps, uint32_t leaves_per_search, int32_t use_graph) {
  GPUAI_RANGE("gpuai_searches_step");
  if (!s) return err(GPUAI_ERR_INVALID, "gpuai_searches_step: NULL");
  if (leaves_per_search == 0 || leaves_per_search > s->qmax)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_step: leaves_per_search outside 1..max_leaves_per_step");
  std::lock_guard<std::mutex> lock(s->mu);
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  if (!use_graph) {
    for (uint32_t k = 0; k < steps; k++) {
      const int rc = enqueue_step(s, leaves_per_search);
      if (rc) return rc;
    }
    return GPUAI_OK;
  }
  if (!s->graph || s->graph_q != leaves_per_search) {
    if (s->graph) cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
    cudaGraph_t g = nullptr;
    SCK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const int rc = enqueue_step(s, leaves_per_search);
    const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    SCK(e, "end capture");
    const cudaError_t ei = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    SCK(ei, "graph instantiate");
    s->graph_q = leaves_per_search;
  }
  for (uint32_t k = 0; k < steps; k++) SCK(cudaGraphLaunch(s->graph, s->stream), "graph launch");
  return GPUAI_OK;
}

int gpuai_searches_poll(gpuai_searches *s, uint64_t *done, uint64_t *budget, uint32_t n, uint32_t *status) {
  GPUAI_RANGE("gpuai_searches_poll");
  if (!s || !done || !budget) return err(GPUAI_ERR_INVALID, "gpuai_searches_poll: NULL");
  if (n > s->slots) return err(GPUAI_ERR_INVALID, "gpuai_searches_poll: n exceeds max_searches");
  std::lock_guard<std::mutex> lock(s->mu);
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  uint32_t st = 0;
  SCK(cudaMemcpyAsync(done, s->tab.done, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s->stream), "poll");
  SCK(cudaMemcpyAsync(budget, s->tab.budget, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s->stream), "poll");
  SCK(cudaMemcpyAsync(&st, s->ctl + 1, sizeof st, cudaMemcpyDeviceToHost, s->stream), "poll");
  SCK(cudaStreamSynchronize(s->stream), "search steps");
  if (st) SCK(cudaMemsetAsync(s->ctl + 1, 0, sizeof(uint32_t), s->stream), "clear status");  // reported once
  for (uint32_t i = 0; i < n; i++)
    if (s->start[i] < 0) done[i] = budget[i] = 0;
  if (status) *status = st;
  if (st) return err(GPUAI_ERR_LIMIT, "gpuai_searches_poll: a kernel reported a limit");
  return GPUAI_OK;
}

int gpuai_searches_set_net(gpuai_searches *s, gpuai_net *net, float value_weight, float c_puct) {
  if (!s) return err(GPUAI_ERR_INVALID, "gpuai_searches_set_net: NULL");
  if (!(value_weight >= 0.0f && value_weight <= 1.0f) || !(c_puct > 0.0f && c_puct < 1.0e6f))
    return err(GPUAI_ERR_INVALID, "gpuai_searches_set_net: value_weight must be in [0, 1] and c_puct > 0");
  std::lock_guard<std::mutex> lock(s->mu);
  for (uint32_t i = 0; i < s->slots; i++)
    if (s->start[i] >= 0) return err(GPUAI_ERR_INVALID, "gpuai_searches_set_net: searches are admitted");
  if (net && ga::net::device_of(net) != s->device)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_set_net: network and searches are on different devices");
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  if (net && !s->pool.prior) {
    const size_t L = (size_t)s->slots * s->qmax;
    SCK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "network stream");
    SCK(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming), "event");
    SCK(cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming), "event");
    SCK(dalloc(s, &s->pool.prior, (size_t)s->pool_nodes * kPriors), "prior pool");
    SCK(dalloc(s, &s->leaves.value, L), "leaf values");
    SCK(ga::net::fwd_alloc(s->fw, (uint32_t)L, s->allocations, true), "network workspace");
  }
  s->net = net;
  s->lrn.c_puct = c_puct;
  s->lrn.value_weight = value_weight;
  if (s->graph) cudaGraphExecDestroy(s->graph);  // the step's launches change
  s->graph = nullptr;
  return GPUAI_OK;
}

int gpuai_searches_set_proposal(gpuai_searches *s, uint32_t guided_plies, float temperature) {
  if (!s) return err(GPUAI_ERR_INVALID, "gpuai_searches_set_proposal: NULL");
  if (guided_plies > ga::net::kMaxGuidedPlies)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_set_proposal: guided_plies above 32");
  if (!(temperature > 0.0f && temperature < 1.0e6f))
    return err(GPUAI_ERR_INVALID, "gpuai_searches_set_proposal: temperature must be positive");
  std::lock_guard<std::mutex> lock(s->mu);
  if (guided_plies > 0 && !s->net)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_set_proposal: attach a network first (gpuai_searches_set_net)");
  for (uint32_t i = 0; i < s->slots; i++)
    if (s->start[i] >= 0) return err(GPUAI_ERR_INVALID, "gpuai_searches_set_proposal: searches are admitted");
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  const size_t P = (size_t)s->slots * s->qmax * s->ppl;
  if (guided_plies > 0 && !s->pcur) {
    SCK(dalloc(s, &s->pcur, P), "proposal boards");
    SCK(dalloc(s, &s->pstream, P), "proposal streams");
    SCK(dalloc(s, &s->psizes, 2), "proposal sizes");
  }
  if (guided_plies > 1 && !s->pfw.rows) SCK(ga::net::fwd_alloc(s->pfw, (uint32_t)P, s->allocations, true), "network workspace");
  s->guided = guided_plies;
  s->inv_temperature = 1.0f / temperature;
  if (s->graph) cudaGraphExecDestroy(s->graph);  // the step's launches change
  s->graph = nullptr;
  return GPUAI_OK;
}

int gpuai_searches_children(gpuai_searches *s, int32_t slot, gpuai_move *moves, uint32_t *visits,
                            uint32_t *score2, uint32_t max_children, uint32_t *nchildren, uint32_t *nodes_used) {
  if (!s || !nchildren) return err(GPUAI_ERR_INVALID, "gpuai_searches_children: NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  if (slot < 0 || (uint32_t)slot >= s->slots || s->start[slot] < 0)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_children: no such search");
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  const int32_t r = s->start[slot];
  int32_t next = 0;
  uint4 rb, ri;
  SCK(cudaMemcpyAsync(&ri, s->pool.info + r, 16, cudaMemcpyDeviceToHost, s->stream), "children");
  SCK(cudaMemcpyAsync(&rb, s->pool.board + r, 16, cudaMemcpyDeviceToHost, s->stream), "children");
  SCK(cudaMemcpyAsync(&next, s->tab.node_next + slot, 4, cudaMemcpyDeviceToHost, s->stream), "children");
  SCK(cudaStreamSynchronize(s->stream), "children");
  if (nodes_used) *nodes_used = (uint32_t)(next - r);
  const int32_t k = ((ri.y >> 16) & kExpanded) ? (int32_t)(ri.y & 0xffffu) : 0;
  const int32_t first = (int32_t)ri.x;
  *nchildren = (uint32_t)k;
  if (k <= 0) return GPUAI_OK;
  std::vector<uint4> ci(k);
  SCK(cudaMemcpyAsync(ci.data(), s->pool.info + first, 16 * k, cudaMemcpyDeviceToHost, s->stream), "children");
  SCK(cudaStreamSynchronize(s->stream), "children");
  std::vector<uint32_t> v(k), sc(k);
  for (int32_t i = 0; i < k; i++) {
    v[i] = ci[i].z;
    sc[i] = ci[i].w;
  }
  // full move records from the root's move list (same order as the children)
  gpuai::State root_state;
  root_state.b = gpuai_board{rb.x, rb.y, rb.z, rb.w};
  const std::vector<gpuai::Move> all_moves = root_state.getMoves();
  std::vector<gpuai_move> all;
  for (const gpuai::Move &m : all_moves) all.push_back(m.m);
  for (uint32_t i = 0; i < (uint32_t)k && i < max_children; i++) {
    if (visits) visits[i] = v[i];
    if (score2) score2[i] = sc[i];
    if (moves && i < all.size()) moves[i] = all[i];
  }
  return GPUAI_OK;
}

int gpuai_searches_nodes(gpuai_searches *s, int32_t slot, uint32_t max_nodes, uint32_t *info, gpuai_board *boards,
                         int32_t *parent, uint16_t *priors, uint32_t *nnodes) {
  if (!s || !nnodes) return err(GPUAI_ERR_INVALID, "gpuai_searches_nodes: NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  if (slot < 0 || (uint32_t)slot >= s->slots || s->start[slot] < 0)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_nodes: no such search");
  if (priors && !s->pool.prior) return err(GPUAI_ERR_INVALID, "gpuai_searches_nodes: the searches keep no priors");
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  const int32_t r = s->start[slot];
  int32_t next = 0;
  SCK(cudaMemcpyAsync(&next, s->tab.node_next + slot, 4, cudaMemcpyDeviceToHost, s->stream), "nodes");
  SCK(cudaStreamSynchronize(s->stream), "nodes");
  const uint32_t used = (uint32_t)(next - r);
  *nnodes = used;
  const uint32_t n = used < max_nodes ? used : max_nodes;
  if (n == 0) return GPUAI_OK;
  std::vector<uint4> inf(n);
  std::vector<int32_t> par(n);
  SCK(cudaMemcpyAsync(inf.data(), s->pool.info + r, 16 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "nodes");
  SCK(cudaMemcpyAsync(par.data(), s->pool.parent + r, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "nodes");
  if (boards)
    SCK(cudaMemcpyAsync(boards, s->pool.board + r, 16 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "nodes");
  if (priors)
    SCK(cudaMemcpyAsync(priors, s->pool.prior + (size_t)r * kPriors, 2 * kPriors * (size_t)n,
                        cudaMemcpyDeviceToHost, s->stream),
        "nodes");
  SCK(cudaStreamSynchronize(s->stream), "nodes");
  for (uint32_t i = 0; i < n; i++) {
    if (info) {
      info[4 * i] = inf[i].x == 0xffffffffu ? 0xffffffffu : inf[i].x - (uint32_t)r;
      info[4 * i + 1] = inf[i].y;
      info[4 * i + 2] = inf[i].z;
      info[4 * i + 3] = inf[i].w;
    }
    if (parent) parent[i] = par[i] < 0 ? -1 : par[i] - r;
  }
  return GPUAI_OK;
}

int gpuai_searches_leaves(gpuai_searches *s, uint32_t max_leaves, uint32_t *nleaves, int32_t *search, int32_t *node,
                          gpuai_board *boards, uint64_t *streams, int8_t *outcomes, float *net_value,
                          uint16_t *net_logits) {
  if (!s || !nleaves) return err(GPUAI_ERR_INVALID, "gpuai_searches_leaves: NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  if ((net_value || net_logits) && !s->net)
    return err(GPUAI_ERR_INVALID, "gpuai_searches_leaves: no network is attached");
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  uint32_t sizes[2] = {0, 0};
  SCK(cudaMemcpyAsync(sizes, s->leaves.sizes, 8, cudaMemcpyDeviceToHost, s->stream), "leaves");
  SCK(cudaStreamSynchronize(s->stream), "leaves");
  *nleaves = sizes[0];
  const uint32_t n = sizes[0] < max_leaves ? sizes[0] : max_leaves;
  if (n == 0) return GPUAI_OK;
  std::vector<int32_t> srch(n), nd(n);
  SCK(cudaMemcpyAsync(srch.data(), s->leaves.search, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "leaves");
  SCK(cudaMemcpyAsync(nd.data(), s->leaves.node, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "leaves");
  if (boards)
    SCK(cudaMemcpyAsync(boards, s->leaves.board, 16 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "leaves");
  if (streams)
    SCK(cudaMemcpyAsync(streams, s->leaves.stream, 8 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "leaves");
  if (outcomes)
    SCK(cudaMemcpyAsync(outcomes, s->leaves.out, (size_t)n * s->ppl, cudaMemcpyDeviceToHost, s->stream), "leaves");
  if (net_value)
    SCK(cudaMemcpyAsync(net_value, s->fw.vraw, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream), "leaves");
  if (net_logits)
    SCK(cudaMemcpyAsync(net_logits, s->fw.logits_b, 2 * (size_t)n * ga::net::kOut, cudaMemcpyDeviceToHost,
                        s->stream),
        "leaves");
  SCK(cudaStreamSynchronize(s->stream), "leaves");
  for (uint32_t i = 0; i < n; i++) {
    if (search) search[i] = srch[i];
    const int32_t st = (srch[i] >= 0 && (uint32_t)srch[i] < s->slots) ? s->start[srch[i]] : -1;
    if (node) node[i] = st < 0 ? -1 : nd[i] - st;
  }
  return GPUAI_OK;
}

}  // extern "C"
