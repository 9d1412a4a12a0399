// rules.cuh -- 8x8 checkers rules on 32-bit bitboards, for device and host.
//
// Square s = row*4 + col/2 over the 32 dark squares (row 0 holds PLAYER_1's
// back rank; dark squares are col = 1-(row%2), +2, ...), the same numbering
// as the reference's thread-to-square map (src/state.cu:185-188).
//
// The move list order is the reference's State::genMoves order
// (src/state.cu:171-180, 239-245, 255-340, 388-420):
//   * captures are forced; all capture sequences of all squares come first,
//     squares ascending, each square's maximal sequences in depth-first order:
//     men try dc=-1 then dc=+1 (forward only), kings try
//     (+1,+1),(+1,-1),(-1,+1),(-1,-1);
//   * a sequence is listed only when it cannot be extended; captured pieces
//     stay on the board while the sequence is searched, and a king never lands
//     twice on one square (src/state.cu:134-139);
//   * otherwise direct moves, squares ascending, directions (+1,+1),(+1,-1),
//     (-1,+1),(-1,-1) restricted to the forward pair for men.
// A man that ends a move on the far row is promoted (src/state.cu:276,315-320).
//
// Directions: D0 = (+1,+1), D1 = (+1,-1), D2 = (-1,+1), D3 = (-1,-1) as
// (d_row, d_col).  PLAYER_1 men move along D0/D1, PLAYER_2 men along D2/D3.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define GA_HD __host__ __device__ __forceinline__
#else
#define GA_HD inline
#endif

namespace ga {

constexpr int kDrawPlies = 50;      // NUM_DRAW_MOVES (src/state.hpp:14)
constexpr int kMaxDepth = 15;       // capture sequences longer than this are reported
constexpr uint32_t kRow7 = 0xF0000000u;
constexpr uint32_t kRow0 = 0x0000000Fu;

struct Board {
  uint32_t p1, p2, kings, meta;  // meta: bit 0 side to move, bits 8..15 plies since capture
};

GA_HD int popc(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __popc(x);
#else
  return __builtin_popcount(x);
#endif
}

GA_HD int ctz(uint32_t x) {  // x != 0
#if defined(__CUDA_ARCH__)
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}

// One diagonal step of every square of b in direction D; squares leaving the
// board vanish.  Even rows (bits 0-3, 8-11, ...) and odd rows shift by
// different amounts because of the 4-squares-per-row packing.
template <int D>
GA_HD uint32_t step(uint32_t b) {
  if (D == 0) return ((b & 0x07070707u) << 5) | ((b & 0xF0F0F0F0u) << 4);
  if (D == 1) return ((b & 0x0F0F0F0Fu) << 4) | ((b & 0xE0E0E0E0u) << 3);
  if (D == 2) return ((b & 0x07070707u) >> 3) | ((b & 0xF0F0F0F0u) >> 4);
  return ((b & 0x0F0F0F0Fu) >> 4) | ((b & 0xE0E0E0E0u) >> 5);
}

// Square offset of a jump (two steps) in direction d: +9, +7, -7, -9.
GA_HD int jump_off(int d) { return d == 0 ? 9 : (d == 1 ? 7 : (d == 2 ? -7 : -9)); }

// Square offset of a single step from square s in direction d.
GA_HD int step_off(int s, int d) {
  int even = ((s >> 2) & 1) ^ 1;  // row parity of s
  int base = d == 0 ? 4 : (d == 1 ? 3 : (d == 2 ? -4 : -5));
  return base + even;
}

// Square jumped over when moving from a to b = a + jump_off(d).
GA_HD int mid_square(int a, int b) {
  int even = ((a >> 2) & 1) ^ 1;
  return (a + b + (even ? 1 : -1)) >> 1;
}

// Per-ply view of a position from the side to move.
struct Side {
  uint32_t own, opp, ownK, empty;
  int turn;      // 0 = PLAYER_1 to move
  uint32_t jd[4];  // squares from which a jump in direction d is possible
};

GA_HD void make_side(const Board &b, Side &s) {
  s.turn = (int)(b.meta & 1u);
  s.own = s.turn ? b.p2 : b.p1;
  s.opp = s.turn ? b.p1 : b.p2;
  s.ownK = s.own & b.kings;
  s.empty = ~(b.p1 | b.p2);
  // jd[d] = {s : s+d is an opponent, s+2d is empty}; step<3-d> is the inverse of step<d>.
  s.jd[0] = step<3>(s.opp) & step<3>(step<3>(s.empty));
  s.jd[1] = step<2>(s.opp) & step<2>(step<2>(s.empty));
  s.jd[2] = step<1>(s.opp) & step<1>(step<1>(s.empty));
  s.jd[3] = step<0>(s.opp) & step<0>(step<0>(s.empty));
}

// Pieces of the side to move that have at least one capture.
GA_HD uint32_t jumpers(const Side &s) {
  uint32_t men = s.own & ~s.ownK;
  uint32_t fwd = s.turn ? (s.jd[2] | s.jd[3]) : (s.jd[0] | s.jd[1]);
  return (men & fwd) | (s.ownK & (s.jd[0] | s.jd[1] | s.jd[2] | s.jd[3]));
}

// Direct-move source masks md[d] (squares that can step in direction d).
GA_HD void direct_masks(const Side &s, uint32_t md[4]) {
  uint32_t m0 = s.turn ? s.ownK : s.own;  // D0/D1 movers: P1 men and all kings
  uint32_t m2 = s.turn ? s.own : s.ownK;  // D2/D3 movers: P2 men and all kings
  md[0] = m0 & step<3>(s.empty);
  md[1] = m0 & step<2>(s.empty);
  md[2] = m2 & step<1>(s.empty);
  md[3] = m2 & step<0>(s.empty);
}

// Ordered set of capture directions available at square t.  Bit j is the
// j-th direction in the piece's search order: kings D0,D1,D2,D3; PLAYER_1 men
// D1,D0; PLAYER_2 men D3,D2.  `visited` holds landing squares already used by
// the sequence (the cycle check of src/state.cu:134-139).
GA_HD uint32_t capture_dirs(const Side &s, int t, bool king, uint32_t visited) {
  uint32_t v[4];
#pragma unroll
  for (int d = 0; d < 4; d++) {
    uint32_t can = (s.jd[d] >> t) & 1u;
    uint32_t land = (uint32_t)(t + jump_off(d)) & 31u;
    v[d] = can & ~(visited >> land) & 1u;
  }
  if (king) return v[0] | (v[1] << 1) | (v[2] << 2) | (v[3] << 3);
  return s.turn ? (v[3] | (v[2] << 1)) : (v[1] | (v[0] << 1));
}

GA_HD int dir_of(int j, bool king, int turn) { return king ? j : (turn ? 3 - j : 1 - j); }

// Depth-first walk of the maximal capture sequences of the piece on square o,
// in reference order.  Calls leaf(to, removed, depth, dirs) for each sequence
// (dirs: 2 bits per jump, first jump in the low bits); the walk stops early
// when leaf returns true.  Returns the number of sequences visited, or -1 if a
// sequence would exceed kMaxDepth jumps.
template <class Leaf>
GA_HD int capture_walk(const Side &s, int o, Leaf &&leaf) {
  const bool king = (s.ownK >> o) & 1u;
  int t = o, depth = 0, leaves = 0;
  uint32_t visited = 0, removed = 0, dirs = 0;
  uint64_t rem_stack = 0;
  uint32_t rem = capture_dirs(s, t, king, visited);
  if (rem == 0) return 0;
  for (;;) {
    if (rem) {
      int j = ctz(rem);
      rem &= rem - 1;
      int d = dir_of(j, king, s.turn);
      if (depth >= kMaxDepth) return -1;
      rem_stack |= (uint64_t)rem << (4 * depth);
      dirs |= (uint32_t)d << (2 * depth);
      depth++;
      int nt = t + jump_off(d);
      removed |= 1u << mid_square(t, nt);
      visited |= 1u << nt;
      t = nt;
      rem = capture_dirs(s, t, king, visited);
      if (rem) continue;
      // leaf: no further jump from t
      bool stop = leaf(t, removed, depth, dirs);
      leaves++;
      if (stop) return leaves;
    }
    if (depth == 0) break;
    depth--;
    int d = (int)(dirs >> (2 * depth)) & 3;
    dirs &= ~(3u << (2 * depth));
    rem = (uint32_t)(rem_stack >> (4 * depth)) & 15u;
    rem_stack &= ~((uint64_t)15u << (4 * depth));
    int pt = t - jump_off(d);
    removed &= ~(1u << mid_square(pt, t));
    visited &= ~(1u << t);
    t = pt;
  }
  return leaves;
}

// Apply a move of the side to move: piece from -> to, capturing `removed`.
GA_HD void apply_move(Board &b, int from, int to, uint32_t removed) {
  const int turn = (int)(b.meta & 1u);
  const uint32_t fb = 1u << from, tb = 1u << to;
  uint32_t own = turn ? b.p2 : b.p1;
  uint32_t opp = turn ? b.p1 : b.p2;
  const bool was_king = (b.kings & fb) != 0;
  own = (own & ~fb) | tb;
  opp &= ~removed;
  uint32_t kings = b.kings & ~(removed | fb);
  const uint32_t far = turn ? kRow0 : kRow7;
  if (was_king || (tb & far)) kings |= tb;
  b.p1 = turn ? opp : own;
  b.p2 = turn ? own : opp;
  b.kings = kings;
  uint32_t msc = (b.meta >> 8) & 0xffu;
  msc = removed ? 0u : (msc < 255u ? msc + 1u : 255u);
  b.meta = (uint32_t)(turn ^ 1) | (msc << 8);
}

// Promotion flag of a move as the reference records it.
GA_HD bool promotes(const Board &b, int from, int to) {
  const int turn = (int)(b.meta & 1u);
  const uint32_t far = turn ? kRow0 : kRow7;
  return !((b.kings >> from) & 1u) && ((far >> to) & 1u);
}


// Packed 32-byte move record (gpuai_move): from, to, jumps, promoted,
// path[12] (landing squares), removed[12] (captured squares), pad[4] = 0;
// unused path/removed slots are 0xFF.  dirs holds 2 bits per jump.
GA_HD void pack_move(const Board &b, int from, int to, int jumps, uint32_t dirs, uint32_t w[8]) {
  w[0] = (uint32_t)from | ((uint32_t)to << 8) | ((uint32_t)jumps << 16) |
         ((promotes(b, from, to) ? 1u : 0u) << 24);
#pragma unroll
  for (int q = 1; q < 7; q++) w[q] = 0xffffffffu;
  w[7] = 0;
  int t = from;
  for (int q = 0; q < jumps && q < 12; q++) {
    const int d = (int)(dirs >> (2 * q)) & 3;
    const int nt = t + jump_off(d);
    const int mid = mid_square(t, nt);
    const int pb = 4 + q, rb = 16 + q;  // byte offsets of path[q], removed[q]
    w[pb >> 2] = (w[pb >> 2] & ~(0xffu << (8 * (pb & 3)))) | ((uint32_t)nt << (8 * (pb & 3)));
    w[rb >> 2] = (w[rb >> 2] & ~(0xffu << (8 * (rb & 3)))) | ((uint32_t)mid << (8 * (rb & 3)));
    t = nt;
  }
}

// ---------------------------------------------------------------- Philox

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
GA_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
#if defined(__CUDA_ARCH__)
    uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

GA_HD uint32_t mulhi_index(uint32_t r, uint32_t n) {
#if defined(__CUDA_ARCH__)
  return __umulhi(r, n);
#else
  return (uint32_t)(((uint64_t)r * n) >> 32);
#endif
}

// Random stream (seed, id, tag): draw k is word k&3 of
// philox4x32_10(ctr = {k>>2, id_lo, id_hi, tag}, key = {seed_lo, seed_hi}).
struct Stream {
  uint32_t k0, k1, id0, id1, tag;
  uint32_t k;       // draws consumed
  uint32_t buf[4];  // block k>>2 when (k&3) != 0

  GA_HD void init(uint64_t seed, uint64_t id, uint32_t tag_) {
    k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
    id0 = (uint32_t)id; id1 = (uint32_t)(id >> 32);
    tag = tag_; k = 0;
  }
  GA_HD uint32_t next() {
    uint32_t w = k & 3u;
    if (w == 0) {
      buf[0] = k >> 2; buf[1] = id0; buf[2] = id1; buf[3] = tag;
      philox4x32_10(buf, k0, k1);
    }
    k++;
    uint32_t r = buf[0];
    r = w == 1 ? buf[1] : r;
    r = w == 2 ? buf[2] : r;
    r = w == 3 ? buf[3] : r;
    return r;
  }
};

// ------------------------------------------------------------ move lists

// Number of legal moves of the side to move (J = jumpers(s)); -1 on a
// capture deeper than kMaxDepth.
GA_HD int count_moves(const Side &s, uint32_t J) {
  if (J) {
    int n = 0;
    for (uint32_t m = J; m; m &= m - 1) {
      int c = capture_walk(s, ctz(m), [](int, uint32_t, int, uint32_t) { return false; });
      if (c < 0) return -1;
      n += c;
    }
    return n;
  }
  uint32_t md[4];
  direct_masks(s, md);
  return popc(md[0]) + popc(md[1]) + popc(md[2]) + popc(md[3]);
}

// Visit the legal moves in list order: fn(from, to, removed, jumps, dirs)
// returns true to stop.  Returns the number of moves visited, -1 on a capture
// deeper than kMaxDepth.
template <class Fn>
GA_HD int for_each_move(const Side &s, uint32_t J, Fn &&fn) {
  int n = 0;
  if (J) {
    for (uint32_t m = J; m; m &= m - 1) {
      const int o = ctz(m);
      bool stop = false;
      int c = capture_walk(s, o, [&](int t, uint32_t removed, int depth, uint32_t dirs) {
        stop = fn(o, t, removed, depth, dirs);
        return stop;
      });
      if (c < 0) return -1;
      n += c;
      if (stop) return n;
    }
    return n;
  }
  uint32_t md[4];
  direct_masks(s, md);
  for (uint32_t any = md[0] | md[1] | md[2] | md[3]; any; any &= any - 1) {
    const int sq = ctz(any);
#pragma unroll
    for (int d = 0; d < 4; d++)
      if ((md[d] >> sq) & 1u) {
        n++;
        if (fn(sq, sq + step_off(sq, d), 0u, 0, (uint32_t)d)) return n;
      }
  }
  return n;
}

// ------------------------------------------------------------ move scoring

// Reference heuristic (src/heuristic.cu:20-49, src/heuristic.hpp:5-8) in Q16
// fixed point: weight = (own + d_own) / (opp + d_opp) with man = 1, king = 4,
// plus noise ~ N(0, 0.11) approximated by a centred Irwin-Hall sum of four
// 16-bit uniforms (two stream draws).  Integer arithmetic keeps the device
// and the CPU replay bit-identical.
constexpr int32_t kHeurNoiseK = 12486;  // 0.11 * 2^16 / (2^16 * sqrt(4/12)) * 2^16

GA_HD int32_t heur_noise_q16(uint32_t a, uint32_t b) {
  int32_t sum = (int32_t)(a & 0xffffu) + (int32_t)(a >> 16) + (int32_t)(b & 0xffffu) +
                (int32_t)(b >> 16);
  int64_t x = (int64_t)(sum - 131070) * kHeurNoiseK;
  return (int32_t)(x >> 16);
}

GA_HD int32_t heur_weight_q16(int num, int den) {
  if (den <= 0) return 0x3fffffff;
  return (int32_t)(((uint32_t)num << 16) / (uint32_t)den);
}

// Sum of the row numbers of the squares in m.
GA_HD int row_sum(uint32_t m) {
  return popc(m & 0xF0F0F0F0u) + 2 * popc(m & 0xFF00FF00u) + 4 * popc(m & 0xFFFF0000u);
}

// eps-greedy evaluation change of a move for the mover: men 4, kings 8, plus
// one unit per row a man has advanced toward promotion.
GA_HD int eps_delta(const Board &b, const Side &s, int from, int to, uint32_t removed) {
  const uint32_t capK = removed & b.kings, capM = removed & ~b.kings;
  const int nM = popc(capM);
  // opponent men advance toward row 0 when the mover is PLAYER_1
  const int adv_removed = s.turn ? row_sum(capM) : 7 * nM - row_sum(capM);
  int d = 8 * popc(capK) + 4 * nM + adv_removed;
  if (!((s.ownK >> from) & 1u)) {
    const int rf = from >> 2, rt = to >> 2;
    const int af = s.turn ? 7 - rf : rf, at = s.turn ? 7 - rt : rt;
    const uint32_t far = s.turn ? kRow0 : kRow7;
    d += ((far >> to) & 1u) ? 4 - af : at - af;
  }
  return d;
}

// ------------------------------------------------------------ one random ply

// Outcome of a finished game from the side to move's view is computed by the
// caller; this returns the number of legal moves and applies move
// index(n) for n >= 1.  `pick` maps n (>= 2) to an index in [0, n).
// Returns -1 on an internal limit (capture deeper than kMaxDepth).
template <class Pick>
GA_HD int play_ply(Board &b, Pick &&pick) {
  Side s;
  make_side(b, s);
  uint32_t J = jumpers(s);
  if (J) {
    // count all capture sequences, squares ascending
    int n = 0;
    for (uint32_t m = J; m; m &= m - 1) {
      int c = capture_walk(s, ctz(m), [](int, uint32_t, int, uint32_t) { return false; });
      if (c < 0) return -1;
      n += c;
    }
    uint32_t i = n >= 2 ? pick((uint32_t)n) : 0u;
    for (uint32_t m = J; m; m &= m - 1) {
      int o = ctz(m);
      int to = -1;
      uint32_t rem_mask = 0;
      uint32_t want = i;
      int c = capture_walk(s, o, [&](int t, uint32_t removed, int, uint32_t) {
        if (want == 0) { to = t; rem_mask = removed; return true; }
        want--;
        return false;
      });
      if (to >= 0) { apply_move(b, o, to, rem_mask); return n; }
      i -= (uint32_t)c;
    }
    return -1;  // unreachable
  }
  uint32_t md[4];
  direct_masks(s, md);
  int n = popc(md[0]) + popc(md[1]) + popc(md[2]) + popc(md[3]);
  if (n == 0) return 0;
  uint32_t i = n >= 2 ? pick((uint32_t)n) : 0u;
  uint32_t any = md[0] | md[1] | md[2] | md[3];
  for (;;) {
    int sq = ctz(any);
    uint32_t c0 = (md[0] >> sq) & 1u, c1 = (md[1] >> sq) & 1u, c2 = (md[2] >> sq) & 1u,
             c3 = (md[3] >> sq) & 1u;
    uint32_t c = c0 + c1 + c2 + c3;
    if (i < c) {
      // i-th set direction at sq, ascending
      int d;
      uint32_t dm = c0 | (c1 << 1) | (c2 << 2) | (c3 << 3);
      for (uint32_t q = 0; q < i; q++) dm &= dm - 1;
      d = ctz(dm);
      apply_move(b, sq, sq + step_off(sq, d), 0u);
      return n;
    }
    i -= c;
    any &= any - 1;
  }
}

// ------------------------------------------------------------ per-ply policies
// Each returns the number of legal moves (0: the side to move has lost), -1 on a limit.

GA_HD int ply_random(Board &b, Stream &rs) {
  return play_ply(b, [&](uint32_t n) { return mulhi_index(rs.next(), n); });
}

// Reference heuristic: argmax over moves of weight + noise (first maximum
// wins, as in src/heuristicPlayout.cpp:31-35).
GA_HD int ply_ref_heuristic(Board &b, Stream &rs) {
  Side s;
  make_side(b, s);
  const uint32_t J = jumpers(s);
  const int n = count_moves(s, J);
  if (n <= 0) return n;
  const uint32_t oppAll = s.opp;
  const int ownScore = popc(s.own) + 3 * popc(s.ownK);
  const int oppScore = popc(oppAll) + 3 * popc(oppAll & b.kings);
  int bf = -1, bt = 0;
  uint32_t br = 0;
  int32_t bw = 0;
  const bool draw = n >= 2;
  for_each_move(s, J, [&](int from, int to, uint32_t removed, int, uint32_t) {
    const bool prom = !((s.ownK >> from) & 1u) && (((s.turn ? kRow0 : kRow7) >> to) & 1u);
    const int dOwn = prom ? 3 : 0;
    const int dOpp = popc(removed) + 3 * popc(removed & b.kings);
    int32_t w = heur_weight_q16(ownScore + dOwn, oppScore - dOpp);
    if (draw) {
      uint32_t x = rs.next();
      uint32_t y = rs.next();
      w += heur_noise_q16(x, y);
    }
    if (bf < 0 || w > bw) { bf = from; bt = to; br = removed; bw = w; }
    return false;
  });
  apply_move(b, bf, bt, br);
  return n;
}

constexpr uint32_t kEpsThreshold = 429496730u;  // ceil(0.1 * 2^32)

GA_HD int ply_eps_greedy(Board &b, Stream &rs) {
  Side s;
  make_side(b, s);
  const uint32_t J = jumpers(s);
  const int n = count_moves(s, J);
  if (n <= 0) return n;
  int target = 0;  // index in the move list
  if (n >= 2) {
    if (rs.next() < kEpsThreshold) {
      target = (int)mulhi_index(rs.next(), (uint32_t)n);
    } else {
      int best = -1000000, ties = 0;
      for_each_move(s, J, [&](int from, int to, uint32_t removed, int, uint32_t) {
        int d = eps_delta(b, s, from, to, removed);
        if (d > best) { best = d; ties = 1; } else if (d == best) ties++;
        return false;
      });
      uint32_t pick = ties > 1 ? mulhi_index(rs.next(), (uint32_t)ties) : 0u;
      int idx = 0;
      for_each_move(s, J, [&](int from, int to, uint32_t removed, int, uint32_t) {
        if (eps_delta(b, s, from, to, removed) == best) {
          if (pick == 0) { target = idx; return true; }
          pick--;
        }
        idx++;
        return false;
      });
    }
  }
  int idx = 0;
  for_each_move(s, J, [&](int from, int to, uint32_t removed, int, uint32_t) {
    if (idx++ == target) { apply_move(b, from, to, removed); return true; }
    return false;
  });
  return n;
}

template <int POLICY>
GA_HD int ply(Board &b, Stream &rs) {
  if (POLICY == 1) return ply_ref_heuristic(b, rs);
  if (POLICY == 2) return ply_eps_greedy(b, rs);
  return ply_random(b, rs);
}

}  // namespace ga
