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
#define GA_UNROLL _Pragma("unroll")
#else
#define GA_HD inline
#define GA_UNROLL
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
GA_HD int jump_off(int d) { return (int)((0x00021012u >> (8 * d)) & 0xffu) - 9; }

// Square offset of a single step from square s in direction d.
GA_HD int step_off(int s, int d) {
  const int even = ((s >> 2) & 1) ^ 1;  // row parity of s
  return (int)((0x00010809u >> (8 * d)) & 0xffu) - 5 + even;  // 4, 3, -4, -5 on odd rows
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

// Jump sources per direction (both the jumped and the landing square on the
// board); a jump moves the square index by +9, +7, -7, -9 for D0..D3.
constexpr uint32_t kJumpSrc0 = 0x00777777u, kJumpSrc1 = 0x00EEEEEEu;
constexpr uint32_t kJumpSrc2 = 0x77777700u, kJumpSrc3 = 0xEEEEEE00u;

// Landing squares of jumps in direction D from the squares of x (x must be
// valid jump sources for D).
template <int D>
GA_HD uint32_t jump2(uint32_t x) {
  if (D == 0) return x << 9;
  if (D == 1) return x << 7;
  if (D == 2) return x >> 7;
  return x >> 9;
}

// Squares s with s + jump(D) in x and s a valid jump source.
template <int D>
GA_HD uint32_t jump2_back(uint32_t x) {
  if (D == 0) return (x >> 9) & kJumpSrc0;
  if (D == 1) return (x >> 7) & kJumpSrc1;
  if (D == 2) return (x << 7) & kJumpSrc2;
  return (x << 9) & kJumpSrc3;
}

GA_HD void make_side(const Board &b, Side &s) {
  s.turn = (int)(b.meta & 1u);
  s.own = s.turn ? b.p2 : b.p1;
  s.opp = s.turn ? b.p1 : b.p2;
  s.ownK = s.own & b.kings;
  s.empty = ~(b.p1 | b.p2);
  // jd[d] = {s : s+d is an opponent, s+2d is empty}; step<3-d> is the inverse of
  // step<d>, and step<3-d>(empty) is also the direct-move source mask of d.
  s.jd[0] = step<3>(s.opp & step<3>(s.empty));
  s.jd[1] = step<2>(s.opp & step<2>(s.empty));
  s.jd[2] = step<1>(s.opp & step<1>(s.empty));
  s.jd[3] = step<0>(s.opp & step<0>(s.empty));
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
GA_UNROLL
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
      int j = (int)((0x12131210u >> (2u * rem)) & 3u);  // lowest set bit of the 4-bit set
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
GA_UNROLL
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
GA_UNROLL
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
GA_UNROLL
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

// Position of the rem-th set bit (ascending) of a 4-bit mask dm.
GA_HD int nth_bit4(uint32_t dm, uint32_t rem) {
  const uint32_t idx = dm * 4u + rem;  // 0..63, 2-bit entries, 16 per word
  const uint32_t w = idx >> 4;
  const uint32_t word = w == 0 ? 0x04010000u : (w == 1 ? 0x24090802u : (w == 2 ? 0x340D0C03u : 0xE439380Eu));
  return (int)((word >> (2u * (idx & 15u))) & 3u);
}

// Bits 0..3 of x spread to bits 0, 8, 16, 24 (x < 16).
GA_HD uint32_t spread4(uint32_t x) { return (x * 0x00204081u) & 0x01010101u; }

// Number of bytes k of P with P_k <= i, where the bytes of P are
// non-decreasing prefix sums below 128 and i < 128.  No byte borrows from its
// neighbour: each byte computes (0x80 | i) - P_k >= 1.
GA_HD uint32_t bytes_le(uint32_t P, uint32_t i) {
  const uint32_t D = ((i * 0x01010101u) | 0x80808080u) - P;
  return (((D & 0x80808080u) >> 7) * 0x01010101u) >> 24;
}

// Move i of the list whose per-direction source masks are M0..M3 (a square's
// moves in one direction each; squares ascending, within a square the
// directions ascending, or descending for a man's captures, which search
// dc = -1 first).  Returns the source square, the destination square and the
// captured squares.  No search over the squares: the per-square move counts
// (0..4) are three bit planes; the moves below squares 8, 16 and 24 are
// counted with POPC (the XU pipe, idle in the playout kernel, whose integer
// ALU pipe is the busy one) and three compares pick the byte; the chosen
// byte's low half is counted the same way; the chosen half's four counts are
// spread to bytes by one multiply and a byte-parallel compare of their prefix
// sums picks the square; the direction is the rank among the square's
// direction bits, found by three compares.  Every square holds at most four
// moves, so every prefix sum of a half fits a byte below 128.
GA_HD void nth_move(uint32_t M0, uint32_t M1, uint32_t M2, uint32_t M3, uint32_t i, bool capture,
                         uint32_t men, int &from, int &to, uint32_t &removed) {
  const uint32_t a0 = M0 ^ M1, a1 = M0 & M1, b0 = M2 ^ M3, b1 = M2 & M3;
  const uint32_t S0 = a0 ^ b0, k0 = a0 & b0;
  const uint32_t S1 = a1 ^ b1 ^ k0, S2 = (a1 & b1) | (k0 & (a1 ^ b1));
  // moves on squares below 8, 16, 24
  const uint32_t P1 = (uint32_t)(popc(S0 & 0xFFu) + 2 * popc(S1 & 0xFFu) + 4 * popc(S2 & 0xFFu));
  const uint32_t P2 = (uint32_t)(popc(S0 & 0xFFFFu) + 2 * popc(S1 & 0xFFFFu) + 4 * popc(S2 & 0xFFFFu));
  const uint32_t P3 = (uint32_t)(popc(S0 & 0xFFFFFFu) + 2 * popc(S1 & 0xFFFFFFu) + 4 * popc(S2 & 0xFFFFFFu));
  const bool g1 = i >= P1, g2 = i >= P2, g3 = i >= P3;
  const uint32_t sh = g3 ? 24u : (g2 ? 16u : (g1 ? 8u : 0u));
  const uint32_t rem = i - (g3 ? P3 : (g2 ? P2 : (g1 ? P1 : 0u)));
  const uint32_t e0 = S0 >> sh, e1 = S1 >> sh, e2 = S2 >> sh;
  const uint32_t tlo = (uint32_t)(popc(e0 & 15u) + 2 * popc(e1 & 15u) + 4 * popc(e2 & 15u));
  const bool hi = rem >= tlo;
  const uint32_t hs = hi ? 4u : 0u;
  const uint32_t Q = spread4((e0 >> hs) & 15u) + 2u * spread4((e1 >> hs) & 15u) + 4u * spread4((e2 >> hs) & 15u);
  const uint32_t R = Q * 0x01010101u;
  const uint32_t rem2 = hi ? rem - tlo : rem;
  const uint32_t q = bytes_le(R, rem2);
  const uint32_t sq = sh + hs + q;
  const uint32_t r0 = rem2 - (((R << 8) >> (8u * q)) & 0xffu);
  const uint32_t cnt = (Q >> (8u * q)) & 0xffu;
  const uint32_t x0 = (M0 >> sq) & 1u, x1 = (M1 >> sq) & 1u, x2 = (M2 >> sq) & 1u;
  const uint32_t r = (capture && ((men >> sq) & 1u)) ? cnt - 1u - r0 : r0;
  const uint32_t c01 = x0 + x1;
  const uint32_t d = (uint32_t)(r >= x0) + (uint32_t)(r >= c01) + (uint32_t)(r >= c01 + x2);
  const uint32_t sd = 8u * d;
  const int s = (int)sq;
  const int mid = s + (int)((0x00010809u >> sd) & 0xffu) - 5 + (((s >> 2) & 1) ^ 1);
  from = s;
  to = capture ? s + (int)((0x00021012u >> sd) & 0xffu) - 9 : mid;
  removed = capture ? 1u << mid : 0u;
}

// Move masks of a position in which no capture can continue, so that every
// legal move is a direct move or a single jump: M[d] = the squares that move
// in direction d and `capture` whether they jump; move i of the list is then
// nth_move(M[0], M[1], M[2], M[3], i, capture, men, ...) and the count is
// the masks' population.  Returns false when some capture can continue (the
// list then needs the search, for_each_move).
GA_HD bool simple_move_masks(const Side &s, uint32_t M[4], bool &capture) {
  const uint32_t men = s.own & ~s.ownK;
  const uint32_t m01 = s.turn ? s.ownK : s.own;  // D0/D1 movers: P1 men and all kings
  const uint32_t m23 = s.turn ? s.own : s.ownK;  // D2/D3 movers: P2 men and all kings
  const uint32_t J0 = m01 & s.jd[0], J1 = m01 & s.jd[1], J2 = m23 & s.jd[2], J3 = m23 & s.jd[3];
  capture = (J0 | J1 | J2 | J3) != 0;
  if (capture) {
    const uint32_t jall = s.jd[0] | s.jd[1] | s.jd[2] | s.jd[3];
    const uint32_t jf = s.turn ? (s.jd[2] | s.jd[3]) : (s.jd[0] | s.jd[1]);
    const uint32_t lm = jump2<0>(J0 & men) | jump2<1>(J1 & men) | jump2<2>(J2 & men) | jump2<3>(J3 & men);
    const uint32_t lk = jump2<0>(J0 & s.ownK) | jump2<1>(J1 & s.ownK) | jump2<2>(J2 & s.ownK) |
                        jump2<3>(J3 & s.ownK);
    if ((lk & jall) | (lm & jf)) return false;
    M[0] = J0;
    M[1] = J1;
    M[2] = J2;
    M[3] = J3;
    return true;
  }
  M[0] = m01 & step<3>(s.empty);
  M[1] = m01 & step<2>(s.empty);
  M[2] = m23 & step<1>(s.empty);
  M[3] = m23 & step<0>(s.empty);
  return true;
}

// Squares of the side to move whose capture can continue after the first
// jump (they need the depth-first search); J[d] are the first-jump sources.
GA_HD uint32_t continuing_sources(const Side &s, const uint32_t J[4]) {
  const uint32_t men = s.own & ~s.ownK;
  const uint32_t jall = s.jd[0] | s.jd[1] | s.jd[2] | s.jd[3];
  const uint32_t jf = s.turn ? (s.jd[2] | s.jd[3]) : (s.jd[0] | s.jd[1]);
  const uint32_t cm = (J[0] & jump2_back<0>(jf)) | (J[1] & jump2_back<1>(jf)) | (J[2] & jump2_back<2>(jf)) |
                      (J[3] & jump2_back<3>(jf));
  const uint32_t ck = (J[0] & jump2_back<0>(jall)) | (J[1] & jump2_back<1>(jall)) |
                      (J[2] & jump2_back<2>(jall)) | (J[3] & jump2_back<3>(jall));
  return (cm & men) | (ck & s.ownK);
}

// General ply: returns the number of legal moves and applies move
// pick(n) for n >= 1, where `pick` maps n to an index in [0, n), drawing from
// the random stream only when n >= 2.
// Captures whose first jump can be extended are enumerated by the
// depth-first search (counts of the first four such squares are kept, so each
// is walked once to count and at most once more to select); single jumps are
// counted from the direction masks.  Returns -1 on an internal limit (capture
// deeper than kMaxDepth).
template <class Pick>
GA_HD int play_ply(Board &b, Pick &&pick) {
  Side s;
  make_side(b, s);
  const uint32_t m01 = s.turn ? s.ownK : s.own;
  const uint32_t m23 = s.turn ? s.own : s.ownK;
  const uint32_t J[4] = {m01 & s.jd[0], m01 & s.jd[1], m23 & s.jd[2], m23 & s.jd[3]};
  const uint32_t Jall = J[0] | J[1] | J[2] | J[3];
  if (Jall) {
    const uint32_t men = s.own & ~s.ownK;
    const uint32_t X = continuing_sources(s, J);
    const uint32_t M0 = J[0] & ~X, M1 = J[1] & ~X, M2 = J[2] & ~X, M3 = J[3] & ~X;
    int n = popc(M0) + popc(M1) + popc(M2) + popc(M3);
    if (X != 0 && (X & (X - 1u)) == 0) {
      // One square x whose capture can continue (almost every such ply): its
      // sequences sit between the single jumps of the squares below x and
      // those above it, so only x is walked, once to count and once to select.
      const int x = popc(X - 1u);
      const uint32_t below = X - 1u;
      const uint32_t nb = (uint32_t)(popc(M0 & below) + popc(M1 & below) + popc(M2 & below) + popc(M3 & below));
      const int c = capture_walk(s, x, [](int, uint32_t, int, uint32_t) { return false; });
      if (c < 0) return -1;
      n += c;
      const uint32_t i = pick((uint32_t)n);
      int from = x, to = x;
      uint32_t removed = 0;
      if (i - nb < (uint32_t)c) {  // i in [nb, nb + c): a sequence of x
        uint32_t want = i - nb;
        capture_walk(s, x, [&](int t, uint32_t rm, int, uint32_t) {
          if (want == 0) { to = t; removed = rm; return true; }
          want--;
          return false;
        });
      } else {
        nth_move(M0, M1, M2, M3, i < nb ? i : i - (uint32_t)c, true, men, from, to, removed);
      }
      apply_move(b, from, to, removed);
      return n;
    }
    uint32_t cache = 0;  // 8-bit sequence counts of the first four searched squares
    int q = 0;
    for (uint32_t m = X; m; m &= m - 1) {
      const int c = capture_walk(s, ctz(m), [](int, uint32_t, int, uint32_t) { return false; });
      if (c < 0) return -1;
      n += c;
      if (q < 4) cache |= (uint32_t)(c < 255 ? c : 255) << (8 * q++);
    }
    uint32_t i = pick((uint32_t)n);
    q = 0;
    for (uint32_t m = Jall; m; m &= m - 1) {
      const int sq = ctz(m);
      if ((X >> sq) & 1u) {
        uint32_t c = q < 4 ? (cache >> (8 * q)) & 0xffu : 255u;
        if (c == 255u) c = (uint32_t)capture_walk(s, sq, [](int, uint32_t, int, uint32_t) { return false; });
        q++;
        if (i >= c) {
          i -= c;
          continue;
        }
        int to = -1;
        uint32_t rem_mask = 0, want = i;
        capture_walk(s, sq, [&](int t, uint32_t removed, int, uint32_t) {
          if (want == 0) { to = t; rem_mask = removed; return true; }
          want--;
          return false;
        });
        apply_move(b, sq, to, rem_mask);
        return n;
      }
      const uint32_t dm = ((J[0] >> sq) & 1u) | (((J[1] >> sq) & 1u) << 1) | (((J[2] >> sq) & 1u) << 2) |
                          (((J[3] >> sq) & 1u) << 3);
      const uint32_t cnt = (uint32_t)popc(dm);
      if (i >= cnt) {
        i -= cnt;
        continue;
      }
      // men search dc = -1 first: the reverse of the ascending direction order
      const uint32_t rem = ((men >> sq) & 1u) ? cnt - 1u - i : i;
      const int d = nth_bit4(dm, rem);
      const int to = sq + jump_off(d);
      apply_move(b, sq, to, 1u << mid_square(sq, to));
      return n;
    }
    return -1;  // unreachable: i < n
  }
  uint32_t md[4];
  direct_masks(s, md);
  const int n = popc(md[0]) + popc(md[1]) + popc(md[2]) + popc(md[3]);
  if (n == 0) return 0;
  uint32_t i = pick((uint32_t)n);
  for (uint32_t any = md[0] | md[1] | md[2] | md[3];; any &= any - 1) {
    const int sq = ctz(any);
    const uint32_t dm = ((md[0] >> sq) & 1u) | (((md[1] >> sq) & 1u) << 1) | (((md[2] >> sq) & 1u) << 2) |
                        (((md[3] >> sq) & 1u) << 3);
    const uint32_t c = (uint32_t)popc(dm);
    if (i < c) {
      const int d = nth_bit4(dm, i);
      apply_move(b, sq, sq + step_off(sq, d), 0u);
      return n;
    }
    i -= c;
  }
}

// ------------------------------------------------------------ men's multi-jumps

// Number of maximal capture continuations C(t) in 1..4 for a man of the side
// to move that has just landed on square t, for every square at once, as
// three bit-planes.  Men only move forward, so C(t) depends on the original
// board alone (captured pieces stay on the board during the search, and no
// square is visited twice): C(t) = 1 without a further jump, else the sum of
// C over the landing squares of the possible jumps.  FA/FB are the forward
// directions in search order (dc = -1 first).  Two rounds are exact for every
// square a first jump can land on.
struct ManTree {
  uint32_t c0, c1, c2;
  GA_HD uint32_t at(int t) const {
    return ((c0 >> t) & 1u) + 2u * ((c1 >> t) & 1u) + 4u * ((c2 >> t) & 1u);
  }
};

template <int FA, int FB>
GA_HD ManTree man_tree(const Side &s) {
  const uint32_t A = s.jd[FA], B = s.jd[FB], any = A | B;
  uint32_t c0 = ~0u, c1 = 0u, c2 = 0u;
GA_UNROLL
  for (int r = 0; r < 2; r++) {
    const uint32_t a0 = jump2_back<FA>(c0) & A, a1 = jump2_back<FA>(c1) & A, a2 = jump2_back<FA>(c2) & A;
    const uint32_t b0 = jump2_back<FB>(c0) & B, b1 = jump2_back<FB>(c1) & B, b2 = jump2_back<FB>(c2) & B;
    const uint32_t s0 = a0 ^ b0, k0 = a0 & b0;
    const uint32_t s1 = a1 ^ b1 ^ k0, k1 = (a1 & b1) | (k0 & (a1 ^ b1));
    const uint32_t s2 = a2 ^ b2 ^ k1;
    c0 = s0 | ~any;
    c1 = s1 & any;
    c2 = s2 & any;
  }
  return ManTree{c0, c1, c2};
}

// Number of capture sequences a man on each square of m starts with a jump in
// direction F, weighted by the continuations C of its landing square.
template <int F>
GA_HD int man_weight(uint32_t m, const ManTree &c) {
  return popc(m & jump2_back<F>(c.c0)) + 2 * popc(m & jump2_back<F>(c.c1)) + 4 * popc(m & jump2_back<F>(c.c2));
}

// A capture ply where some man can continue a capture but no king can: the
// move list is counted with man_tree instead of a search and move i is found
// by descending it.
template <int FA, int FB, class Pick>
GA_HD int play_ply_men_multi(Board &b, const Side &s, const uint32_t J[4], Pick &&pick) {
  const uint32_t men = s.own & ~s.ownK;
  const ManTree c = man_tree<FA, FB>(s);
  const uint32_t mA = J[FA] & men, mB = J[FB] & men;
  const uint32_t k0 = J[0] & s.ownK, k1 = J[1] & s.ownK, k2 = J[2] & s.ownK, k3 = J[3] & s.ownK;
  const int n = man_weight<FA>(mA, c) + man_weight<FB>(mB, c) + popc(k0) + popc(k1) + popc(k2) + popc(k3);
  uint32_t i = pick((uint32_t)n);
  for (uint32_t X = J[0] | J[1] | J[2] | J[3]; X; X &= X - 1) {
    const int sq = ctz(X);
    if ((men >> sq) & 1u) {
      const uint32_t wa = ((mA >> sq) & 1u) ? c.at(sq + jump_off(FA)) : 0u;
      const uint32_t wb = ((mB >> sq) & 1u) ? c.at(sq + jump_off(FB)) : 0u;
      if (i >= wa + wb) {
        i -= wa + wb;
        continue;
      }
      // descend: at each landing take the first direction whose subtree holds i
      int t = sq;
      uint32_t removed = 0;
      uint32_t availA = (mA >> sq) & 1u, availB = (mB >> sq) & 1u;
      while (availA | availB) {
        const uint32_t w = availA ? c.at(t + jump_off(FA)) : 0u;
        const int f = (availA && i < w) ? FA : FB;
        if (f == FB) i -= w;
        const int nt = t + jump_off(f);
        removed |= 1u << mid_square(t, nt);
        t = nt;
        availA = (s.jd[FA] >> t) & 1u;
        availB = (s.jd[FB] >> t) & 1u;
      }
      apply_move(b, sq, t, removed);
      return n;
    }
    const uint32_t dm = ((k0 >> sq) & 1u) | (((k1 >> sq) & 1u) << 1) | (((k2 >> sq) & 1u) << 2) |
                        (((k3 >> sq) & 1u) << 3);
    const uint32_t cnt = (uint32_t)popc(dm);
    if (i >= cnt) {
      i -= cnt;
      continue;
    }
    const int d = nth_bit4(dm, i);
    const int to = sq + jump_off(d);
    apply_move(b, sq, to, 1u << mid_square(sq, to));
    return n;
  }
  return -1;  // unreachable: i < n
}

// A capture ply where only men can continue, and the side to move has one
// first jump whose chain never forks, has exactly one legal move (about two
// thirds of men's multi-jump plies in random play).  It is played here by
// following the chain on the jump masks of the position, as the men's tree
// (play_ply_men_multi) would play its only move: captured men stay on the
// board until the move is applied and a man only jumps forward, so the chain
// is fixed by the position.  A ply with one move takes no draw under any
// policy.  Returns false, with the board untouched, when there are two or
// more moves.
GA_HD bool play_forced_men_multi(Board &b, const Side &s, uint32_t J0, uint32_t J1, uint32_t J2, uint32_t J3) {
  if (popc(J0) + popc(J1) + popc(J2) + popc(J3) != 1) return false;
  const int d = J0 ? 0 : (J1 ? 1 : (J2 ? 2 : 3));
  const int from = ctz(J0 | J1 | J2 | J3);
  const int dA = s.turn ? 2 : 0;  // forward jumps of the side's men: D0/D1 or D2/D3
  const uint32_t JA = s.turn ? s.jd[2] : s.jd[0], JB = s.turn ? s.jd[3] : s.jd[1];  // constant indices: registers
  int t = from + jump_off(d);
  uint32_t removed = 1u << mid_square(from, t);
GA_UNROLL
  for (int k = 0; k < 3; k++) {  // a man jumps at most three times in all
    const uint32_t a = (JA >> t) & 1u, c = (JB >> t) & 1u;
    if (a & c) return false;  // the chain forks: two or more moves
    if (!(a | c)) break;
    const int nt = t + jump_off(a ? dA : dA + 1);
    removed |= 1u << mid_square(t, nt);
    t = nt;
  }
  apply_move(b, from, t, removed);
  return true;
}

// A capture ply where a king's capture can continue, with one first jump in
// all and a chain that never forks, has exactly one legal move (about 70 % of
// those plies in random play).  It is played here by following the chain with
// the depth-first search's rules (capture_dirs: the position's jump masks, no
// landing square twice in one sequence), as play_ply would play its only
// move.  Returns false, with the board untouched, when there are two or more
// moves or the chain reaches the depth limit (the search then reports it).
GA_HD bool play_forced_king_chain(Board &b, const Side &s, uint32_t J0, uint32_t J1, uint32_t J2, uint32_t J3) {
  if (popc(J0) + popc(J1) + popc(J2) + popc(J3) != 1) return false;
  const int d0 = J0 ? 0 : (J1 ? 1 : (J2 ? 2 : 3));
  const int from = ctz(J0 | J1 | J2 | J3);
  if (!((s.ownK >> from) & 1u)) return false;  // only a king's chain is followed here
  int t = from + jump_off(d0);
  uint32_t removed = 1u << mid_square(from, t), visited = 1u << t;
  for (int depth = 1;; depth++) {  // ends: each jump lands on a square not yet visited
    const uint32_t rem = capture_dirs(s, t, true, visited);
    if (rem == 0) break;
    if ((rem & (rem - 1u)) != 0 || depth >= kMaxDepth) return false;
    const int d = (int)((0x12131210u >> (2u * rem)) & 3u);  // the one direction left
    const int nt = t + jump_off(d);
    removed |= 1u << mid_square(t, nt);
    visited |= 1u << nt;
    t = nt;
  }
  apply_move(b, from, t, removed);
  return true;
}

constexpr int kNeedMen = -2;   // a men's multi-jump ply was deferred
constexpr int kNeedKing = -3;  // a ply where a king's capture can continue was deferred

// Deferred-ply schedule of the playout kernel (iteration it of its warp
// loop): Philox blocks are generated on it % 4 == 0 (it % 2 == 0 for
// eps-greedy), men's multi-jumps are played on it % kMenPeriod == kMenPhase,
// king capture searches on it % king_period(policy) == kKingPhase (powers of
// 2, phases away from the refill and the compaction iterations); once the
// work runs out, a warp with at most sparse_lanes(policy) games defers nothing.  The
// uniform random policy waits longer for king searches (16 iterations) than
// the other two (8), whose plies cost more and leave fewer lanes waiting.
constexpr uint32_t kMenPeriod = 4, kMenPhase = 2;
constexpr uint32_t kKingPeriod = 16, kKingPhase = 6;
GA_HD constexpr uint32_t king_period(int policy) { return policy == 0 ? kKingPeriod : kKingPeriod / 2; }
// Men's multi-jumps are deferred for the eps-greedy and reference-heuristic
// policies only: the uniform random policy plays them at once (measured on
// one box: 0.3748 against 0.3761 ms on the benchmark batch, 3.92 against
// 3.96 ms on 64 x 65,536), the eps-greedy one loses 3 % without deferral.
GA_HD constexpr bool defer_men(int policy) { return policy != 0; }
// a deferred ply must have a phase that comes round, or its game never ends
static_assert((kMenPeriod & (kMenPeriod - 1u)) == 0 && kMenPhase < kMenPeriod, "men's phase outside its period");
static_assert((kKingPeriod & (kKingPeriod - 1u)) == 0 && kKingPhase < kKingPeriod / 2,
              "king phase outside the shorter king period");
// Once the work runs out, a warp with at most sparse_lanes(policy) games
// defers nothing: for the uniform random policy that is every warp (its
// batch tail is the longest games' plies, which a deferral would delay;
// measured 0.6 % faster than a limit of 4 or 16), for the other two 4 games.
GA_HD constexpr uint32_t sparse_lanes(int policy) { return policy == 0 ? 32u : 4u; }

// One uniformly random ply, branch-free for direct moves and for captures
// that cannot be extended (the common cases).  Positions where some capture
// can continue take the bit-sliced men's tree (play_ply_men_multi) when only
// men continue, or the depth-first search with the cycle check (play_ply)
// when a king does.  A caller that batches these rarer plies passes
// men_now / king_now = false: the ply then returns kNeedMen / kNeedKing
// without touching the board or the stream, and is played by a later call
// that allows it.  Same move list order, same index -> move map as play_ply.
template <class Pick>
GA_HD int play_ply_sched(Board &b, Pick &&pick, bool men_now, bool king_now) {
  Side s;
  make_side(b, s);
  const uint32_t men = s.own & ~s.ownK;
  const uint32_t m01 = s.turn ? s.ownK : s.own;  // D0/D1 movers: P1 men and all kings
  const uint32_t m23 = s.turn ? s.own : s.ownK;  // D2/D3 movers: P2 men and all kings
  const uint32_t J0 = m01 & s.jd[0], J1 = m01 & s.jd[1], J2 = m23 & s.jd[2], J3 = m23 & s.jd[3];
  const bool capture = (J0 | J1 | J2 | J3) != 0;
  // landing squares from which the same piece could jump again
  const uint32_t jall = s.jd[0] | s.jd[1] | s.jd[2] | s.jd[3];
  const uint32_t jf = s.turn ? (s.jd[2] | s.jd[3]) : (s.jd[0] | s.jd[1]);
  const uint32_t lm = jump2<0>(J0 & men) | jump2<1>(J1 & men) | jump2<2>(J2 & men) | jump2<3>(J3 & men);
  const uint32_t lk = jump2<0>(J0 & s.ownK) | jump2<1>(J1 & s.ownK) | jump2<2>(J2 & s.ownK) |
                      jump2<3>(J3 & s.ownK);
  const uint32_t cont_k = lk & jall, cont_m = lm & jf;
  if (cont_k | cont_m) {
    if (cont_k) {
      if (play_forced_king_chain(b, s, J0, J1, J2, J3)) return 1;
      if (!king_now) return kNeedKing;
      return play_ply(b, pick);  // a king can continue: depth-first search with the cycle check
    }
    if (play_forced_men_multi(b, s, J0, J1, J2, J3)) return 1;
    if (!men_now) return kNeedMen;
    // only men continue: counted on the bit-sliced continuation tree
    const uint32_t J[4] = {J0, J1, J2, J3};
    return s.turn ? play_ply_men_multi<3, 2>(b, s, J, pick) : play_ply_men_multi<1, 0>(b, s, J, pick);
  }
  const uint32_t M0 = capture ? J0 : (m01 & step<3>(s.empty));
  const uint32_t M1 = capture ? J1 : (m01 & step<2>(s.empty));
  const uint32_t M2 = capture ? J2 : (m23 & step<1>(s.empty));
  const uint32_t M3 = capture ? J3 : (m23 & step<0>(s.empty));
  const int n = popc(M0) + popc(M1) + popc(M2) + popc(M3);
  if (n == 0) return 0;
  const uint32_t i = pick((uint32_t)n);
  int from, to;
  uint32_t removed;
  nth_move(M0, M1, M2, M3, i, capture, men, from, to, removed);
  apply_move(b, from, to, removed);
  return n;
}

// One uniformly random ply with every kind of ply played at once.
template <class Pick>
GA_HD int play_ply_fast(Board &b, Pick &&pick) {
  return play_ply_sched(b, pick, true, true);
}

// Random draws of one stream buffered eight at a time, so that a warp can
// generate Philox blocks for all its lanes at the same loop iteration.
// refill() keeps at least four draws buffered; next() consumes one.
struct DrawRing {
  uint32_t a0, a1, a2, a3, b0, b1, b2, b3;  // slots 0-3 and 4-7
  uint32_t k, avail;
  uint32_t k0, k1, id0, id1, tag;

  GA_HD void start(uint64_t seed, uint64_t id, uint32_t tag_) {
    k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
    id0 = (uint32_t)id; id1 = (uint32_t)(id >> 32);
    tag = tag_; k = 0; avail = 0;
  }
  GA_HD void refill() {
    if (avail >= 4) return;
    const uint32_t pos = k + avail;  // multiple of 4
    uint32_t c[4] = {pos >> 2, id0, id1, tag};
    philox4x32_10(c, k0, k1);
    const bool hi = (pos & 4u) != 0;
    a0 = hi ? a0 : c[0]; a1 = hi ? a1 : c[1]; a2 = hi ? a2 : c[2]; a3 = hi ? a3 : c[3];
    b0 = hi ? c[0] : b0; b1 = hi ? c[1] : b1; b2 = hi ? c[2] : b2; b3 = hi ? c[3] : b3;
    avail += 4;
  }
  // Move index in [0, n) for n >= 1; a draw is consumed only when n >= 2.
  GA_HD uint32_t pick(uint32_t n) {
    const bool hi = (k & 4u) != 0;
    const uint32_t w = k & 3u;
    const uint32_t x0 = hi ? b0 : a0, x1 = hi ? b1 : a1, x2 = hi ? b2 : a2, x3 = hi ? b3 : a3;
    const uint32_t r = w == 0 ? x0 : (w == 1 ? x1 : (w == 2 ? x2 : x3));
    const uint32_t use = n >= 2 ? 1u : 0u;
    k += use;
    avail -= use;
    return use ? mulhi_index(r, n) : 0u;
  }
  GA_HD uint32_t next() {
    const bool hi = (k & 4u) != 0;
    const uint32_t w = k & 3u;
    const uint32_t x0 = hi ? b0 : a0, x1 = hi ? b1 : a1, x2 = hi ? b2 : a2, x3 = hi ? b3 : a3;
    const uint32_t r = w == 0 ? x0 : (w == 1 ? x1 : (w == 2 ? x2 : x3));
    k++;
    avail--;
    return r;
  }
};

// Draws from a DrawRing for code that may take any number of them: a block is
// generated whenever fewer than four are buffered (for the rare plies that
// enumerate their moves; the warp loop keeps Philox convergent otherwise).
struct RingOnDemand {
  DrawRing &r;
  GA_HD uint32_t next() {
    r.refill();
    return r.next();
  }
};

// ------------------------------------------------------------ per-ply policies
// Each returns the number of legal moves (0: the side to move has lost), -1 on a limit.

template <class Rng>
GA_HD int ply_random(Board &b, Rng &rs) {
  return play_ply_fast(b, [&](uint32_t n) { return n >= 2 ? mulhi_index(rs.next(), n) : 0u; });
}

// Reference heuristic: argmax over moves of weight + noise (first maximum
// wins, as in src/heuristicPlayout.cpp:31-35).
template <class Rng>
GA_HD int ply_ref_heuristic(Board &b, Rng &rs) {
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

template <class Rng>
GA_HD int ply_eps_greedy(Board &b, Rng &rs) {
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

// ------------------------------------------------------------ eps-greedy without enumeration

// Bit plane q of a per-square value c + sgn * row (4 squares per row).
GA_HD constexpr uint32_t row_value_plane(int q, int c, int sgn) {
  uint32_t m = 0;
  for (int r = 0; r < 8; r++)
    if (((c + sgn * r) >> q) & 1) m |= 0xFu << (4 * r);
  return m;
}

// eps_delta + 1 of a single jump by a man that does not promote, minus 3,
// for a captured man, by the jumping square's row: 4 + the captured man's
// advancement.  PLAYER_1 moving up (captured man one row above): 10 - row;
// down: 12 - row; PLAYER_2 up: 5 + row; down: 3 + row.  Four bit planes each.
struct RowValue { uint32_t q0, q1, q2, q3; };
GA_HD constexpr RowValue row_value(int c, int sgn) {
  return RowValue{row_value_plane(0, c, sgn), row_value_plane(1, c, sgn), row_value_plane(2, c, sgn),
                  row_value_plane(3, c, sgn)};
}

// The moves of largest eps_delta among the moves M[0..3] of a position where
// no capture can continue, as subsets B[0..3] (list order is kept, so move i
// of B is the i-th best move of the list).  Direct moves: a man's step +1, a
// king's 0, a promoting step -2.  Single jumps: captured king 8, captured man
// 4 + its advancement; a man's jump +2, a promoting jump -1, a king's 0.
// The jump values (+1, at most 13) are kept as four bit planes per direction
// and the maximum is found bit by bit from the top plane.
template <int D>
GA_HD void eps_jump_planes(const Side &s, uint32_t m, uint32_t oppK, uint32_t men, uint32_t promoJ, uint32_t y[4]) {
  constexpr bool up = D < 2;
  constexpr RowValue p1 = up ? row_value(10, -1) : row_value(12, -1);
  constexpr RowValue p2 = up ? row_value(5, 1) : row_value(3, 1);
  const uint32_t w0 = s.turn ? p2.q0 : p1.q0, w1 = s.turn ? p2.q1 : p1.q1;
  const uint32_t w2 = s.turn ? p2.q2 : p1.q2, w3 = s.turn ? p2.q3 : p1.q3;
  const uint32_t ck = m & step<3 - D>(oppK);  // the jumped square holds a king: value 8
  const uint32_t x0 = w0 & ~ck, x1 = w1 & ~ck, x2 = w2 & ~ck, x3 = w3 | ck;
  const uint32_t mnp = m & men & ~promoJ;
  const uint32_t a0 = (m & s.ownK) | mnp, a1 = mnp;  // + 1 for a king, + 3 for a man, + 0 for a promoting man
  const uint32_t c0 = x0 & a0;
  const uint32_t c1 = (x1 & a1) | (c0 & (x1 ^ a1));
  const uint32_t c2 = x2 & c1;
  y[0] = x0 ^ a0;
  y[1] = x1 ^ a1 ^ c0;
  y[2] = x2 ^ c1;
  y[3] = x3 ^ c2;
}

GA_HD void eps_best(const Board &b, const Side &s, bool capture, const uint32_t M[4], uint32_t B[4]) {
  const uint32_t men = s.own & ~s.ownK;
  if (!capture) {
    const uint32_t promoD = s.turn ? 0x000000F0u : 0x0F000000u;  // a man stepping from here promotes
    uint32_t np = 0, kk = 0;
GA_UNROLL
    for (int d = 0; d < 4; d++) {
      np |= M[d] & men & ~promoD;
      kk |= M[d] & s.ownK;
    }
GA_UNROLL
    for (int d = 0; d < 4; d++)
      B[d] = np ? (M[d] & men & ~promoD) : (kk ? (M[d] & s.ownK) : (M[d] & men & promoD));
    return;
  }
  const uint32_t oppK = s.opp & b.kings;
  const uint32_t promoJ = s.turn ? 0x00000F00u : 0x00F00000u;  // a man jumping from here promotes
  uint32_t y0[4], y1[4], y2[4], y3[4];
  eps_jump_planes<0>(s, M[0], oppK, men, promoJ, y0);
  eps_jump_planes<1>(s, M[1], oppK, men, promoJ, y1);
  eps_jump_planes<2>(s, M[2], oppK, men, promoJ, y2);
  eps_jump_planes<3>(s, M[3], oppK, men, promoJ, y3);
  uint32_t c0 = M[0], c1 = M[1], c2 = M[2], c3 = M[3];
GA_UNROLL
  for (int q = 3; q >= 0; q--) {
    const uint32_t t0 = c0 & y0[q], t1 = c1 & y1[q], t2 = c2 & y2[q], t3 = c3 & y3[q];
    const bool any = (t0 | t1 | t2 | t3) != 0;
    c0 = any ? t0 : c0;
    c1 = any ? t1 : c1;
    c2 = any ? t2 : c2;
    c3 = any ? t3 : c3;
  }
  B[0] = c0; B[1] = c1; B[2] = c2; B[3] = c3;
}

// One eps-greedy ply (the move ply_eps_greedy plays, with the same draws):
// branch-free for direct moves and captures that cannot continue; the rarer
// plies are deferred as in play_ply_sched (kNeedMen / kNeedKing) or played by
// ply_eps_greedy's enumeration.
template <class Rng>
GA_HD int play_ply_eps_sched(Board &b, Rng &rs, bool men_now, bool king_now) {
  Side s;
  make_side(b, s);
  const uint32_t men = s.own & ~s.ownK;
  const uint32_t m01 = s.turn ? s.ownK : s.own;
  const uint32_t m23 = s.turn ? s.own : s.ownK;
  const uint32_t J0 = m01 & s.jd[0], J1 = m01 & s.jd[1], J2 = m23 & s.jd[2], J3 = m23 & s.jd[3];
  const bool capture = (J0 | J1 | J2 | J3) != 0;
  const uint32_t jall = s.jd[0] | s.jd[1] | s.jd[2] | s.jd[3];
  const uint32_t jf = s.turn ? (s.jd[2] | s.jd[3]) : (s.jd[0] | s.jd[1]);
  const uint32_t lm = jump2<0>(J0 & men) | jump2<1>(J1 & men) | jump2<2>(J2 & men) | jump2<3>(J3 & men);
  const uint32_t lk = jump2<0>(J0 & s.ownK) | jump2<1>(J1 & s.ownK) | jump2<2>(J2 & s.ownK) |
                      jump2<3>(J3 & s.ownK);
  const uint32_t cont_k = lk & jall, cont_m = lm & jf;
  if (cont_k | cont_m) {
    if (cont_k ? play_forced_king_chain(b, s, J0, J1, J2, J3) : play_forced_men_multi(b, s, J0, J1, J2, J3))
      return 1;
    if (cont_k && !king_now) return kNeedKing;
    if (!cont_k && !men_now) return kNeedMen;
    return ply_eps_greedy(b, rs);
  }
  const uint32_t M[4] = {capture ? J0 : (m01 & step<3>(s.empty)), capture ? J1 : (m01 & step<2>(s.empty)),
                         capture ? J2 : (m23 & step<1>(s.empty)), capture ? J3 : (m23 & step<0>(s.empty))};
  const int n = popc(M[0]) + popc(M[1]) + popc(M[2]) + popc(M[3]);
  if (n == 0) return 0;
  uint32_t B[4];
  eps_best(b, s, capture, M, B);
  uint32_t S0 = M[0], S1 = M[1], S2 = M[2], S3 = M[3], idx = 0;
  if (n >= 2) {
    const bool uniform = rs.next() < kEpsThreshold;
    const uint32_t ties = (uint32_t)(popc(B[0]) + popc(B[1]) + popc(B[2]) + popc(B[3]));
    const uint32_t cnt = uniform ? (uint32_t)n : ties;
    S0 = uniform ? S0 : B[0];
    S1 = uniform ? S1 : B[1];
    S2 = uniform ? S2 : B[2];
    S3 = uniform ? S3 : B[3];
    if (cnt >= 2) idx = mulhi_index(rs.next(), cnt);
  }
  int from, to;
  uint32_t removed;
  nth_move(S0, S1, S2, S3, idx, capture, men, from, to, removed);
  apply_move(b, from, to, removed);
  return n;
}

// ------------------------------------------------------------ reference heuristic, one step per move

// The reference-heuristic ply (the move and the draws of ply_ref_heuristic)
// for plies where no capture can continue: the ply's four material weights are
// computed once (direct moves: with or without promotion; single jumps: a man
// or a king captured, with or without promotion), then one loop step per move
// in list order adds the move's noise (two draws) and keeps the first
// maximum.  A cursor walks the source squares in order and each square's
// directions in search order (men's captures dc = -1 first).  The loop runs
// loop_n(n) >= n steps; steps past the ply's own moves do nothing, so the
// lanes of a warp can run one common trip count, and refill() before every
// even step keeps a ring of draws filled for the two draws per step.  Plies
// where a capture can continue are deferred (kNeedMen / kNeedKing) or played
// by ply_ref_heuristic with `more`, a source of draws that never runs dry.
template <class Rng, class More, class LoopN, class Refill>
GA_HD int play_ply_heur_sched(Board &b, Rng &rs, More &more, bool men_now, bool king_now, LoopN &&loop_n,
                              Refill &&refill) {
  Side s;
  make_side(b, s);
  const uint32_t men = s.own & ~s.ownK;
  const uint32_t m01 = s.turn ? s.ownK : s.own;
  const uint32_t m23 = s.turn ? s.own : s.ownK;
  const uint32_t J0 = m01 & s.jd[0], J1 = m01 & s.jd[1], J2 = m23 & s.jd[2], J3 = m23 & s.jd[3];
  const bool capture = (J0 | J1 | J2 | J3) != 0;
  const uint32_t jall = s.jd[0] | s.jd[1] | s.jd[2] | s.jd[3];
  const uint32_t jf = s.turn ? (s.jd[2] | s.jd[3]) : (s.jd[0] | s.jd[1]);
  const uint32_t lm = jump2<0>(J0 & men) | jump2<1>(J1 & men) | jump2<2>(J2 & men) | jump2<3>(J3 & men);
  const uint32_t lk = jump2<0>(J0 & s.ownK) | jump2<1>(J1 & s.ownK) | jump2<2>(J2 & s.ownK) |
                      jump2<3>(J3 & s.ownK);
  const uint32_t cont_k = lk & jall, cont_m = lm & jf;
  if (cont_k | cont_m) {
    if (cont_k ? play_forced_king_chain(b, s, J0, J1, J2, J3) : play_forced_men_multi(b, s, J0, J1, J2, J3))
      return 1;
    if (cont_k && !king_now) return kNeedKing;
    if (!cont_k && !men_now) return kNeedMen;
    return ply_ref_heuristic(b, more);
  }
  const uint32_t M0 = capture ? J0 : (m01 & step<3>(s.empty)), M1 = capture ? J1 : (m01 & step<2>(s.empty));
  const uint32_t M2 = capture ? J2 : (m23 & step<1>(s.empty)), M3 = capture ? J3 : (m23 & step<0>(s.empty));
  const int n = popc(M0) + popc(M1) + popc(M2) + popc(M3);
  if (n == 0) return 0;
  const int ownScore = popc(s.own) + 3 * popc(s.ownK);
  const int oppScore = popc(s.opp) + 3 * popc(s.opp & b.kings);
  // weights: [promotes][captured piece is a king]; direct moves capture nothing
  const int dm = capture ? 1 : 0, dk = capture ? 4 : 0;
  const int32_t w00 = heur_weight_q16(ownScore, oppScore - dm), w01 = heur_weight_q16(ownScore, oppScore - dk);
  const int32_t w10 = heur_weight_q16(ownScore + 3, oppScore - dm), w11 = heur_weight_q16(ownScore + 3, oppScore - dk);
  // a man moving from these squares promotes (a step or a jump towards the far row)
  const uint32_t promo = capture ? (s.turn ? 0x00000F00u : 0x00F00000u) : (s.turn ? 0x000000F0u : 0x0F000000u);
  const uint32_t oppK = s.opp & b.kings;
  int best_sq = -1, best_d = 0;
  if (n == 1) {  // one move, no draws
    best_sq = ctz(M0 | M1 | M2 | M3);
    best_d = (int)ctz((((M0 >> best_sq) & 1u) | (((M1 >> best_sq) & 1u) << 1) | (((M2 >> best_sq) & 1u) << 2) |
                       (((M3 >> best_sq) & 1u) << 3)));
  } else {
    uint32_t rest = M0 | M1 | M2 | M3;  // source squares still to visit
    int sq = 0;
    uint32_t dbits = 0;  // directions of sq still to visit, in search order
    bool rev = false;    // dbits holds a man's captures: bit 0 is dc = -1
    int32_t bw = 0;
    const uint32_t steps = loop_n((uint32_t)n);
    for (uint32_t k = 0; k < steps; k++) {
      if ((k & 1u) == 0) refill();
      if (k >= (uint32_t)n) continue;
      if (dbits == 0) {
        sq = ctz(rest);
        rest &= rest - 1u;
        const uint32_t x0 = (M0 >> sq) & 1u, x1 = (M1 >> sq) & 1u, x2 = (M2 >> sq) & 1u, x3 = (M3 >> sq) & 1u;
        rev = capture && ((men >> sq) & 1u);
        // a man's captures: P1 searches D1 then D0, P2 D3 then D2
        dbits = rev ? (s.turn ? (x3 | (x2 << 1)) : (x1 | (x0 << 1))) : (x0 | (x1 << 1) | (x2 << 2) | (x3 << 3));
      }
      const uint32_t j = (0x12131210u >> (2u * dbits)) & 3u;  // lowest set bit of the 4-bit set
      dbits &= dbits - 1u;
      const int d = rev ? (s.turn ? 3 - (int)j : 1 - (int)j) : (int)j;
      const uint32_t pr = ((promo & men) >> sq) & 1u;
      const int mid = sq + step_off(sq, d);
      const uint32_t ck = capture ? (oppK >> mid) & 1u : 0u;
      int32_t w = pr ? (ck ? w11 : w10) : (ck ? w01 : w00);
      const uint32_t x = rs.next();
      const uint32_t y = rs.next();
      w += heur_noise_q16(x, y);
      if (best_sq < 0 || w > bw) {
        best_sq = sq;
        best_d = d;
        bw = w;
      }
    }
  }
  const int mid = best_sq + step_off(best_sq, best_d);
  const int to = capture ? best_sq + jump_off(best_d) : mid;
  apply_move(b, best_sq, to, capture ? 1u << mid : 0u);
  return n;
}

template <int POLICY, class Rng>
GA_HD int ply(Board &b, Rng &rs) {
  if (POLICY == 1) return ply_ref_heuristic(b, rs);
  if (POLICY == 2) return ply_eps_greedy(b, rs);
  return ply_random(b, rs);
}

}  // namespace ga
