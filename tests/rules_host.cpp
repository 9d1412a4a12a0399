// rules_host.cpp -- host build of the device rules header, for CPU tests only.
//
// gpu_ai_gb300/csrc/rules.cuh is written __host__ __device__; compiling it
// with g++ lets the CPU test suite check the exact code the kernels run
// (move lists, per-ply policies, random streams) against the oracle without
// a GPU.  Nothing in the product loads this library.
#include "../gpu_ai_gb300/csrc/rules.cuh"

#include <cstring>

using namespace ga;

static Board load(const uint32_t *p) { return Board{p[0], p[1], p[2], p[3]}; }

extern "C" {

int rh_genmoves_b16(const uint32_t *pos, uint32_t n, uint8_t *out, uint32_t max_moves,
                    uint8_t *counts) {
  int rc = 0;
  for (uint32_t i = 0; i < n; i++) {
    const Board b = load(pos + 4 * (size_t)i);
    Side s;
    make_side(b, s);
    uint32_t k = 0;
    int c = for_each_move(s, jumpers(s), [&](int from, int to, uint32_t, int jumps, uint32_t dirs) {
      if (k < max_moves) {
        uint32_t w[8];
        pack_move(b, from, to, jumps, dirs, w);
        std::memcpy(out + 32 * ((size_t)i * max_moves + k), w, 32);
      }
      k++;
      return false;
    });
    if (c < 0 || k > max_moves) rc = -1;
    counts[i] = (uint8_t)(k > 255 ? 255 : k);
  }
  return rc;
}

int rh_count_moves(const uint32_t *pos) {
  const Board b = load(pos);
  Side s;
  make_side(b, s);
  return count_moves(s, jumpers(s));
}

// One playout with the kernel's per-ply code; returns the outcome.
int rh_playout(const uint32_t *pos, uint64_t seed, uint64_t id, int policy, uint32_t *plies,
               uint32_t *draws) {
  Board b = load(pos);
  Stream rs;
  rs.init(seed, id, 0);
  uint32_t p = 0;
  int outcome = 0;
  for (;;) {
    if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) { outcome = 0; break; }
    int n = policy == 1 ? ply<1>(b, rs) : (policy == 2 ? ply<2>(b, rs) : ply<0>(b, rs));
    if (n == 0) { outcome = (b.meta & 1u) ? 1 : -1; break; }
    if (n < 0) { outcome = -100; break; }
    p++;
  }
  if (plies) *plies = p;
  if (draws) *draws = rs.k;
  return outcome;
}

// The same playout with the warp loop's schedule (uniform random policy 0,
// reference heuristic 1, eps-greedy 2): Philox blocks generated every fourth
// (every second for eps-greedy) iteration (DrawRing), the reference
// heuristic's per-move loop run for more steps than the ply's moves (as for a
// warp's longest move list) with its own refills, men's multi-jumps and king
// capture searches deferred to their own iterations, as the warp loop does;
// from iteration sparse_from on nothing is deferred (the kernel's schedule for
// a warp left with few games).
int rh_playout_ring(const uint32_t *pos, uint64_t seed, uint64_t id, uint32_t sparse_from, int policy,
                    uint32_t *plies, uint32_t *draws) {
  Board b = load(pos);
  DrawRing rs;
  rs.start(seed, id, 0);
  auto pick = [&](uint32_t n) { return rs.pick(n); };
  uint32_t p = 0;
  int outcome = 0;
  uint32_t pend = 0;
  for (uint32_t it = 0;; ++it) {
    if ((it & (policy == 2 ? 1u : 3u)) == 0) rs.refill();  // eps-greedy takes up to two draws per ply
    const bool sparse = it >= sparse_from;
    const bool men_ok = sparse || (it & (kMenPeriod - 1u)) == kMenPhase;
    const bool king_ok = sparse || (it & (king_period(policy) - 1u)) == kKingPhase;
    if ((pend == 1u && !men_ok) || (pend == 2u && !king_ok)) continue;
    if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) { outcome = 0; break; }
    int n;
    if (policy == 2) {
      n = play_ply_eps_sched(b, rs, men_ok, king_ok);
    } else if (policy == 1) {
      RingOnDemand more{rs};
      n = play_ply_heur_sched(b, rs, more, men_ok, king_ok, [&](uint32_t m) { return m + (uint32_t)(it % 3); },
                              [&] { rs.refill(); });
    } else {
      n = play_ply_sched(b, pick, men_ok, king_ok);
    }
    if (n == kNeedMen || n == kNeedKing) { pend = n == kNeedMen ? 1u : 2u; continue; }
    pend = 0;
    if (n == 0) { outcome = (b.meta & 1u) ? 1 : -1; break; }
    if (n < 0) { outcome = -100; break; }
    p++;
  }
  if (plies) *plies = p;
  if (draws) *draws = rs.k;
  return outcome;
}

void rh_random_positions(uint64_t seed, uint32_t n, uint32_t min_plies, uint32_t max_plies,
                         uint32_t *out) {
  for (uint32_t p = 0; p < n; p++) {
    Stream rs;
    rs.init(seed, p, 1);
    Board b = {0x00000FFFu, 0xFFF00000u, 0u, 0u};
    const uint32_t np = min_plies + mulhi_index(rs.next(), max_plies - min_plies + 1u);
    for (uint32_t q = 0; q < np; q++) {
      if (((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies) break;
      if (ply_random(b, rs) <= 0) break;
    }
    out[4 * p] = b.p1; out[4 * p + 1] = b.p2; out[4 * p + 2] = b.kings; out[4 * p + 3] = b.meta;
  }
}

}  // extern "C"

extern "C" {
// Branch-free eps-greedy ply (play_ply_eps_sched) against the enumerating
// ply_eps_greedy on n pseudo-random boards (any occupancy, kings included,
// seeded splitmix64): same move count, same board after the ply, same draws.
// Returns the number of boards that differ.
// play_ply_sched (every ply allowed) against the depth-first play_ply on n
// pseudo-random boards: same move count, board and draws.  *forced counts the
// boards whose ply was a men's multi-jump with one legal move (played by
// play_forced_men_multi without the men's tree), *forced_king those whose
// ply was a king's continuing capture with one legal move (played by
// play_forced_king_chain without the search).  Returns the number of boards
// that differ.
long rh_random_fast_matches_dfs(uint64_t n, uint64_t seed, uint64_t *forced, uint64_t *forced_king) {
  uint64_t x = seed;
  auto next = [&]() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  long bad = 0;
  uint64_t nf = 0, nk = 0;
  for (uint64_t t = 0; t < n; t++) {
    uint32_t occ = (uint32_t)next() & (uint32_t)next();
    if (t & 1) occ |= (uint32_t)next() & (uint32_t)next();
    const uint32_t side = (uint32_t)next();
    const uint32_t kmask = t % 3 == 0 ? (uint32_t)next() : (t % 3 == 1 ? 0u : (uint32_t)next() & (uint32_t)next());
    const Board b0 = {occ & side, occ & ~side, occ & kmask, (uint32_t)(next() & 1)};
    Board a = b0, c = b0, f = b0;
    DrawRing ra, rc;
    ra.start(seed, t, 0);
    rc.start(seed, t, 0);
    ra.refill();
    rc.refill();
    const int na = play_ply_sched(a, [&](uint32_t m) { return ra.pick(m); }, true, true);
    const int nc = play_ply(c, [&](uint32_t m) { return rc.pick(m); });
    if (na != nc || a.p1 != c.p1 || a.p2 != c.p2 || a.kings != c.kings || a.meta != c.meta || ra.k != rc.k) bad++;
    Side sd;
    make_side(f, sd);
    const uint32_t men = sd.own & ~sd.ownK;
    const uint32_t m01 = sd.turn ? sd.ownK : sd.own, m23 = sd.turn ? sd.own : sd.ownK;
    const uint32_t J0 = m01 & sd.jd[0], J1 = m01 & sd.jd[1], J2 = m23 & sd.jd[2], J3 = m23 & sd.jd[3];
    const uint32_t jall = sd.jd[0] | sd.jd[1] | sd.jd[2] | sd.jd[3];
    const uint32_t jf = sd.turn ? (sd.jd[2] | sd.jd[3]) : (sd.jd[0] | sd.jd[1]);
    const uint32_t lm = jump2<0>(J0 & men) | jump2<1>(J1 & men) | jump2<2>(J2 & men) | jump2<3>(J3 & men);
    const uint32_t lk = jump2<0>(J0 & sd.ownK) | jump2<1>(J1 & sd.ownK) | jump2<2>(J2 & sd.ownK) |
                        jump2<3>(J3 & sd.ownK);
    if ((lm & jf) && !(lk & jall) && play_forced_men_multi(f, sd, J0, J1, J2, J3)) {
      nf++;
      if (nc != 1) bad++;  // the forced path claims a single move
    } else if ((lk & jall) && play_forced_king_chain(f, sd, J0, J1, J2, J3)) {
      nk++;
      if (nc != 1 || f.p1 != c.p1 || f.p2 != c.p2 || f.kings != c.kings || f.meta != c.meta) bad++;
    }
  }
  if (forced) *forced = nf;
  if (forced_king) *forced_king = nk;
  return bad;
}

// One uniform random ply of board b (p1, p2, kings, meta) played by the
// kernels' play_ply_sched and by the depth-first play_ply on the same draws:
// boards after the ply into fast_out / dfs_out, move counts into *n_fast /
// *n_dfs.
void rh_ply_fast_and_dfs(const uint32_t *b, uint64_t seed, uint32_t *fast_out, uint32_t *dfs_out, int *n_fast,
                         int *n_dfs) {
  Board a = load(b), c = load(b);
  DrawRing ra, rc;
  ra.start(seed, 0, 0);
  rc.start(seed, 0, 0);
  ra.refill();
  rc.refill();
  *n_fast = play_ply_sched(a, [&](uint32_t m) { return ra.pick(m); }, true, true);
  *n_dfs = play_ply(c, [&](uint32_t m) { return rc.pick(m); });
  const uint32_t fa[4] = {a.p1, a.p2, a.kings, a.meta}, fc[4] = {c.p1, c.p2, c.kings, c.meta};
  for (int i = 0; i < 4; i++) {
    fast_out[i] = fa[i];
    dfs_out[i] = fc[i];
  }
}

long rh_eps_fast_matches_enum(uint64_t n, uint64_t seed) {
  uint64_t x = seed;
  auto next = [&]() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  long bad = 0;
  for (uint64_t t = 0; t < n; t++) {
    uint32_t occ = (uint32_t)next() & (uint32_t)next();
    if (t & 1) occ |= (uint32_t)next() & (uint32_t)next();
    const uint32_t side = (uint32_t)next();
    const uint32_t kmask = t % 3 == 0 ? (uint32_t)next() : (t % 3 == 1 ? 0u : ~0u);
    const Board b0 = {occ & side, occ & ~side, occ & kmask, (uint32_t)(next() & 1)};
    Board a = b0, c = b0;
    Stream ra, rc;
    ra.init(seed, t, 0);
    rc.init(seed, t, 0);
    const int na = ply_eps_greedy(a, ra);
    const int nc = play_ply_eps_sched(c, rc, true, true);
    if (na != nc || a.p1 != c.p1 || a.p2 != c.p2 || a.kings != c.kings || a.meta != c.meta || ra.k != rc.k) bad++;
  }
  return bad;
}
}

extern "C" {
// play_ply_heur_sched (loop run for n + t % 5 steps) against the enumerating
// ply_ref_heuristic on n pseudo-random boards: same move count, board and
// draws.  Returns the number of boards that differ.
long rh_heur_fast_matches_enum(uint64_t n, uint64_t seed) {
  uint64_t x = seed;
  auto next = [&]() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  long bad = 0;
  for (uint64_t t = 0; t < n; t++) {
    uint32_t occ = (uint32_t)next() & (uint32_t)next();
    if (t & 1) occ |= (uint32_t)next() & (uint32_t)next();
    const uint32_t side = (uint32_t)next();
    const uint32_t kmask = t % 3 == 0 ? (uint32_t)next() : (t % 3 == 1 ? 0u : ~0u);
    const Board b0 = {occ & side, occ & ~side, occ & kmask, (uint32_t)(next() & 1)};
    Board a = b0, c = b0;
    Stream ra, rc;
    ra.init(seed, t, 0);
    rc.init(seed, t, 0);
    const int na = ply_ref_heuristic(a, ra);
    const int nc = play_ply_heur_sched(c, rc, rc, true, true, [&](uint32_t m) { return m + (uint32_t)(t % 5); },
                                       [] {});
    if (na != nc || a.p1 != c.p1 || a.p2 != c.p2 || a.kings != c.kings || a.meta != c.meta || ra.k != rc.k) bad++;
  }
  return bad;
}
}

extern "C" {
// simple_move_masks + nth_move (the network kernels' per-lane move list)
// against for_each_move on n pseudo-random boards: on every board where no
// capture can continue, move i of the masks is move i of the list (from, to,
// captured squares) and the counts agree.  *simple counts those boards,
// *captures the ones among them that capture.  Returns the number of boards
// that differ.
long rh_simple_moves_match_enum(uint64_t n, uint64_t seed, uint64_t *simple, uint64_t *captures) {
  uint64_t x = seed;
  auto next = [&]() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  long bad = 0;
  uint64_t ns = 0, nc = 0;
  for (uint64_t t = 0; t < n; t++) {
    uint32_t occ = (uint32_t)next() & (uint32_t)next();
    if (t & 1) occ |= (uint32_t)next() & (uint32_t)next();
    const uint32_t side = (uint32_t)next();
    const uint32_t kmask = t % 3 == 0 ? (uint32_t)next() : (t % 3 == 1 ? 0u : (uint32_t)next() & (uint32_t)next());
    const Board b = {occ & side, occ & ~side, occ & kmask, (uint32_t)(next() & 1)};
    Side sd;
    make_side(b, sd);
    uint32_t M[4];
    bool capture = false;
    if (!simple_move_masks(sd, M, capture)) continue;
    ns++;
    nc += capture ? 1u : 0u;
    const int k = popc(M[0]) + popc(M[1]) + popc(M[2]) + popc(M[3]);
    int i = 0;
    bool differ = false;
    const int listed = for_each_move(sd, jumpers(sd), [&](int from, int to, uint32_t removed, int, uint32_t) {
      int f = -1, o = -1;
      uint32_t r = 0;
      if (i < k) nth_move(M[0], M[1], M[2], M[3], (uint32_t)i, capture, sd.own & ~sd.ownK, f, o, r);
      if (f != from || o != to || r != removed) differ = true;
      i++;
      return false;
    });
    if (differ || listed != k) bad++;
  }
  if (simple) *simple = ns;
  if (captures) *captures = nc;
  return bad;
}
}
