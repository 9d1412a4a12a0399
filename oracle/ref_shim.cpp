// ref_shim.cpp -- C entry points over the reference's own host code.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) against
// the reference's unmodified sources, where they are present, into
// oracle/_ref/libref.so.  It converts the project's 16-byte board records to
// the reference's State (src/state.hpp:119-122) and calls:
//   State::genMoves                       src/state.cu:239-245
//   State::move                           src/state.cu:57-92
//   HostPlayoutDriver::runPlayouts        src/playout.cpp:17-32
//   HostHeuristicPlayoutDriver::runPlayouts src/heuristicPlayout.cpp:12-48
//   GameTree::select / update               src/mcts.cpp:63-191
// The tests use it to pin the plain-C restatement in oracle.c.
#include "state.hpp"
#include "playout.hpp"
#include "mcts.hpp"

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

void sq_rc(int sq, int &r, int &c) {
  r = sq >> 2;
  c = 2 * (sq & 3) + ((r & 1) ? 0 : 1);
}

State from_b16(const uint32_t *b) {
  State s;
  std::memset(&s, 0, sizeof(s));
  for (int sq = 0; sq < 32; sq++) {
    int r, c;
    sq_rc(sq, r, c);
    uint32_t bit = 1u << sq;
    BoardItem &it = s.board[r][c];
    it.occupied = false;
    it.type = CHECKER;
    it.owner = PLAYER_1;
    if (b[0] & bit) { it.occupied = true; it.owner = PLAYER_1; }
    if (b[1] & bit) { it.occupied = true; it.owner = PLAYER_2; }
    if (it.occupied && (b[2] & bit)) it.type = CHECKER_KING;
  }
  s.turn = (b[3] & 1u) ? PLAYER_2 : PLAYER_1;
  s.movesSinceLastCapture = (b[3] >> 8) & 0xffu;
  return s;
}

void to_b16(const State &s, uint32_t *b) {
  b[0] = b[1] = b[2] = 0;
  for (int sq = 0; sq < 32; sq++) {
    int r, c;
    sq_rc(sq, r, c);
    const BoardItem &it = s.board[r][c];
    if (!it.occupied) continue;
    if (it.owner == PLAYER_1) b[0] |= 1u << sq; else b[1] |= 1u << sq;
    if (it.type == CHECKER_KING) b[2] |= 1u << sq;
  }
  unsigned msc = s.movesSinceLastCapture > 255u ? 255u : s.movesSinceLastCapture;
  b[3] = (s.turn == PLAYER_2 ? 1u : 0u) | (msc << 8);
}

int sq_of(Loc l) { return l.row * 4 + l.col / 2; }

void pack(const Move &m, uint8_t *out) {
  std::memset(out, 0xff, 32);
  out[0] = (uint8_t)sq_of(m.from);
  out[1] = (uint8_t)sq_of(m.to);
  out[2] = m.jumps;
  out[3] = m.promoted ? 1 : 0;
  for (int i = 0; i < m.jumps && i < 12; i++) {
    out[4 + i] = (uint8_t)sq_of(m.intermediate[i]);
    out[16 + i] = (uint8_t)sq_of(m.removed[i]);
  }
  out[28] = out[29] = out[30] = out[31] = 0;
}

int8_t outcome(PlayerId p) { return p == PLAYER_1 ? 1 : (p == PLAYER_2 ? -1 : 0); }

}  // namespace

extern "C" {

int ref_sizeof_state() { return (int)sizeof(State); }
int ref_sizeof_move() { return (int)sizeof(Move); }

int ref_genmoves_b16(const uint32_t *b16, uint32_t n, uint8_t *out, uint32_t max_moves,
                     uint8_t *counts) {
  int overflow = 0;
  for (uint32_t i = 0; i < n; i++) {
    State s = from_b16(b16 + 4 * (size_t)i);
    Move moves[MAX_MOVES];
    int k = s.genMoves(moves);
    counts[i] = (uint8_t)k;
    if ((uint32_t)k > max_moves) { overflow = 1; k = (int)max_moves; }
    for (int j = 0; j < k; j++) pack(moves[j], out + 32 * ((size_t)i * max_moves + j));
  }
  return overflow ? -1 : 0;
}

// Apply move number idx of genMoves to the board record in place.
int ref_apply_b16(uint32_t *b16, int idx) {
  State s = from_b16(b16);
  Move moves[MAX_MOVES];
  int k = s.genMoves(moves);
  if (idx < 0 || idx >= k) return -1;
  s.move(moves[idx]);
  to_b16(s, b16);
  return 0;
}

void ref_host_playouts(const uint32_t *b16, uint32_t n, int8_t *out, unsigned seed) {
  std::vector<State> states(n);
  for (uint32_t i = 0; i < n; i++) states[i] = from_b16(b16 + 4 * (size_t)i);
  std::srand(seed);
  HostPlayoutDriver d;
  std::vector<PlayerId> r = d.runPlayouts(states);
  for (uint32_t i = 0; i < n; i++) out[i] = outcome(r[i]);
}

void ref_host_heuristic_playouts(const uint32_t *b16, uint32_t n, int8_t *out) {
  std::vector<State> states(n);
  for (uint32_t i = 0; i < n; i++) states[i] = from_b16(b16 + 4 * (size_t)i);
  HostHeuristicPlayoutDriver d;
  std::vector<PlayerId> r = d.runPlayouts(states);
  for (uint32_t i = 0; i < n; i++) out[i] = outcome(r[i]);
}

// Deterministic stand-in outcome of a playout from a board record, shared
// with the project's tree test so both trees see the same results.
static PlayerId fake_outcome(const uint32_t *b, uint64_t salt) {
  uint64_t x = ((uint64_t)b[0] | ((uint64_t)b[1] << 32)) ^ ((uint64_t)b[2] * 0x9E3779B97F4A7C15ull) ^
               ((uint64_t)b[3] * 0xC2B2AE3D27D4EB4Full) ^ salt;
  x ^= x >> 31; x *= 0x7FB5D329728EA185ull; x ^= x >> 27; x *= 0x81DADEF4BC2DD44Dull; x ^= x >> 33;
  const unsigned r = (unsigned)(x % 7);
  return r < 3 ? PLAYER_1 : (r < 6 ? PLAYER_2 : PLAYER_NONE);
}

// Runs `iters` rounds of select(trials[i]) / update on the reference's
// GameTree from `root`, outcomes from fake_outcome; writes per root child
// {total, wins P1, wins P2} and returns the number of children.
int ref_tree_run(const uint32_t *root, const uint32_t *trials, int iters, uint64_t salt, uint32_t *out,
                 int max_children) {
  GameTree tree(from_b16(root));
  for (int i = 0; i < iters; i++) {
    std::vector<State> leaves = tree.select(trials[i]);
    std::vector<PlayerId> res(leaves.size());
    for (size_t k = 0; k < leaves.size(); k++) {
      uint32_t b[4];
      to_b16(leaves[k], b);
      res[k] = fake_outcome(b, salt);
    }
    tree.update(res);
  }
  // child statistics through the public interface: score() = wins / total
  State s = from_b16(root);
  std::vector<Move> moves = s.getMoves();
  int n = 0;
  for (const Move &m : moves) {
    if (n >= max_children) break;
    std::shared_ptr<GameTree> child = tree.move(m);
    const unsigned total = child->getTotalTrials();
    const bool stats = total > 0 && !child->state.isGameOver();  // getScore is wins/total there
    out[3 * n] = total;
    out[3 * n + 1] = stats ? (uint32_t)(child->getScore(PLAYER_1) * total + 0.5) : 0u;
    out[3 * n + 2] = stats ? (uint32_t)(child->getScore(PLAYER_2) * total + 0.5) : 0u;
    n++;
  }
  return n;
}

}  // extern "C"
