// host_tree.cpp -- drives the project's host UCT tree (gpu_ai_gb300/csrc/host)
// with a deterministic stand-in for playouts, for CPU tests: the same
// select/update schedule and outcome function as the reference tree runner in
// oracle/ref_shim.cpp, so the two trees' statistics can be compared exactly.
#include "../gpu_ai_gb300/csrc/host/mcts.hpp"
#include "../gpu_ai_gb300/csrc/host/state.hpp"

#include <cstring>

using namespace gpuai;

static PlayerId fake_outcome(const gpuai_board &bb, uint64_t salt) {
  const uint32_t b[4] = {bb.p1, bb.p2, bb.kings, bb.meta};
  uint64_t x = ((uint64_t)b[0] | ((uint64_t)b[1] << 32)) ^ ((uint64_t)b[2] * 0x9E3779B97F4A7C15ull) ^
               ((uint64_t)b[3] * 0xC2B2AE3D27D4EB4Full) ^ salt;
  x ^= x >> 31; x *= 0x7FB5D329728EA185ull; x ^= x >> 27; x *= 0x81DADEF4BC2DD44Dull; x ^= x >> 33;
  const unsigned r = (unsigned)(x % 7);
  return r < 3 ? PLAYER_1 : (r < 6 ? PLAYER_2 : PLAYER_NONE);
}

extern "C" {

// perspective 0 = mover, 1 = the reference's (child to move).  Writes per
// root child {total, wins P1, wins P2} (wins 0 for finished games) and
// returns the number of children, -1 on an inconsistency.
int ht_tree_run(const uint32_t *root, const uint32_t *trials, int iters, uint64_t salt, uint32_t *out,
                int max_children, int perspective, uint32_t *leaves_seen) {
  State s;
  s.b = gpuai_board{root[0], root[1], root[2], root[3]};
  GameTree tree(s, perspective ? GameTree::Perspective::ChildToMove : GameTree::Perspective::Mover);
  uint32_t seen = 0;
  for (int i = 0; i < iters; i++) {
    std::vector<State> leaves = tree.select(trials[i]);
    if (leaves.size() != trials[i]) return -1;
    std::vector<PlayerId> res(leaves.size());
    for (size_t k = 0; k < leaves.size(); k++) res[k] = fake_outcome(leaves[k].b, salt);
    tree.update(res);
    seen += (uint32_t)leaves.size();
  }
  if (leaves_seen) *leaves_seen = seen;
  int n = 0;
  for (const GameTree::ChildStat &c : tree.rootChildren(PLAYER_1)) {
    if (n >= max_children) break;
    out[3 * n] = c.trials;
    out[3 * n + 1] = c.terminal ? 0u : c.wins[0];
    out[3 * n + 2] = c.terminal ? 0u : c.wins[1];
    n++;
  }
  if (tree.getTotalTrials() != seen) return -1;
  return n;
}

// Re-rooting keeps the chosen child's statistics: returns its total before
// and after GameTree::move.
int ht_tree_reroot(const uint32_t *root, unsigned trials, int iters, uint64_t salt, uint32_t *before,
                   uint32_t *after) {
  State s;
  s.b = gpuai_board{root[0], root[1], root[2], root[3]};
  GameTree tree(s);
  for (int i = 0; i < iters; i++) {
    std::vector<State> leaves = tree.select(trials);
    std::vector<PlayerId> res(leaves.size());
    for (size_t k = 0; k < leaves.size(); k++) res[k] = fake_outcome(leaves[k].b, salt);
    tree.update(res);
  }
  const Move best = tree.getOptMove(s.turn());
  for (const GameTree::ChildStat &c : tree.rootChildren(s.turn()))
    if (c.move == best) *before = c.trials;
  tree.move(best);
  *after = tree.getTotalTrials();
  State t = s;
  t.move(best);
  return tree.state() == t ? 0 : -1;
}

// A forced move whose only child has one finished, lost playout while the
// parent has one playout in total (reached when an expanding select's update
// was cancelled): every UCB1 weight is zero.  Returns 0 when the next select
// still places all its trials.
int ht_zero_weights(const uint32_t *root) {
  State s;
  s.b = gpuai_board{root[0], root[1], root[2], root[3]};
  if (s.getMoves().size() != 1) return -2;
  GameTree tree(s);
  tree.select(2);  // expands the root; its update is dropped
  std::vector<State> one = tree.select(1);
  tree.update(std::vector<PlayerId>(one.size(), s.getNextTurn()));
  try {
    std::vector<State> l = tree.select(5);
    tree.update(std::vector<PlayerId>(l.size(), PLAYER_NONE));
    return l.size() == 5 ? 0 : -1;
  } catch (const std::exception &) {
    return -1;
  }
}

}  // extern "C"
