// mcts.hpp -- host UCT tree that produces leaf batches for the GPU playouts.
//
// Same interface and batch semantics as the reference's GameTree
// (src/mcts.hpp:12-64, src/mcts.cpp:63-191): select(trials) spreads a whole
// batch of trials over the tree in proportion to UCB1 weights, expanding a
// leaf when it receives more than one trial, and returns the leaf states in
// depth-first order; update(results) takes the outcomes back in the same
// order.  The nodes live in one vector (indices instead of shared_ptr), and
// move() re-roots by copying the kept subtree.
//
// UCB1 perspective: by default a child's win rate is taken for the player who
// made the move into it.  The reference uses the player to move at the child
// (src/mcts.cpp:189), which rates moves by the opponent's wins; pass
// Perspective::ChildToMove to reproduce that (with the reference's exact
// expression, exploration constant fixed at sqrt(2)).
#pragma once

#include <cmath>
#include <vector>

#include "state.hpp"

namespace gpuai {

class GameTree {
 public:
  enum class Perspective { Mover, ChildToMove };

  explicit GameTree(const State &root, Perspective p = Perspective::Mover, double c = std::sqrt(2.0));

  const State &state() const { return nodes_[0].state; }
  unsigned getTotalTrials() const { return nodes_[0].total; }
  size_t size() const { return nodes_.size(); }
  bool expanded() const { return nodes_[0].expanded; }

  // Fraction of finished playouts won by `player` (a finished game: 1 for the
  // winner, 0.5 each for a draw).
  double getScore(PlayerId player) const { return score(0, player); }
  // The root move whose child scores best for `player` (first best on ties).
  Move getOptMove(PlayerId player) const;
  // Per-child statistics of the root: move, finished playouts, score for `player`.
  struct ChildStat { Move move; unsigned trials; unsigned wins[2]; bool terminal; double score; };
  std::vector<ChildStat> rootChildren(PlayerId player) const;

  // Keep the subtree reached by `m` (or start a fresh tree from the position
  // after `m` if the root was never expanded).
  void move(const Move &m);

  // Distribute `trials` leaf slots over the tree; returns one state per slot.
  std::vector<State> select(unsigned trials);
  // Outcomes of the last select, playoutsPerLeaf consecutive results per slot.
  void update(const std::vector<PlayerId> &results, unsigned playoutsPerLeaf = 1);

 private:
  struct Node {
    State state;
    Move in_move;          // move from the parent into this node
    int32_t parent = -1;
    int32_t first_child = -1;
    uint32_t nchildren = 0;
    bool expanded = false;
    bool terminal = false;
    unsigned assigned = 0;  // leaf slots assigned in the last select
    unsigned total = 0;     // finished playouts through this node
    unsigned wins[2] = {0, 0};
  };

  std::vector<Node> nodes_;
  Perspective perspective_;
  double c_;

  int32_t add_node(const State &s, const Move &in, int32_t parent);
  double score(int32_t n, PlayerId player) const;
  struct Wins { unsigned w[2]; };
  double ucb1(int32_t child, double log_parent) const;
  void select_rec(int32_t n, unsigned trials, std::vector<State> &out);
  Wins update_rec(int32_t n, const std::vector<PlayerId> &results, size_t &at, unsigned k);
};

}  // namespace gpuai
