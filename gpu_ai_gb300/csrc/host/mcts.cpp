// mcts.cpp -- host UCT tree (see mcts.hpp).
#include "mcts.hpp"

#include <limits>
#include <stdexcept>

namespace gpuai {

GameTree::GameTree(const State &root, Perspective p, double c) : perspective_(p), c_(c) {
  add_node(root, Move{}, -1);
}

int32_t GameTree::add_node(const State &s, const Move &in, int32_t parent) {
  Node nd;
  nd.state = s;
  nd.in_move = in;
  nd.parent = parent;
  nd.terminal = s.isGameOver();
  nodes_.push_back(nd);
  return (int32_t)nodes_.size() - 1;
}

double GameTree::score(int32_t n, PlayerId player) const {
  const Node &nd = nodes_[n];
  if (nd.terminal) {
    const PlayerId w = nd.state.getWinner();
    return w == PLAYER_NONE ? 0.5 : (w == player ? 1.0 : 0.0);
  }
  if (nd.total == 0) return 0.0;
  return (double)nd.wins[player] / nd.total;
}

// UCB1 weight of a child (src/mcts.cpp:182-191): untried children first.
// log_parent = log of the parent's finished playouts, computed once per parent.
double GameTree::ucb1(int32_t child, double log_parent) const {
  const Node &nd = nodes_[child];
  if (nd.total == 0) return std::numeric_limits<double>::infinity();
  if (perspective_ == Perspective::ChildToMove)  // the reference's expression, long double included
    return (double)nd.wins[nd.state.turn()] / nd.total + std::sqrt(2.0L * log_parent / nd.total);
  const PlayerId who = nodes_[nd.parent].state.turn();
  return (double)nd.wins[who] / nd.total + c_ * std::sqrt(log_parent / nd.total);
}

Move GameTree::getOptMove(PlayerId player) const {
  const Node &root = nodes_[0];
  if (!root.expanded || root.nchildren == 0) throw std::runtime_error("getOptMove: the root has not been expanded");
  double best = -std::numeric_limits<double>::infinity();
  int32_t bi = -1;
  for (uint32_t i = 0; i < root.nchildren; i++) {
    const double sc = score(root.first_child + (int32_t)i, player);
    if (sc > best) {
      best = sc;
      bi = root.first_child + (int32_t)i;
    }
  }
  return nodes_[bi].in_move;
}

std::vector<GameTree::ChildStat> GameTree::rootChildren(PlayerId player) const {
  std::vector<ChildStat> out;
  const Node &root = nodes_[0];
  if (!root.expanded) return out;
  for (uint32_t i = 0; i < root.nchildren; i++) {
    const int32_t c = root.first_child + (int32_t)i;
    out.push_back(ChildStat{nodes_[c].in_move, nodes_[c].total, {nodes_[c].wins[0], nodes_[c].wins[1]},
                            nodes_[c].terminal, score(c, player)});
  }
  return out;
}

void GameTree::move(const Move &m) {
  const Node &root = nodes_[0];
  int32_t keep = -1;
  if (root.expanded)
    for (uint32_t i = 0; i < root.nchildren; i++)
      if (nodes_[root.first_child + (int32_t)i].in_move == m) keep = root.first_child + (int32_t)i;
  if (keep < 0) {
    State s = root.state;
    s.move(m);
    nodes_.clear();
    add_node(s, Move{}, -1);
    return;
  }
  // copy the kept subtree breadth-first; children stay contiguous
  std::vector<Node> fresh;
  fresh.reserve(nodes_.size());
  fresh.push_back(nodes_[keep]);
  fresh[0].parent = -1;
  fresh[0].in_move = Move{};
  for (size_t q = 0; q < fresh.size(); q++) {
    if (!fresh[q].expanded) continue;
    const int32_t old_first = fresh[q].first_child;
    fresh[q].first_child = (int32_t)fresh.size();
    for (uint32_t i = 0; i < fresh[q].nchildren; i++) {
      Node c = nodes_[old_first + (int32_t)i];
      c.parent = (int32_t)q;
      fresh.push_back(c);
    }
  }
  nodes_.swap(fresh);
}

std::vector<State> GameTree::select(unsigned trials) {
  std::vector<State> out;
  out.reserve(trials);
  select_rec(0, trials, out);
  return out;
}

void GameTree::select_rec(int32_t n, unsigned trials, std::vector<State> &out) {
  if (trials == 0) {
    nodes_[n].assigned = 0;
    return;
  }
  // a finished game: every slot plays out from it (src/mcts.cpp:65-68)
  if (nodes_[n].terminal) {
    nodes_[n].assigned = trials;
    for (unsigned t = 0; t < trials; t++) out.push_back(nodes_[n].state);
    return;
  }
  if (!nodes_[n].expanded) {
    if (trials > 1) {  // expand: one child per legal move, in move order
      const std::vector<Move> moves = nodes_[n].state.getMoves();
      const int32_t first = (int32_t)nodes_.size();
      for (const Move &m : moves) {
        State s = nodes_[n].state;
        s.move(m);
        add_node(s, m, n);
      }
      nodes_[n].first_child = first;
      nodes_[n].nchildren = (uint32_t)moves.size();
      nodes_[n].expanded = true;
    } else {
      nodes_[n].assigned = trials;
      if (trials == 1) out.push_back(nodes_[n].state);
      return;
    }
  }
  const int32_t first = nodes_[n].first_child;
  const uint32_t nc = nodes_[n].nchildren;
  // per-child weights and shares; a position has at most 64 legal moves
  double w[64];
  unsigned give[64];
  bool extra[64];
  if (nc > 64) throw std::logic_error("select: more than 64 children");
  double wsum = 0;
  unsigned untried = 0;
  const double log_parent = nodes_[n].total ? std::log((double)nodes_[n].total) : 0.0;
  for (uint32_t i = 0; i < nc; i++) {
    w[i] = ucb1(first + (int32_t)i, log_parent);
    wsum += w[i];
    if (nodes_[first + (int32_t)i].total == 0) untried++;
    give[i] = 0;
    extra[i] = false;
  }
  // All weights zero (a parent with one finished playout whose children have
  // not won yet, e.g. a forced move): the proportional split below would be
  // 0/0, so the weights count as equal.
  if (untried == 0 && !(wsum > 0 && std::isfinite(wsum))) {
    for (uint32_t i = 0; i < nc; i++) w[i] = 1.0;
    wsum = (double)nc;
  }
  unsigned assigned = 0;
  for (uint32_t i = 0; i < nc; i++) {
    if (untried > 0) give[i] = nodes_[first + (int32_t)i].total == 0 ? trials / untried : 0;
    else if (trials > 0) give[i] = (unsigned)(trials * (w[i] / wsum));
    assigned += give[i];
  }
  // remaining slots go one each to the heaviest children (src/mcts.cpp:120-136)
  while (assigned < trials) {
    double mw = -std::numeric_limits<double>::infinity();
    int opt = -1;
    for (uint32_t i = 0; i < nc; i++)
      if (!extra[i] && w[i] > mw) {
        mw = w[i];
        opt = (int)i;
      }
    if (opt < 0) throw std::logic_error("select: cannot place the remaining trials");
    extra[opt] = true;
    give[opt]++;
    assigned++;
  }
  nodes_[n].assigned = trials;
  for (uint32_t i = 0; i < nc; i++) select_rec(first + (int32_t)i, give[i], out);
}

void GameTree::update(const std::vector<PlayerId> &results, unsigned playoutsPerLeaf) {
  if (results.size() != (size_t)nodes_[0].assigned * playoutsPerLeaf)
    throw std::invalid_argument("update: result count does not match the last select");
  size_t at = 0;
  update_rec(0, results, at, playoutsPerLeaf);
}

// Adds the outcomes of node n's slots (results[at ...], k per slot, in the
// depth-first order of select) to n and its subtree; returns the wins of
// PLAYER_1 and PLAYER_2 among them and advances `at`.  A leaf's results are
// counted once; inner nodes add their children's counts.
GameTree::Wins GameTree::update_rec(int32_t n, const std::vector<PlayerId> &results, size_t &at, unsigned k) {
  Node &nd = nodes_[n];
  const unsigned cnt = nd.assigned * k;
  Wins w{0, 0};
  if (nd.expanded && !nd.terminal) {
    for (uint32_t i = 0; i < nd.nchildren; i++) {
      const int32_t c = nd.first_child + (int32_t)i;
      if (nodes_[c].assigned) {
        const Wins cw = update_rec(c, results, at, k);
        w.w[0] += cw.w[0];
        w.w[1] += cw.w[1];
      }
    }
  } else {
    for (size_t q = at; q < at + cnt; q++)
      if (results[q] != PLAYER_NONE) w.w[results[q]]++;
    at += cnt;
  }
  Node &me = nodes_[n];  // nodes_ does not grow here, but keep the reference fresh after recursion
  me.total += cnt;
  me.wins[0] += w.w[0];
  me.wins[1] += w.w[1];
  me.assigned = 0;
  return w;
}

}  // namespace gpuai
