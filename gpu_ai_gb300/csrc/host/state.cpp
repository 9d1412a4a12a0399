// state.cpp -- host side of the State / Move interface (see state.hpp).
#include "state.hpp"

#include "../rules.cuh"

#include <cstring>

namespace gpuai {

namespace {
ga::Board to_ga(const gpuai_board &b) { return ga::Board{b.p1, b.p2, b.kings, b.meta}; }
gpuai_board from_ga(const ga::Board &b) { return gpuai_board{b.p1, b.p2, b.kings, b.meta}; }
}  // namespace

uint32_t Move::removed_mask() const {
  uint32_t r = 0;
  for (unsigned i = 0; i < m.jumps && i < 12; i++) r |= 1u << m.removed[i];
  return r;
}

bool Move::operator==(const Move &o) const {
  if (m.from != o.m.from || m.to != o.m.to || m.jumps != o.m.jumps || m.promoted != o.m.promoted) return false;
  for (unsigned i = 0; i < m.jumps && i < 12; i++)
    if (m.removed[i] != o.m.removed[i] || m.path[i] != o.m.path[i]) return false;
  return true;
}

std::vector<Move> State::getMoves() const {
  std::vector<Move> out;
  const ga::Board g = to_ga(b);
  ga::Side s;
  ga::make_side(g, s);
  ga::for_each_move(s, ga::jumpers(s), [&](int from, int to, uint32_t, int jumps, uint32_t dirs) {
    Move mv;
    uint32_t w[8];
    ga::pack_move(g, from, to, jumps, dirs, w);
    std::memcpy(&mv.m, w, sizeof w);
    out.push_back(mv);
    return false;
  });
  return out;
}

void State::move(const Move &mv) {
  ga::Board g = to_ga(b);
  ga::apply_move(g, mv.m.from, mv.m.to, mv.removed_mask());
  b = from_ga(g);
}

bool State::isGameOver() const {
  if (movesSinceLastCapture() >= NUM_DRAW_MOVES) return true;
  const ga::Board g = to_ga(b);
  ga::Side s;
  ga::make_side(g, s);
  return ga::count_moves(s, ga::jumpers(s)) == 0;
}

PlayerId State::getWinner() const {
  return movesSinceLastCapture() < NUM_DRAW_MOVES ? getNextTurn() : PLAYER_NONE;
}

State getStartingState() {
  State s;
  s.b = gpuai_board{0x00000FFFu, 0xFFF00000u, 0u, 0u};
  return s;
}

std::vector<State> genRandomStates(unsigned n, uint64_t seed, unsigned min_plies, unsigned max_plies) {
  std::vector<State> out(n);
  for (unsigned p = 0; p < n; p++) {
    ga::Stream rs;
    rs.init(seed, p, 1);
    ga::Board g{0x00000FFFu, 0xFFF00000u, 0u, 0u};
    const uint32_t np = min_plies + ga::mulhi_index(rs.next(), max_plies - min_plies + 1u);
    for (uint32_t q = 0; q < np; q++) {
      if (((g.meta >> 8) & 0xffu) >= NUM_DRAW_MOVES) break;
      if (ga::ply_random(g, rs) <= 0) break;
    }
    out[p].b = from_ga(g);
  }
  return out;
}

std::ostream &operator<<(std::ostream &os, PlayerId p) {
  switch (p) {
    case PLAYER_1: return os << "Player 1";
    case PLAYER_2: return os << "Player 2";
    default: return os << "Player NONE";
  }
}

std::ostream &operator<<(std::ostream &os, Loc l) {
  return os << (char)('a' + l.col) << (BOARD_SIZE - l.row);
}

std::ostream &operator<<(std::ostream &os, const Move &m) {
  os << m.from() << " to " << m.to();
  if (m.jumps()) {
    if (m.jumps() > 1) {
      os << " via";
      for (unsigned i = 0; i + 1 < m.jumps(); i++) os << " " << m.intermediate(i);
    }
    os << ", captured";
    for (unsigned i = 0; i < m.jumps(); i++) os << " " << m.removed(i);
  }
  if (m.promoted()) os << ", promoted to king";
  return os;
}

std::ostream &operator<<(std::ostream &os, const State &s) {
  os << s.turn() << "'s turn\n";
  for (int r = 0; r < BOARD_SIZE; r++) {
    os << (BOARD_SIZE - r) << " ";
    for (int c = 0; c < BOARD_SIZE; c++) {
      char ch = '.';
      if ((r + c) % 2 == 1) {
        const uint32_t bit = 1u << (r * 4 + c / 2);
        const bool king = (s.b.kings & bit) != 0;
        if (s.b.p1 & bit) ch = king ? 'k' : 'o';
        else if (s.b.p2 & bit) ch = king ? 'K' : 'O';
        else ch = ' ';
      }
      os << ch << ' ';
    }
    os << "\n";
  }
  os << "  a b c d e f g h";
  return os;
}

}  // namespace gpuai
