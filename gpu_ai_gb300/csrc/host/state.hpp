// state.hpp -- the reference's State / Move / Loc interface on bitboards.
//
// Mirrors src/state.hpp:21-122,253-296 (PlayerId, Loc, State, Move) so that
// host code written against the reference (the UCT tree, players, the
// run_ai driver) reads the same, while the board is the 16-byte record the
// kernels use and the rules are the same rules.cuh code the GPU runs.  Move
// generation here serves tree expansion and players; playouts always run on
// the GPU through PlayoutDriver.
#pragma once

#include <stdint.h>

#include <ostream>
#include <string>
#include <vector>

#include "gpuai.h"

namespace gpuai {

enum PlayerId { PLAYER_1 = 0, PLAYER_2 = 1, PLAYER_NONE = -1 };

constexpr int BOARD_SIZE = 8;
constexpr unsigned NUM_DRAW_MOVES = 50;

// Board coordinates; row 0 is PLAYER_1's back rank (src/state.hpp:34-68).
struct Loc {
  uint8_t row = 0, col = 0;
  Loc() = default;
  Loc(uint8_t r, uint8_t c) : row(r), col(c) {}
  static Loc of_square(int sq) { return Loc((uint8_t)(sq >> 2), (uint8_t)(2 * (sq & 3) + (((sq >> 2) & 1) ? 0 : 1))); }
  int square() const { return row * 4 + col / 2; }
  bool operator==(const Loc &o) const { return row == o.row && col == o.col; }
  bool operator!=(const Loc &o) const { return !(*this == o); }
};

// A move (src/state.hpp:253-296): from, to, captured squares and landing
// squares of each jump, promotion.  Equality compares what the reference's
// Move::operator== compares (src/state.cu:440-454).
struct Move {
  gpuai_move m{};
  Loc from() const { return Loc::of_square(m.from); }
  Loc to() const { return Loc::of_square(m.to); }
  unsigned jumps() const { return m.jumps; }
  bool promoted() const { return m.promoted != 0; }
  Loc removed(unsigned i) const { return Loc::of_square(m.removed[i]); }
  Loc intermediate(unsigned i) const { return Loc::of_square(m.path[i]); }
  uint32_t removed_mask() const;
  bool operator==(const Move &o) const;
  bool operator!=(const Move &o) const { return !(*this == o); }
};

// A position (src/state.hpp:119-250) held as the 16-byte board record.
struct State {
  gpuai_board b{0, 0, 0, 0};

  PlayerId turn() const { return (b.meta & 1u) ? PLAYER_2 : PLAYER_1; }
  unsigned movesSinceLastCapture() const { return (b.meta >> 8) & 0xffu; }
  PlayerId getNextTurn() const { return turn() == PLAYER_1 ? PLAYER_2 : PLAYER_1; }

  // Legal moves in the reference's State::genMoves order.
  std::vector<Move> getMoves() const;
  // Apply a move of the side to move (State::move, src/state.cu:57-92).
  void move(const Move &m);
  // No legal move, or 50 plies without a capture (src/state.cpp:16-18).
  bool isGameOver() const;
  // Winner of a finished game; PLAYER_NONE for a draw (src/state.cpp:20-23).
  PlayerId getWinner() const;

  bool operator==(const State &o) const {
    return b.p1 == o.b.p1 && b.p2 == o.b.p2 && b.kings == o.b.kings && b.meta == o.b.meta;
  }
  bool operator!=(const State &o) const { return !(*this == o); }
};

// The standard start, PLAYER_1 to move (src/state.cpp:25-40).
State getStartingState();

// Seeded positions: position i plays U{min..max} uniformly random plies from
// the start (the project's random streams, tag 1), computed on the host.
std::vector<State> genRandomStates(unsigned n, uint64_t seed, unsigned min_plies, unsigned max_plies);

std::ostream &operator<<(std::ostream &, PlayerId);
std::ostream &operator<<(std::ostream &, Loc);
std::ostream &operator<<(std::ostream &, const Move &);
std::ostream &operator<<(std::ostream &, const State &);

}  // namespace gpuai
