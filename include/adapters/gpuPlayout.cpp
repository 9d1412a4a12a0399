// gpuPlayout.cpp -- GB300 playouts behind the reference's PlayoutDriver
#include "playout.hpp"
#include "gpuai.h"
#include <cstring>
#include <stdexcept>

namespace {
gpuai_board toBoard(const State &s) {
  gpuai_board b = {0, 0, 0, 0};
  for (int r = 0; r < BOARD_SIZE; r++)
    for (int c = 1 - (r % 2); c < BOARD_SIZE; c += 2) {
      const BoardItem &it = s.board[r][c];
      if (!it.occupied) continue;
      uint32_t bit = 1u << (r * 4 + c / 2);
      (it.owner == PLAYER_1 ? b.p1 : b.p2) |= bit;
      if (it.type == CHECKER_KING) b.kings |= bit;
    }
  unsigned msc = s.movesSinceLastCapture > 255 ? 255 : s.movesSinceLastCapture;
  b.meta = (s.turn == PLAYER_2 ? 1u : 0u) | (msc << 8);
  return b;
}
}  // namespace

class GpuPlayoutDriver : public PlayoutDriver {
public:
  explicit GpuPlayoutDriver(int32_t policy = GPUAI_POLICY_RANDOM, int device = 0) : policy(policy) {
    if (gpuai_create(device, &ctx) != GPUAI_OK) throw std::runtime_error(gpuai_last_error());
  }
  ~GpuPlayoutDriver() { gpuai_destroy(ctx); }

  std::vector<PlayerId> runPlayouts(std::vector<State> states) {
    std::vector<PlayerId> out(states.size());
    if (states.empty()) return out;
    // identical consecutive leaves (GameTree::select returns copies of a
    // terminal or single-trial state) become one board with a repeat count
    std::vector<gpuai_board> pos;
    std::vector<uint32_t> reps;
    for (const State &s : states) {
      gpuai_board b = toBoard(s);
      if (!pos.empty() && memcmp(&pos.back(), &b, sizeof b) == 0) reps.back()++;
      else { pos.push_back(b); reps.push_back(1); }
    }
    std::vector<int8_t> res(states.size());
    if (gpuai_playouts(ctx, pos.data(), reps.data(), pos.size(), seed, next_stream, policy,
                       res.data()) != GPUAI_OK)
      throw std::runtime_error(gpuai_last_error());
    next_stream += states.size();
    for (size_t i = 0; i < res.size(); i++)
      out[i] = res[i] > 0 ? PLAYER_1 : (res[i] < 0 ? PLAYER_2 : PLAYER_NONE);
    return out;
  }
  std::string getName() const {
    return policy == GPUAI_POLICY_RANDOM ? "device_gb300" : "device_gb300_heuristic";
  }

private:
  gpuai_ctx *ctx = nullptr;
  int32_t policy;
  uint64_t seed = 2016, next_stream = 0;
};
