// match.cpp -- game match: GPU MCTS against the reference's mcts_host.
//
// TEST / MEASUREMENT INFRASTRUCTURE (links the CPU oracle).  The opponent is
// the reference's mcts_host player, MCTSPlayer(50, 0, t, HostPlayoutDriver)
// (src/player.cpp:162-163), rebuilt from parts checked against the
// reference: the project's GameTree in the reference's UCB1 mode (statistics
// identical to src/mcts.cpp's GameTree) and the oracle's restatement of
// HostPlayoutDriver (src/playout.cpp:17-32, rand() % n over the reference move
// list on all host threads).  Both players search concurrently, as in the
// reference's game_test (src/driver.cpp:177-264), with the same time per move.
//
//   match -n GAMES --ms-per-move T [-a PLAYER] [--seed S]
//
// Colours alternate; the line "RESULT {json}" reports wins/draws/losses of
// the GPU player and the 95% Wilson interval of its score.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>

#include "../gpu_ai_gb300/csrc/host/player.hpp"
#include "../oracle/oracle.h"

using namespace gpuai;

namespace {

// HostPlayoutDriver, restated in the oracle.
class OracleHostDriver : public PlayoutDriver {
 public:
  std::vector<PlayerId> runPlayouts(std::vector<State> states) override {
    std::vector<PlayerId> out(states.size());
    if (states.empty()) return out;
    std::vector<or_board16> b(states.size());
    for (size_t i = 0; i < states.size(); i++) b[i] = or_board16{states[i].b.p1, states[i].b.p2, states[i].b.kings, states[i].b.meta};
    std::vector<int8_t> r(states.size());
    or_host_playouts(b.data(), (uint32_t)b.size(), r.data(), 0, seed_++);
    for (size_t i = 0; i < r.size(); i++) out[i] = r[i] > 0 ? PLAYER_1 : (r[i] < 0 ? PLAYER_2 : PLAYER_NONE);
    return out;
  }
  std::string getName() const override { return "host"; }

 private:
  unsigned seed_ = 1;
};

std::unique_ptr<Player> mcts_host(unsigned ms) {
  MCTSConfig cfg;
  cfg.initialNumPlayouts = 50;
  cfg.numPlayoutsScale = 0.0f;
  cfg.maxBatch = 50;
  cfg.timeoutMs = ms;
  cfg.perspective = GameTree::Perspective::ChildToMove;
  return std::make_unique<MCTSPlayer>(cfg, std::make_unique<OracleHostDriver>());
}

PlayerId play(Player *p[2], unsigned max_plies) {
  State s = getStartingState();
  for (int i = 0; i < 2; i++) p[i]->start();
  unsigned plies = 0;
  while (!s.isGameOver() && plies < max_plies) {
    const Move m = p[s.turn()]->getMove(s, false);
    for (int i = 0; i < 2; i++) p[i]->move(m);
    s.move(m);
    plies++;
  }
  for (int i = 0; i < 2; i++) p[i]->stop();
  return s.isGameOver() ? s.getWinner() : PLAYER_NONE;
}

}  // namespace

int main(int argc, char **argv) {
  unsigned games = 10, ms = 100, max_plies = 400;
  std::string gpu = "mcts_device_multiple";
  uint64_t seed = 1;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    if (a == "-n" && i + 1 < argc) games = (unsigned)std::stoul(argv[++i]);
    else if (a == "--ms-per-move" && i + 1 < argc) ms = (unsigned)std::stoul(argv[++i]);
    else if (a == "-a" && i + 1 < argc) gpu = argv[++i];
    else if (a == "--seed" && i + 1 < argc) seed = std::stoull(argv[++i]);
    else if (a == "--max-plies" && i + 1 < argc) max_plies = (unsigned)std::stoul(argv[++i]);
    else { std::cerr << "usage: match -n GAMES --ms-per-move T [-a PLAYER] [--seed S]\n"; return 1; }
  }
  unsigned win = 0, draw = 0, loss = 0;
  uint64_t gpu_playouts = 0;
  for (unsigned g = 0; g < games; g++) {
    std::unique_ptr<Player> a = getPlayer(gpu, ms, 0, seed + g);
    std::unique_ptr<Player> h = mcts_host(ms);
    const int gpu_side = (int)(g % 2);
    Player *p[2];
    p[gpu_side] = a.get();
    p[1 - gpu_side] = h.get();
    const PlayerId w = play(p, max_plies);
    if (w == PLAYER_NONE) draw++;
    else if ((int)w == gpu_side) win++;
    else loss++;
    if (auto *m = dynamic_cast<MCTSPlayer *>(a.get())) gpu_playouts += m->playoutsRun();
    std::cout << "game " << g << ": gpu plays " << (gpu_side ? "Player 2" : "Player 1") << ", "
              << (w == PLAYER_NONE ? "draw" : ((int)w == gpu_side ? "gpu won" : "host won")) << std::endl;
  }
  const double n = games, score = (win + 0.5 * draw) / (n > 0 ? n : 1);
  const double z = 1.96, den = 1 + z * z / n;
  const double centre = (score + z * z / (2 * n)) / den;
  const double half = z * std::sqrt(score * (1 - score) / n + z * z / (4 * n * n)) / den;
  std::printf("RESULT {\"games\": %u, \"ms_per_move\": %u, \"gpu_player\": \"%s\", \"wins\": %u, \"draws\": %u, "
              "\"losses\": %u, \"score\": %.4f, \"ci95\": [%.4f, %.4f], \"gpu_playouts\": %llu}\n",
              games, ms, gpu.c_str(), win, draw, loss, score, centre - half, centre + half,
              (unsigned long long)gpu_playouts);
  return 0;
}
