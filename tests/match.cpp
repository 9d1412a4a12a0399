// match.cpp -- game matches: GPU MCTS against the reference's mcts_host, or
// two GPU MCTS players against each other.
//
// TEST / MEASUREMENT INFRASTRUCTURE (links the CPU oracle).  The host opponent
// is the reference's mcts_host player, MCTSPlayer(50, 0, t, HostPlayoutDriver)
// (src/player.cpp:162-163), rebuilt from parts checked against the
// reference: the project's GameTree in the reference's UCB1 mode (statistics
// identical to src/mcts.cpp's GameTree) and the oracle's restatement of
// HostPlayoutDriver (src/playout.cpp:17-32, rand() % n over the reference move
// list on the host threads).  Both players search concurrently, as in the
// reference's game_test (src/driver.cpp:177-264), with the same time per move.
//
//   match -n GAMES --ms-per-move T [-a PLAYER] [-b PLAYER] [--seed S]
//         [--positions N --min-plies A --max-plies B --pos-seed P]
//         [--batch-min M --batch-max X --ppl K] [--parallel G] [--max-game-plies L]
//
// PLAYER is host (mcts_host) or a GPU player: mcts_device_multiple (uniform
// random playouts), mcts_device_heuristic (the reference heuristic),
// mcts_device_eps_greedy (greedy by material and advancement, eps = 0.1).
// GPU players send leaf batches of max(batch-min, min(batch-max, 5% of the
// tree's playouts)) leaf slots with K playouts each.  With --positions, game g
// starts from seeded position (g / 2) mod N (U{A..B} random plies from the
// start, gpuai_random_positions' positions), each played with both colours;
// otherwise from the start.  G games run at once (each with its own players;
// a host player then runs its playouts on hardware threads / G threads).
// The line "RESULT {json}" reports wins/draws/losses of player A, the 95%
// Wilson interval of its score and each side's playouts per second.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../gpu_ai_gb300/csrc/host/player.hpp"
#include "../oracle/oracle.h"

using namespace gpuai;

namespace {

// HostPlayoutDriver, restated in the oracle.
class OracleHostDriver : public PlayoutDriver {
 public:
  explicit OracleHostDriver(int threads, unsigned seed) : threads_(threads), seed_(seed) {}
  std::vector<PlayerId> runPlayouts(std::vector<State> states) override {
    std::vector<PlayerId> out(states.size());
    if (states.empty()) return out;
    std::vector<or_board16> b(states.size());
    for (size_t i = 0; i < states.size(); i++) b[i] = or_board16{states[i].b.p1, states[i].b.p2, states[i].b.kings, states[i].b.meta};
    std::vector<int8_t> r(states.size());
    or_host_playouts(b.data(), (uint32_t)b.size(), r.data(), threads_, seed_++);
    for (size_t i = 0; i < r.size(); i++) out[i] = r[i] > 0 ? PLAYER_1 : (r[i] < 0 ? PLAYER_2 : PLAYER_NONE);
    return out;
  }
  std::string getName() const override { return "host"; }

 private:
  int threads_;
  unsigned seed_;
};

struct Options {
  unsigned games = 10, ms = 100, max_plies = 400, positions = 0, min_plies = 10, max_pos_plies = 40;
  unsigned batch_min = 4096, batch_max = 65536, ppl = 1, parallel = 1;
  std::string a = "mcts_device_multiple", b = "host";
  uint64_t seed = 1, pos_seed = 2016;
  float scale = 0.05f;
};

std::unique_ptr<MCTSPlayer> make_player(const std::string &name, const Options &o, int host_threads, uint64_t seed) {
  MCTSConfig cfg;
  cfg.timeoutMs = o.ms;
  if (name == "host") {
    cfg.initialNumPlayouts = 50;
    cfg.numPlayoutsScale = 0.0f;
    cfg.maxBatch = 50;
    cfg.perspective = GameTree::Perspective::ChildToMove;
    return std::make_unique<MCTSPlayer>(cfg, std::make_unique<OracleHostDriver>(host_threads, (unsigned)seed));
  }
  std::string driver;
  if (name == "mcts_device_multiple" || name == "mcts_device") driver = "device_multiple";
  else if (name == "mcts_device_heuristic") driver = "device_heuristic";
  else if (name == "mcts_device_eps_greedy") driver = "device_eps_greedy";
  else throw std::runtime_error("unknown player " + name);
  cfg.initialNumPlayouts = o.batch_min;
  cfg.numPlayoutsScale = o.scale;
  cfg.maxBatch = o.batch_max;
  cfg.playoutsPerLeaf = o.ppl;
  return std::make_unique<MCTSPlayer>(cfg, getPlayoutDriver(driver, 0, seed));
}

PlayerId play(State s, Player *p[2], unsigned max_plies) {
  for (int i = 0; i < 2; i++) {
    p[i]->setState(s);  // both trees at the game's start position, the one not to move included
    p[i]->start();
  }
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
  Options o;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw std::runtime_error("missing value after " + a);
      return argv[++i];
    };
    if (a == "-n") o.games = (unsigned)std::stoul(next());
    else if (a == "--ms-per-move") o.ms = (unsigned)std::stoul(next());
    else if (a == "-a") o.a = next();
    else if (a == "-b") o.b = next();
    else if (a == "--seed") o.seed = std::stoull(next());
    else if (a == "--max-game-plies" || a == "--max-plies-per-game") o.max_plies = (unsigned)std::stoul(next());
    else if (a == "--positions") o.positions = (unsigned)std::stoul(next());
    else if (a == "--min-plies") o.min_plies = (unsigned)std::stoul(next());
    else if (a == "--max-plies") o.max_pos_plies = (unsigned)std::stoul(next());
    else if (a == "--pos-seed") o.pos_seed = std::stoull(next());
    else if (a == "--batch-min") o.batch_min = (unsigned)std::stoul(next());
    else if (a == "--batch-max") o.batch_max = (unsigned)std::stoul(next());
    else if (a == "--batch-scale") o.scale = std::stof(next());
    else if (a == "--ppl") o.ppl = (unsigned)std::stoul(next());
    else if (a == "--parallel") o.parallel = std::max(1u, (unsigned)std::stoul(next()));
    else {
      std::cerr << "usage: match -n GAMES --ms-per-move T [-a PLAYER] [-b PLAYER] [--seed S] [--positions N "
                   "--min-plies A --max-plies B --pos-seed P] [--batch-min M --batch-max X --ppl K] "
                   "[--parallel G]\n";
      return 1;
    }
  }
  std::vector<or_board16> starts;
  if (o.positions) {
    starts.resize(o.positions);
    or_random_positions(o.pos_seed, o.positions, o.min_plies, o.max_pos_plies, starts.data());
  }
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int host_threads = (int)std::max(1u, hw / o.parallel);
  std::atomic<unsigned> next_game{0};
  std::mutex mu;
  unsigned win = 0, draw = 0, loss = 0;
  uint64_t playouts[2] = {0, 0};
  double seconds[2] = {0, 0};
  auto worker = [&]() {
    for (;;) {
      const unsigned g = next_game.fetch_add(1);
      if (g >= o.games) return;
      State s = getStartingState();
      if (o.positions) {
        const or_board16 &b = starts[(g / 2) % o.positions];
        s.b = gpuai_board{b.p1, b.p2, b.kings, b.meta};
      }
      std::unique_ptr<MCTSPlayer> pa = make_player(o.a, o, host_threads, o.seed + 2 * g);
      std::unique_ptr<MCTSPlayer> pb = make_player(o.b, o, host_threads, o.seed + 2 * g + 1);
      const int a_side = (int)(g % 2);  // A plays PLAYER_1 in even games, PLAYER_2 in odd ones
      Player *p[2];
      p[a_side] = pa.get();
      p[1 - a_side] = pb.get();
      const auto t0 = std::chrono::steady_clock::now();
      const PlayerId w = play(s, p, o.max_plies);
      const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      std::lock_guard<std::mutex> lock(mu);
      if (w == PLAYER_NONE) draw++;
      else if ((int)w == a_side) win++;
      else loss++;
      playouts[0] += pa->playoutsRun();
      playouts[1] += pb->playoutsRun();
      seconds[0] += el;
      seconds[1] += el;
      std::cout << "game " << g << ": A (" << o.a << ") plays " << (a_side ? "Player 2" : "Player 1") << ", "
                << (w == PLAYER_NONE ? "draw" : ((int)w == a_side ? "A won" : "B won")) << std::endl;
    }
  };
  std::vector<std::thread> th;
  for (unsigned t = 0; t < o.parallel; t++) th.emplace_back(worker);
  for (auto &t : th) t.join();
  const double n = o.games, score = (win + 0.5 * draw) / (n > 0 ? n : 1);
  const double z = 1.96, den = 1 + z * z / n;
  const double centre = (score + z * z / (2 * n)) / den;
  const double half = z * std::sqrt(score * (1 - score) / n + z * z / (4 * n * n)) / den;
  // a player searches during the whole game (pondering included): playouts per game-second
  std::printf("RESULT {\"games\": %u, \"ms_per_move\": %u, \"a\": \"%s\", \"b\": \"%s\", \"positions\": %u, "
              "\"min_plies\": %u, \"max_plies\": %u, \"pos_seed\": %llu, \"batch_min\": %u, \"batch_max\": %u, "
              "\"playouts_per_leaf\": %u, \"parallel\": %u, \"host_threads_per_game\": %d, \"wins\": %u, "
              "\"draws\": %u, \"losses\": %u, \"score\": %.4f, \"ci95\": [%.4f, %.4f], \"a_playouts\": %llu, "
              "\"b_playouts\": %llu, \"a_playouts_per_s\": %.4g, \"b_playouts_per_s\": %.4g}\n",
              o.games, o.ms, o.a.c_str(), o.b.c_str(), o.positions, o.min_plies, o.max_pos_plies,
              (unsigned long long)o.pos_seed, o.batch_min, o.batch_max, o.ppl, o.parallel, host_threads, win, draw,
              loss, score, centre - half, centre + half, (unsigned long long)playouts[0],
              (unsigned long long)playouts[1], seconds[0] > 0 ? playouts[0] / seconds[0] : 0.0,
              seconds[1] > 0 ? playouts[1] / seconds[1] : 0.0);
  return 0;
}
