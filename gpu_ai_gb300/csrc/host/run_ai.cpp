// run_ai.cpp -- command-line driver with the reference's run modes
// (src/driver.cpp:266-394):
//
//   run_ai -m gen_moves_test -n N            GPU move lists vs host move lists
//   run_ai -m playout_test -n N -1 D1 -2 D2  two playout drivers on the same states
//   run_ai -m game_test -n G -1 P1 -2 P2     G games between two players
//   run_ai -m game -1 P1 -2 P2               one game, printed
//   run_ai -m mcts_bench -n N -1 D1 -2 D2    host UCT searches from N positions with
//                                            GPU leaf batches, per playout driver
//
// Extra options: --seed S (positions and random streams), --ms-per-move T
// (MCTS move time), --device D; for mcts_bench --leaves-min/--leaves-max L
// (leaf slots per batch), --playouts-per-leaf P and --threads T (searches run
// concurrently, one playout driver and CUDA stream each).
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "host/mcts.hpp"
#include "host/player.hpp"
#include "host/playout.hpp"
#include "host/state.hpp"

using namespace gpuai;

namespace {

struct Options {
  std::string mode = "game";
  unsigned n = 0;
  bool n_set = false;
  std::string p1, p2;
  uint64_t seed = 2016;
  unsigned ms_per_move = 1000;
  int device = 0;
  unsigned leaves_min = 16384, leaves_max = 65536, playouts_per_leaf = 4;
  unsigned threads = 0;  // mcts_bench: concurrent searches (0: min(16, hardware threads))
};

void usage(std::ostream &os) {
  os << "usage: run_ai -m {gen_moves_test,playout_test,game_test,game,mcts_bench} [-n N] [-1 X] [-2 Y]\n"
        "              [--seed S] [--ms-per-move T] [--device D]\n"
        "              [--leaves-min L] [--leaves-max L] [--playouts-per-leaf P] [--threads T]\n"
        "  playout drivers: device device_single device_multiple device_coarse device_heuristic\n"
        "                   device_eps_greedy\n"
        "  players: random mcts mcts_device_single mcts_device_multiple mcts_device_coarse\n"
        "           mcts_device_heuristic mcts_device_eps_greedy\n";
}

Options parse(int argc, char **argv) {
  Options o;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto val = [&]() -> std::string {
      if (i + 1 >= argc) throw std::invalid_argument("missing value for " + a);
      return argv[++i];
    };
    if (a == "-h" || a == "--help") { usage(std::cout); std::exit(0); }
    else if (a == "-m" || a == "--mode") o.mode = val();
    else if (a == "-n" || a == "--num_tests") { o.n = (unsigned)std::stoul(val()); o.n_set = true; }
    else if (a == "-1" || a == "--player1") o.p1 = val();
    else if (a == "-2" || a == "--player2") o.p2 = val();
    else if (a == "--seed") o.seed = std::stoull(val());
    else if (a == "--ms-per-move") o.ms_per_move = (unsigned)std::stoul(val());
    else if (a == "--device") o.device = std::stoi(val());
    else if (a == "--leaves-min") o.leaves_min = (unsigned)std::stoul(val());
    else if (a == "--leaves-max") o.leaves_max = (unsigned)std::stoul(val());
    else if (a == "--playouts-per-leaf") o.playouts_per_leaf = (unsigned)std::stoul(val());
    else if (a == "--threads") o.threads = (unsigned)std::stoul(val());
    else throw std::invalid_argument("unknown option " + a);
  }
  if (o.mode != "gen_moves_test" && o.mode != "playout_test" && o.mode != "game_test" && o.mode != "game" &&
      o.mode != "mcts_bench")
    throw std::invalid_argument("Unknown run mode");
  if (o.leaves_min == 0 || o.leaves_max < o.leaves_min || o.playouts_per_leaf == 0)
    throw std::invalid_argument("need 0 < leaves-min <= leaves-max and playouts-per-leaf > 0");
  return o;
}

// random test positions: 1..100 random plies from the start (src/driver.cpp:76-104)
std::vector<State> test_states(unsigned n, uint64_t seed) { return genRandomStates(n, seed, 1, 100); }

int gen_moves_tests(const Options &o) {
  const unsigned n = o.n_set ? o.n : 100000;
  std::vector<State> states = test_states(n, o.seed);
  std::cout << "Testing " << n << " random states have the same moves on the host and device" << std::endl;
  gpuai_ctx *ctx = nullptr;
  if (gpuai_create(o.device, &ctx) != GPUAI_OK) throw std::runtime_error(gpuai_last_error());
  const uint32_t max_moves = 64;
  std::vector<gpuai_board> pos(n);
  for (unsigned i = 0; i < n; i++) pos[i] = states[i].b;
  std::vector<gpuai_move> mv((size_t)n * max_moves);
  std::vector<uint8_t> counts(n);
  const int rc = gpuai_genmoves(ctx, pos.data(), n, mv.data(), max_moves, counts.data());
  gpuai_destroy(ctx);
  if (rc != GPUAI_OK) throw std::runtime_error(gpuai_last_error());
  for (unsigned i = 0; i < n; i++) {
    const std::vector<Move> host = states[i].getMoves();
    bool same = host.size() == counts[i];
    for (size_t k = 0; same && k < host.size(); k++) {
      Move d;
      d.m = mv[(size_t)i * max_moves + k];
      same = d == host[k];
    }
    if (!same) {
      std::cout << "Mismatch in CPU and GPU move lists\n" << states[i] << "\nFailed" << std::endl;
      return 1;
    }
  }
  std::cout << "Passed" << std::endl;
  return 0;
}

std::vector<PlayerId> playout_test(const std::vector<State> &states, PlayoutDriver &d) {
  const auto t1 = std::chrono::high_resolution_clock::now();
  std::vector<PlayerId> r = d.runPlayouts(states);
  const auto t2 = std::chrono::high_resolution_clock::now();
  unsigned w[3] = {0, 0, 0};
  for (PlayerId p : r) w[p == PLAYER_NONE ? 0 : (p == PLAYER_1 ? 1 : 2)]++;
  std::cout << "=== Results ===\nGames drawn: " << w[0] << "\nPlayer 1 wins: " << w[1]
            << "\nPlayer 2 wins: " << w[2]
            << "\nElapsed time: " << std::chrono::duration<double>(t2 - t1).count() << " seconds" << std::endl;
  return r;
}

int playout_tests(const Options &o) {
  const unsigned n = o.n_set ? o.n : 100000;
  const std::string n1 = o.p1.empty() ? "device_multiple" : o.p1, n2 = o.p2.empty() ? "device_coarse" : o.p2;
  std::cout << "Running " << n << " random playouts with " << n1 << " and " << n2 << std::endl;
  std::vector<State> states = test_states(n, o.seed);
  std::unique_ptr<PlayoutDriver> d1 = getPlayoutDriver(n1, o.device, o.seed);
  std::unique_ptr<PlayoutDriver> d2 = getPlayoutDriver(n2, o.device, o.seed + 1);
  d1->runPlayouts(std::vector<State>(states.begin(), states.begin() + (n < 64 ? n : 64)));  // warm up
  std::cout << "Running test 0: " << d1->getName() << "..." << std::endl;
  std::vector<PlayerId> r1 = playout_test(states, *d1);
  std::cout << "\nRunning test 1: " << d2->getName() << "..." << std::endl;
  std::vector<PlayerId> r2 = playout_test(states, *d2);
  unsigned same = 0;
  for (unsigned i = 0; i < n; i++) same += r1[i] == r2[i];
  std::cout << "\nSimilar results: " << (n ? 100.0 * same / n : 0.0) << "%" << std::endl;
  return 0;
}

PlayerId play_game(Player *players[2], bool verbose) {
  State state = getStartingState();
  for (int i = 0; i < 2; i++) players[i]->start();
  while (!state.isGameOver()) {
    if (verbose) std::cout << state << std::endl;
    Player *p = players[state.turn()];
    const Move m = p->getMove(state, verbose);
    if (verbose) std::cout << state.turn() << " moved " << m << "\n" << std::endl;
    for (int i = 0; i < 2; i++) players[i]->move(m);
    state.move(m);
  }
  if (verbose) std::cout << state << std::endl;
  for (int i = 0; i < 2; i++) players[i]->stop();
  const PlayerId w = state.getWinner();
  if (verbose) {
    if (w == PLAYER_NONE) std::cout << "Draw!" << std::endl;
    else std::cout << w << " won!" << std::endl;
  }
  return w;
}

int game_tests(const Options &o, bool single) {
  const std::string n1 = o.p1.empty() ? "mcts" : o.p1, n2 = o.p2.empty() ? "random" : o.p2;
  std::unique_ptr<Player> a = getPlayer(n1, o.ms_per_move, o.device, o.seed);
  std::unique_ptr<Player> b = getPlayer(n2, o.ms_per_move, o.device, o.seed + 7);
  Player *players[2] = {a.get(), b.get()};
  if (single) {
    std::cout << "Playing single game of " << a->getName() << " Player 1 and " << b->getName() << " Player 2"
              << std::endl;
    play_game(players, true);
    return 0;
  }
  const unsigned g = o.n_set ? o.n : 10;
  std::cout << "Playing " << g << " games with " << a->getName() << " Player 1 and " << b->getName()
            << " Player 2" << std::endl;
  unsigned w[3] = {0, 0, 0};
  for (unsigned i = 0; i < g; i++) {
    std::cout << "Playing game " << i << "... " << std::flush;
    const PlayerId r = play_game(players, false);
    std::cout << (r == PLAYER_NONE ? std::string("Draw!") : (r == PLAYER_1 ? "Player 1 won!" : "Player 2 won!"))
              << std::endl;
    w[r == PLAYER_NONE ? 0 : (r == PLAYER_1 ? 1 : 2)]++;
  }
  std::cout << "=== Results ===\nGames drawn: " << w[0] << "\nPlayer 1 wins: " << w[1]
            << "\nPlayer 2 wins: " << w[2] << std::endl;
  return 0;
}

// Host UCT searches as MCTSPlayer's worker runs them (src/player.cpp:134-150):
// select a batch of leaf slots (total trials x 0.05, clamped to
// [leaves_min, leaves_max]), playouts_per_leaf playouts per slot through the
// playout driver, fold the outcomes back; ms_per_move of searching per
// position (10-40 random plies from the start, seeded).  `threads` searches
// run at once, each thread with its own driver (context and CUDA stream), as
// the reference runs one worker thread per MCTSPlayer.  One JSON line per
// driver name: playouts/s over the wall time, and the share of the searching
// threads' time spent inside the driver calls.
int mcts_bench(const Options &o) {
  const unsigned n = o.n_set ? o.n : 32;
  unsigned threads = o.threads;
  if (threads == 0) {
    const unsigned hw = std::thread::hardware_concurrency();
    threads = hw == 0 ? 1 : (hw < 16 ? hw : 16);
  }
  if (threads > n) threads = n;
  const std::vector<State> roots = genRandomStates(n, o.seed, 10, 40);
  std::vector<std::string> names;
  names.push_back(o.p1.empty() ? "device" : o.p1);
  if (!o.p2.empty()) names.push_back(o.p2);
  for (const std::string &name : names) {
    std::vector<std::unique_ptr<PlayoutDriver>> drivers;
    for (unsigned t = 0; t < threads; t++) {
      drivers.push_back(getPlayoutDriver(name, o.device, o.seed + 1000003ull * t));
      drivers.back()->runPlayouts(std::vector<State>(roots.begin(), roots.end()));  // warm up
    }
    struct Acc { uint64_t playouts = 0, batches = 0, leaves = 0, searched = 0; double driver_s = 0, search_s = 0; };
    std::vector<Acc> acc(threads);
    std::atomic<unsigned> next{0};
    std::vector<std::string> errors(threads);
    const auto w0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < threads; t++) {
      pool.emplace_back([&, t] {
        try {
          Acc &a = acc[t];
          for (unsigned i; (i = next.fetch_add(1)) < n;) {
            if (roots[i].isGameOver()) continue;
            a.searched++;
            GameTree tree(roots[i]);
            const auto t0 = std::chrono::steady_clock::now();
            const auto until = t0 + std::chrono::milliseconds(o.ms_per_move);
            while (std::chrono::steady_clock::now() < until) {
              unsigned k = (unsigned)(tree.getTotalTrials() * 0.05);
              k = k < o.leaves_min ? o.leaves_min : (k > o.leaves_max ? o.leaves_max : k);
              const std::vector<State> slots = tree.select(k);
              const auto c0 = std::chrono::steady_clock::now();
              const std::vector<PlayerId> r = drivers[t]->runPlayoutsRepeated(slots, o.playouts_per_leaf);
              a.driver_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count();
              tree.update(r, o.playouts_per_leaf);
              a.playouts += r.size();
              a.leaves += slots.size();
              a.batches++;
            }
            a.search_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
          }
        } catch (const std::exception &e) {
          errors[t] = e.what();
        }
      });
    }
    for (std::thread &th : pool) th.join();
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    for (const std::string &e : errors)
      if (!e.empty()) throw std::runtime_error(e);
    Acc tot;
    for (const Acc &a : acc) {
      tot.playouts += a.playouts; tot.batches += a.batches; tot.leaves += a.leaves; tot.searched += a.searched;
      tot.driver_s += a.driver_s; tot.search_s += a.search_s;
    }
    std::cout << "MCTS_BENCH {\"driver\": \"" << name << "\", \"positions\": " << tot.searched
              << ", \"threads\": " << threads << ", \"ms_per_position\": " << o.ms_per_move
              << ", \"playouts\": " << tot.playouts << ", \"batches\": " << tot.batches
              << ", \"leaves\": " << tot.leaves << ", \"mean_leaves_per_batch\": "
              << (tot.batches ? (double)tot.leaves / tot.batches : 0.0)
              << ", \"playouts_per_leaf\": " << o.playouts_per_leaf << ", \"seconds\": " << wall
              << ", \"playouts_per_s\": " << (wall > 0 ? tot.playouts / wall : 0.0)
              << ", \"search_seconds\": " << tot.search_s << ", \"driver_seconds\": " << tot.driver_s
              << ", \"driver_share\": " << (tot.search_s > 0 ? tot.driver_s / tot.search_s : 0.0)
              << ", \"mean_driver_call_ms\": " << (tot.batches ? 1e3 * tot.driver_s / tot.batches : 0.0) << "}"
              << std::endl;
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  try {
    o = parse(argc, argv);
  } catch (const std::exception &e) {
    std::cerr << e.what() << "\n";
    usage(std::cerr);
    return 1;
  }
  try {
    if (o.mode == "gen_moves_test") return gen_moves_tests(o);
    if (o.mode == "playout_test") return playout_tests(o);
    if (o.mode == "game_test") return game_tests(o, false);
    if (o.mode == "mcts_bench") return mcts_bench(o);
    return game_tests(o, true);
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << std::endl;
    return 2;
  }
}
