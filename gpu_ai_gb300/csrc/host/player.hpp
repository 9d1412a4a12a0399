// player.hpp -- the reference's Player interface (src/player.hpp:20-88).
//
// MCTSPlayer runs the reference's worker loop (src/player.cpp:134-150): a
// background thread repeatedly selects a leaf batch from the UCT tree,
// runs the playouts on the GPU and folds the outcomes back, while getMove
// waits for the move time and returns the best root move.  The move time is
// in milliseconds here (the reference hard-codes seconds).
#pragma once

#include <atomic>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>

#include "mcts.hpp"
#include "playout.hpp"

namespace gpuai {

class Player {
 public:
  virtual ~Player() {}
  virtual std::string getName() const = 0;
  virtual Move getMove(const State &, bool verbose = true) = 0;
  virtual void start() {}
  virtual void stop() {}
  virtual void move(const Move &) {}
  // The game starts from `s` instead of the standard start (the reference's
  // players always start from getStartingState()): a searching player roots
  // its tree there, so that moves passed to move() apply to the right state.
  virtual void setState(const State &) {}
};

// Uniformly random legal move (src/player.cpp:13-16), own seeded generator.
class RandomPlayer : public Player {
 public:
  explicit RandomPlayer(uint64_t seed = 1) : gen_(seed) {}
  std::string getName() const override { return "random"; }
  Move getMove(const State &, bool verbose = true) override;

 private:
  std::mt19937_64 gen_;
};

struct MCTSConfig {
  unsigned initialNumPlayouts = 4096;  // batch size while the tree is small
  float numPlayoutsScale = 0.05f;      // batch = total trials x scale
  unsigned maxBatch = 65536;           // leaf slots per batch, at most
  unsigned playoutsPerLeaf = 1;        // GPU playouts per leaf slot
  unsigned timeoutMs = 1000;           // time per move
  GameTree::Perspective perspective = GameTree::Perspective::Mover;
};

class MCTSPlayer : public Player {
 public:
  MCTSPlayer(MCTSConfig cfg, std::unique_ptr<PlayoutDriver> driver);
  ~MCTSPlayer() override;

  std::string getName() const override { return "mcts_" + driver_->getName(); }
  Move getMove(const State &, bool verbose = true) override;
  void move(const Move &) override;
  void setState(const State &) override;
  void start() override;
  void stop() override;

  uint64_t playoutsRun() const { return playouts_.load(); }
  uint64_t batchesRun() const { return batches_.load(); }

 private:
  MCTSConfig cfg_;
  std::unique_ptr<PlayoutDriver> driver_;
  std::unique_ptr<GameTree> tree_;
  std::mutex mu_;
  std::thread worker_;
  bool updateCancelled_ = false;
  bool running_ = false;
  std::atomic<uint64_t> playouts_{0}, batches_{0};
  std::string error_;

  void worker();
};

// Player by name (src/player.cpp:152-186): random, mcts / mcts_device,
// mcts_device_single, mcts_device_multiple, mcts_device_coarse,
// mcts_device_heuristic, mcts_device_eps_greedy.  The reference's human and
// CPU-playout players are not provided.
std::unique_ptr<Player> getPlayer(const std::string &name, unsigned timeoutMs = 1000, int device = 0,
                                  uint64_t seed = 1);

}  // namespace gpuai
