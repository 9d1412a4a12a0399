// player.cpp -- players (see player.hpp).
#include "player.hpp"

#include <chrono>
#include <iostream>
#include <stdexcept>

namespace gpuai {

Move RandomPlayer::getMove(const State &state, bool) {
  const std::vector<Move> moves = state.getMoves();
  if (moves.empty()) throw std::runtime_error("RandomPlayer: no legal move");
  std::uniform_int_distribution<size_t> pick(0, moves.size() - 1);
  return moves[pick(gen_)];
}

MCTSPlayer::MCTSPlayer(MCTSConfig cfg, std::unique_ptr<PlayoutDriver> driver)
    : cfg_(cfg), driver_(std::move(driver)),
      tree_(std::make_unique<GameTree>(getStartingState(), cfg.perspective)) {
  if (cfg_.playoutsPerLeaf == 0) cfg_.playoutsPerLeaf = 1;
}

MCTSPlayer::~MCTSPlayer() {
  if (running_) stop();
}

Move MCTSPlayer::getMove(const State &state, bool verbose) {
  {
    std::lock_guard<std::mutex> lock(mu_);
    if (state != tree_->state()) {
      tree_ = std::make_unique<GameTree>(state, cfg_.perspective);
      updateCancelled_ = true;
    }
  }
  std::this_thread::sleep_for(std::chrono::milliseconds(cfg_.timeoutMs));
  std::lock_guard<std::mutex> lock(mu_);
  if (!error_.empty()) throw std::runtime_error(error_);
  if (!tree_->expanded()) {
    // the worker has not finished a batch on this tree yet: run one small
    // batch here and drop the worker's batch in flight (its select is stale)
    updateCancelled_ = true;
    std::vector<State> leaves = tree_->select(64);
    tree_->update(driver_->runPlayouts(leaves));
  }
  if (verbose) {
    std::cout << "Tree size: " << tree_->getTotalTrials() << " playouts, " << tree_->size() << " nodes" << std::endl;
    for (int p = 0; p < 2; p++)
      std::cout << (PlayerId)p << " score: " << tree_->getScore((PlayerId)p) << std::endl;
  }
  return tree_->getOptMove(state.turn());
}

void MCTSPlayer::move(const Move &m) {
  std::lock_guard<std::mutex> lock(mu_);
  tree_->move(m);
  updateCancelled_ = true;
}

void MCTSPlayer::setState(const State &s) {
  std::lock_guard<std::mutex> lock(mu_);
  tree_ = std::make_unique<GameTree>(s, cfg_.perspective);
  updateCancelled_ = true;  // a batch in flight was selected on the old tree
}

void MCTSPlayer::start() {
  if (running_) throw std::logic_error("MCTSPlayer already started");
  running_ = true;
  worker_ = std::thread(&MCTSPlayer::worker, this);
}

void MCTSPlayer::stop() {
  {
    std::lock_guard<std::mutex> lock(mu_);
    if (!running_) return;
    updateCancelled_ = true;
    running_ = false;
  }
  worker_.join();
}

void MCTSPlayer::worker() {
  std::unique_lock<std::mutex> lock(mu_);
  while (running_) {
    unsigned n = (unsigned)(tree_->getTotalTrials() * cfg_.numPlayoutsScale);
    if (n < cfg_.initialNumPlayouts) n = cfg_.initialNumPlayouts;
    if (n > cfg_.maxBatch) n = cfg_.maxBatch;
    std::vector<State> leaves = tree_->select(n);
    updateCancelled_ = false;
    lock.unlock();
    std::vector<PlayerId> results;
    try {
      results = cfg_.playoutsPerLeaf == 1 ? driver_->runPlayouts(leaves)
                                          : driver_->runPlayoutsRepeated(leaves, cfg_.playoutsPerLeaf);
    } catch (const std::exception &e) {
      lock.lock();
      error_ = e.what();
      running_ = false;
      break;
    }
    playouts_ += results.size();
    batches_++;
    lock.lock();
    if (!updateCancelled_) tree_->update(results, cfg_.playoutsPerLeaf);
    else updateCancelled_ = false;
  }
}

std::unique_ptr<Player> getPlayer(const std::string &name, unsigned timeoutMs, int device, uint64_t seed) {
  if (name == "random") return std::make_unique<RandomPlayer>(seed);
  MCTSConfig cfg;
  cfg.timeoutMs = timeoutMs;
  std::string driver;
  if (name == "mcts" || name == "mcts_device" || name == "mcts_device_single" || name == "mcts_device_multiple") {
    driver = "device_multiple";
  } else if (name == "mcts_device_coarse") {
    driver = "device_coarse";
    cfg.initialNumPlayouts = 16384;
    cfg.numPlayoutsScale = 0.02f;
  } else if (name == "mcts_device_heuristic") {
    driver = "device_heuristic";
  } else if (name == "mcts_device_eps_greedy") {
    driver = "device_eps_greedy";
  } else if (name == "human" || name == "mcts_host" || name == "mcts_host_heuristic" || name == "mcts_hybrid" ||
             name == "mcts_optimal" || name == "mcts_heuristic") {
    throw std::runtime_error("player '" + name + "' is not provided by this library");
  } else {
    throw std::runtime_error("Unknown player type");
  }
  return std::make_unique<MCTSPlayer>(cfg, getPlayoutDriver(driver, device, seed));
}

}  // namespace gpuai
