// playout.hpp -- the reference's PlayoutDriver interface over the GB300 kernels.
//
// PlayoutDriver is the interface of src/playout.hpp:27-33: a batch of States
// in, one winner per playout out, results in input order, an empty batch
// returns without a launch.  Every driver here runs its playouts in the
// playout kernel through the C ABI; there is no host playout path.  Errors
// are thrown as std::runtime_error (the reference prints and exits).
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "state.hpp"

namespace gpuai {

class PlayoutDriver {
 public:
  virtual ~PlayoutDriver() {}
  virtual std::vector<PlayerId> runPlayouts(std::vector<State>) = 0;
  virtual std::string getName() const = 0;
  // k playouts of every state, results grouped by state (k consecutive per
  // state).  The default replicates the states for runPlayouts.
  virtual std::vector<PlayerId> runPlayoutsRepeated(const std::vector<State> &states, unsigned k);
};

// One libgpuai context (its own CUDA stream) per driver.  Identical
// consecutive states (the tree's select returns copies for multi-trial
// leaves) are sent once with a repetition count.  Each call takes fresh
// random streams: stream ids continue from the previous call.
class DevicePlayoutDriver : public PlayoutDriver {
 public:
  DevicePlayoutDriver(std::string name, int32_t policy, int device = 0, uint64_t seed = 2016);
  ~DevicePlayoutDriver();
  DevicePlayoutDriver(const DevicePlayoutDriver &) = delete;
  DevicePlayoutDriver &operator=(const DevicePlayoutDriver &) = delete;

  std::vector<PlayerId> runPlayouts(std::vector<State> states) override;
  // One call with a repetition count of k for every state (no replication).
  std::vector<PlayerId> runPlayoutsRepeated(const std::vector<State> &states, unsigned k) override;
  // Playouts from already-collapsed positions: reps[i] playouts of states[i].
  std::vector<int8_t> runRepeated(const std::vector<State> &states, const std::vector<uint32_t> &reps);
  std::string getName() const override { return name_; }
  uint64_t playoutsRun() const { return next_stream_; }
  gpuai_ctx *context() const { return ctx_; }

 private:
  std::string name_;
  int32_t policy_;
  uint64_t seed_;
  uint64_t next_stream_ = 0;
  gpuai_ctx *ctx_ = nullptr;
};

// Driver by name (src/playout.cpp:189-223): device, device_single,
// device_multiple, device_coarse (uniform random playouts), device_heuristic
// (the reference heuristic), device_eps_greedy.  The reference's host,
// hybrid and optimal names run playouts on the CPU and are rejected.
std::unique_ptr<PlayoutDriver> getPlayoutDriver(const std::string &name, int device = 0, uint64_t seed = 2016);

}  // namespace gpuai
