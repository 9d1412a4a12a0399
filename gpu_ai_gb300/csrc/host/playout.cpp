// playout.cpp -- PlayoutDriver over the C ABI (see playout.hpp).
#include "playout.hpp"

#include <cstring>
#include <stdexcept>

namespace gpuai {

DevicePlayoutDriver::DevicePlayoutDriver(std::string name, int32_t policy, int device, uint64_t seed)
    : name_(std::move(name)), policy_(policy), seed_(seed) {
  if (gpuai_create(device, &ctx_) != GPUAI_OK) throw std::runtime_error(gpuai_last_error());
}

DevicePlayoutDriver::~DevicePlayoutDriver() { gpuai_destroy(ctx_); }

std::vector<int8_t> DevicePlayoutDriver::runRepeated(const std::vector<State> &states,
                                                     const std::vector<uint32_t> &reps) {
  if (states.size() != reps.size()) throw std::invalid_argument("runRepeated: one repetition count per state");
  uint64_t total = 0;
  for (uint32_t r : reps) total += r;
  std::vector<int8_t> out(total);
  if (total == 0) return out;
  std::vector<gpuai_board> pos(states.size());
  for (size_t i = 0; i < states.size(); i++) pos[i] = states[i].b;
  if (gpuai_playouts(ctx_, pos.data(), reps.data(), (uint32_t)pos.size(), seed_, next_stream_, policy_,
                     out.data()) != GPUAI_OK)
    throw std::runtime_error(gpuai_last_error());
  next_stream_ += total;
  return out;
}

std::vector<PlayerId> DevicePlayoutDriver::runPlayouts(std::vector<State> states) {
  std::vector<PlayerId> out(states.size());
  if (states.empty()) return out;
  std::vector<State> pos;
  std::vector<uint32_t> reps;
  for (const State &s : states) {
    if (!pos.empty() && pos.back() == s) reps.back()++;
    else {
      pos.push_back(s);
      reps.push_back(1);
    }
  }
  const std::vector<int8_t> r = runRepeated(pos, reps);
  for (size_t i = 0; i < r.size(); i++) out[i] = r[i] > 0 ? PLAYER_1 : (r[i] < 0 ? PLAYER_2 : PLAYER_NONE);
  return out;
}

std::vector<PlayerId> PlayoutDriver::runPlayoutsRepeated(const std::vector<State> &states, unsigned k) {
  if (k == 1) return runPlayouts(states);
  std::vector<State> all;
  all.reserve(states.size() * k);
  for (const State &s : states)
    for (unsigned q = 0; q < k; q++) all.push_back(s);
  return runPlayouts(std::move(all));
}

std::vector<PlayerId> DevicePlayoutDriver::runPlayoutsRepeated(const std::vector<State> &states, unsigned k) {
  const std::vector<int8_t> r = runRepeated(states, std::vector<uint32_t>(states.size(), k));
  std::vector<PlayerId> out(r.size());
  for (size_t i = 0; i < r.size(); i++) out[i] = r[i] > 0 ? PLAYER_1 : (r[i] < 0 ? PLAYER_2 : PLAYER_NONE);
  return out;
}

std::unique_ptr<PlayoutDriver> getPlayoutDriver(const std::string &name, int device, uint64_t seed) {
  if (name == "device" || name == "device_single" || name == "device_multiple" || name == "device_coarse")
    return std::make_unique<DevicePlayoutDriver>(name, GPUAI_POLICY_RANDOM, device, seed);
  if (name == "device_heuristic")
    return std::make_unique<DevicePlayoutDriver>(name, GPUAI_POLICY_REF_HEURISTIC, device, seed);
  if (name == "device_eps_greedy")
    return std::make_unique<DevicePlayoutDriver>(name, GPUAI_POLICY_EPS_GREEDY, device, seed);
  if (name == "host" || name == "host_heuristic" || name == "hybrid" || name == "hybrid_heuristic" ||
      name == "optimal" || name == "optimal_heuristic")
    throw std::runtime_error("playout driver '" + name + "' runs playouts on the CPU; this library has none");
  throw std::runtime_error("Unknown playout type");
}

}  // namespace gpuai
