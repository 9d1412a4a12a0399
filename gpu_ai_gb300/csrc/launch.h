// launch.h -- host-side launchers of the playout kernels (internal to libgpuai).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "rules.cuh"

namespace ga {

// Status bits written by the kernels (atomicOr into the status word).
constexpr uint32_t kStatusDepth = 1u;     // capture sequence deeper than kMaxDepth
constexpr uint32_t kStatusOverflow = 2u;  // move list longer than the caller's buffer
constexpr uint32_t kStatusPlyCap = 4u;    // playout exceeded kMaxPlies (cannot happen under the 50-ply rule)
constexpr uint32_t kStatusBounds = 32u;   // a bounds check of a GPUAI_CHECKS build failed (the access was skipped)

// Bounds checks of the checked build (compiled with -DGPUAI_CHECKS,
// libgpuai_checked.so): GA_IN_BOUNDS(cond, status) is `cond`, and a failed
// check sets kStatusBounds in *status; the caller skips the access.  Warp-
// collective code keeps running on every lane.  In the normal build the
// checks compile to `true`.
#if defined(GPUAI_CHECKS) && defined(__CUDA_ARCH__)
__device__ __forceinline__ bool ga_in_bounds(bool ok, uint32_t *status) {
  if (!ok && status != nullptr) atomicOr(status, kStatusBounds);
  return ok;
}
#define GA_IN_BOUNDS(cond, status) (::ga::ga_in_bounds((cond), (status)))
#else
#define GA_IN_BOUNDS(cond, status) (true)
#endif

constexpr int kPlayoutBlock = 256;        // default threads per block
constexpr uint32_t kMaxPlies = 4096;
// Iterations between block compactions once the work runs out (a power of 2,
// >= 4): 16 for the uniform random policy, 8 for the other two, whose plies
// are longer (measured: 8 is 1.2-1.7 % faster for them, 1.5 % slower for the
// uniform policy on the benchmark batch).
GA_HD constexpr uint32_t compact_period(int policy) { return policy == 0 ? 16u : 8u; }

struct PlayoutArgs {
  const Board *pos;
  const uint32_t *offsets;  // npos+1 prefix sums, or nullptr for uniform repetitions
  uint32_t npos;
  uint32_t uniform_reps;
  uint32_t total;
  uint64_t seed;
  uint64_t stream_base;
  int8_t *out;
  uint32_t *counter;              // work counter, zero before launch
  uint32_t *status;               // status bits, zero before launch
  unsigned long long *plies;      // plies played (optional)
  // Optional: first random-stream id of each position (playout j of position
  // p then uses pos_stream[p] + j - first playout of p); nullptr means
  // stream_base + j.
  const uint64_t *pos_stream = nullptr;
  // Optional: {npos, total} read from device memory at kernel start, for
  // launches inside a CUDA graph whose sizes are computed on the device.
  const uint32_t *dev_sizes = nullptr;
};

// One guided ply of learned-proposal playouts (kernels.cu, proposal_ply_kernel):
// every playout's board advances by one move drawn from the network's policy.
constexpr uint32_t kTagProposal = 2;  // random-stream tag of the guided plies' draws
constexpr int kProposalMaxMoves = 64; // more legal moves than this: uniform choice

struct ProposalArgs {
  const Board *in;            // per position (per_position) or per playout
  const uint32_t *offsets;    // per_position: npos+1 prefix sums, or nullptr for uniform_reps
  uint32_t npos;
  uint32_t uniform_reps;
  uint32_t total;             // playouts
  const uint32_t *dev_sizes;  // optional {npos, total} read at kernel start
  bool per_position;          // input boards and logits rows are per position (first guided ply)
  const uint16_t *logits;     // BF16 bit patterns, 1024 per input row (from * 32 + to)
  uint64_t seed;
  uint64_t stream_base;       // stream of playout j: stream_base + j, unless ...
  const uint64_t *pos_stream; // ... per position first ids (per_position), or
  const uint64_t *play_stream;// ... per playout ids (later plies)
  uint32_t ply;               // guided ply index: the draw index on the proposal stream
  float inv_temperature;
  Board *out;                 // per playout (may equal `in` when !per_position)
  uint64_t *out_stream;       // optional: each playout's stream id
  uint32_t *out_sizes;        // optional: {total, total}
  Board *trace_boards;        // optional: each playout's board before this ply
  uint16_t *trace_logits;     // optional: the logits row each playout used
};
cudaError_t launch_proposal_ply(const ProposalArgs &a, cudaStream_t s);

// Playout layouts: a thread per playout (every policy), a warp per playout
// (uniform random policy only), or a thread per playout whose deferred
// multi-jump plies are gathered in a block pool and played by full warps
// (every policy); the outcomes are the same in all three.
constexpr int kLayoutThread = 0, kLayoutWarp = 1, kLayoutPooled = 2;

// Playout kernels are instantiated for blocks of 64, 128, 256 and 512 threads.
bool valid_block(int block);
// Resident blocks per SM of the playout kernel for `policy` and `block`.
cudaError_t playout_occupancy(int policy, int block, int *blocks_per_sm, int layout = kLayoutThread);
cudaError_t launch_playouts(const PlayoutArgs &a, int policy, int block, int grid, cudaStream_t s,
                            int layout = kLayoutThread);
cudaError_t launch_genmoves(const Board *pos, uint32_t n, void *out, uint32_t max_moves,
                            uint8_t *counts, uint32_t *status, cudaStream_t s);
// Positions after U{min_plies..max_plies} plies of `policy` from the start.
cudaError_t launch_random_positions(uint64_t seed, uint32_t n, uint32_t min_plies,
                                    uint32_t max_plies, Board *out, cudaStream_t s, int policy = 0);

// Sets the calling thread's gpuai_last_error() message; returns code.
int record_error(int code, const char *msg);

// An NVTX range over one C-ABI call (visible in Nsight Systems timelines;
// without a tool attached a push/pop costs a few nanoseconds).
struct ApiRange {
  explicit ApiRange(const char *name) { nvtxRangePushA(name); }
  ~ApiRange() { nvtxRangePop(); }
  ApiRange(const ApiRange &) = delete;
  ApiRange &operator=(const ApiRange &) = delete;
};
#define GPUAI_RANGE(name) ::ga::ApiRange gpuai_api_range_(name)

}  // namespace ga
