// noalloc.cu -- playouts for callers that cannot allocate device memory.
//
// Some callers of this library are not allowed to call cudaMalloc: a search
// server that reserves the whole device memory budget for its trees up
// front and hands out only sub-buffers of that reservation, or a move loop
// with a hard per-move time limit that must never stall on the allocator.
// gpuai_playouts_noalloc serves them: the caller passes device buffers for the
// boards and outcomes it already owns, and the only other device memory the
// playout kernel needs -- the work counter, status word, ply counter and the
// per-position repetition prefix sums -- lives in the file-scope array
// g_scratch below, which the CUDA runtime places in every device's memory when
// the library is loaded and keeps there until the process exits.
#include "../../include/gpuai.h"
#include "launch.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <mutex>

namespace {

// Largest number of positions one call accepts (the prefix-sum area).
constexpr uint32_t kMaxPositions = GPUAI_NOALLOC_MAX_POSITIONS;
// Word layout: [0] work counter, [1] status, [2..3] ply count, [64 ..] the
// npos+1 prefix sums of the repetitions.
constexpr uint32_t kOffsetsWord = 64;
constexpr uint32_t kScratchWords = kOffsetsWord + kMaxPositions + 1;

static __device__ __align__(256) uint32_t g_scratch[kScratchWords];

constexpr int kMaxDevices = 64;

// Threads per block for each policy: the uniform random policy runs in
// 512-thread blocks, the others in 256-thread blocks (the allocating entry
// point's default launch shapes).
constexpr int kBlock[3] = {2 * ga::kPlayoutBlock, ga::kPlayoutBlock, ga::kPlayoutBlock};

struct DeviceState {
  std::atomic<bool> ready{false};
  uint32_t *scratch = nullptr;  // device address of g_scratch on this device
  int sms = 0;
  int blocks_per_sm[3] = {0, 0, 0};
  std::mutex call;  // one call at a time per device: calls share g_scratch and `offsets`
  // host staging of the repetition prefix sums (static storage: untouched
  // pages cost nothing until a device's first call with repetitions)
  uint32_t offsets[kMaxPositions + 1];
};

DeviceState g_dev[kMaxDevices];
std::mutex g_setup;

int cuda_error(cudaError_t e, const char *what) {
  char buf[256];
  snprintf(buf, sizeof buf, "gpuai_playouts_noalloc: %s: %s", what, cudaGetErrorString(e));
  return ga::record_error(e == cudaErrorMemoryAllocation ? GPUAI_ERR_OOM : GPUAI_ERR_CUDA, buf);
}

// First call on a device, with that device current: the device address of
// g_scratch (the symbol's name is only a host-side stand-in), SM count and
// occupancy of the playout kernels.
int setup(int dev, DeviceState &d) {
  std::lock_guard<std::mutex> lock(g_setup);
  if (d.ready.load(std::memory_order_acquire)) return GPUAI_OK;
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress");
  e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaDeviceGetAttribute");
  for (int policy = 0; policy < 3; policy++) {
    e = ga::playout_occupancy(policy, kBlock[policy], &d.blocks_per_sm[policy]);
    if (e != cudaSuccess) return cuda_error(e, "occupancy query");
    if (d.blocks_per_sm[policy] < 1) d.blocks_per_sm[policy] = 1;
  }
  d.scratch = static_cast<uint32_t *>(p);
  d.ready.store(true, std::memory_order_release);
  return GPUAI_OK;
}

}  // namespace

extern "C" int gpuai_playouts_noalloc(const gpuai_board *d_pos, const uint32_t *reps, uint32_t npos,
                                      uint64_t seed, uint64_t stream_base, int32_t policy, int8_t *d_out,
                                      void *stream) {
  if (npos == 0) return GPUAI_OK;
  if (!d_pos || !d_out) return ga::record_error(GPUAI_ERR_INVALID, "gpuai_playouts_noalloc: NULL buffer");
  if (policy < 0 || policy > 2)
    return ga::record_error(GPUAI_ERR_INVALID, "gpuai_playouts_noalloc: unknown policy");
  if (npos > kMaxPositions) {
    char buf[160];
    snprintf(buf, sizeof buf, "gpuai_playouts_noalloc: %u positions exceed the maximum of %u", npos,
             kMaxPositions);
    return ga::record_error(GPUAI_ERR_INVALID, buf);
  }
  uint64_t total = npos;
  if (reps) {
    total = 0;
    for (uint32_t p = 0; p < npos; p++) total += reps[p];
  }
  if (total > 0x7fffffffull)
    return ga::record_error(GPUAI_ERR_INVALID, "gpuai_playouts_noalloc: more than 2^31-1 playouts");
  if (total == 0) return GPUAI_OK;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return ga::record_error(GPUAI_ERR_NO_DEVICE, "gpuai_playouts_noalloc: device index out of range");
  DeviceState &d = g_dev[dev];
  if (!d.ready.load(std::memory_order_acquire)) {
    int rc = setup(dev, d);
    if (rc != GPUAI_OK) return rc;
  }
  std::lock_guard<std::mutex> lock(d.call);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t *scratch = d.scratch;
  uint32_t *offsets = nullptr;
  if (reps) {
    // all npos+1 prefix sums staged in the device's static host array, one copy
    offsets = scratch + kOffsetsWord;
    uint32_t acc = 0;
    for (uint32_t p = 0; p < npos; p++) {
      d.offsets[p] = acc;
      acc += reps[p];
    }
    d.offsets[npos] = acc;
    e = cudaMemcpyAsync(offsets, d.offsets, (npos + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_error(e, "copy of the repetition prefix sums");
  }
  // the counter, status and ply count keep the previous call's values: clear them
  e = cudaMemsetAsync(scratch, 0, 4 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return cuda_error(e, "clearing the work counter");
  ga::PlayoutArgs a;
  a.pos = reinterpret_cast<const ga::Board *>(d_pos);
  a.offsets = offsets;
  a.npos = npos;
  a.uniform_reps = 1;
  a.total = (uint32_t)total;
  a.seed = seed;
  a.stream_base = stream_base;
  a.out = d_out;
  a.counter = scratch;
  a.status = scratch + 1;
  a.plies = reinterpret_cast<unsigned long long *>(scratch + 2);
  const long long resident = (long long)d.sms * d.blocks_per_sm[policy];
  const long long need = ((long long)total + kBlock[policy] - 1) / kBlock[policy];
  const int grid = (int)(need < resident ? need : resident);
  e = ga::launch_playouts(a, policy, kBlock[policy], grid, s);
  if (e != cudaSuccess) return cuda_error(e, "playout kernel launch");
  uint32_t status = 0;
  e = cudaMemcpyAsync(&status, scratch + 1, sizeof status, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_error(e, "playout kernel");
  if (status)
    return ga::record_error(GPUAI_ERR_LIMIT, "gpuai_playouts_noalloc: playout kernel reported a limit");
  return GPUAI_OK;
}
