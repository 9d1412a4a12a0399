// capi.cu -- the C ABI of libgpuai (include/gpuai.h).
//
// A context owns one CUDA stream, device buffers that grow on demand, pinned
// host staging and the work counter / status word / ply counter the playout
// kernel uses.  Host-buffer calls stage inputs through pinned memory, launch
// and read back on the context's stream, then synchronise that stream only.
#include "../../include/gpuai.h"
#include "launch.h"

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation)
    return fail(GPUAI_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  return fail(GPUAI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                      \
  do {                                      \
    cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 4096 ? 4096 : bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 4096 ? 4096 : bytes + bytes / 4;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

// Word layout of the context's small device block.
struct Control {
  uint32_t counter;
  uint32_t status;
  unsigned long long plies;
};

}  // namespace

namespace ga {
// Records `msg` as the calling thread's gpuai_last_error() and returns code
// (for entry points defined in other translation units).
int record_error(int code, const char *msg) { return fail(code, "%s", msg); }
}  // namespace ga

struct gpuai_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sms = 0;
  // threads per block by policy: the uniform random kernel runs 512-thread blocks (2 per SM; ~1 % faster
  // than 4 x 256 on 64 x 4,096 batches, equal on large ones: a block packs its games over 16 warps when
  // the work runs out); the 80-register reference-heuristic kernel fits 3 x 256 per SM
  int block[3] = {2 * ga::kPlayoutBlock, ga::kPlayoutBlock, ga::kPlayoutBlock};
  int blocks_per_sm[3] = {0, 0, 0};  // resident blocks per SM used for the grid
  int max_blocks_per_sm[3] = {0, 0, 0};
  int layout[3] = {ga::kLayoutThread, ga::kLayoutThread, ga::kLayoutThread};
  Control *ctl = nullptr;  // device
  Control last_host{};      // control block of the last host-buffer call, as read back
  bool last_was_host = false;
  DevBuf d_in, d_aux;  // staging of host-buffer calls; move lists
  HostBuf h_in;
  std::mutex mu;
};

namespace {

int check_boards(const gpuai_board *pos, uint32_t n) {
  for (uint32_t i = 0; i < n; i++) {
    const gpuai_board &b = pos[i];
    if (b.p1 & b.p2) return fail(GPUAI_ERR_INVALID, "board %u: a square holds both sides' pieces", i);
    if (b.kings & ~(b.p1 | b.p2)) return fail(GPUAI_ERR_INVALID, "board %u: king bit on an empty square", i);
    if (b.meta & ~0xff01u) return fail(GPUAI_ERR_INVALID, "board %u: reserved meta bits set (0x%x)", i, b.meta);
  }
  return GPUAI_OK;
}

int set_device(gpuai_ctx *ctx) {
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  return GPUAI_OK;
}

int grid_for(gpuai_ctx *ctx, int policy, uint32_t total) {
  long long resident = (long long)ctx->sms * ctx->blocks_per_sm[policy];
  const long long per_block = ctx->layout[policy] == ga::kLayoutWarp ? ctx->block[policy] / 32 : ctx->block[policy];
  long long need = ((long long)total + per_block - 1) / per_block;
  long long g = need < resident ? need : resident;
  return (int)(g < 1 ? 1 : g);
}

// Launch on device buffers; ctx->mu held, device current.  ctl is the work
// counter / status / ply block the launch uses; it is zeroed here unless the
// caller has already zeroed it on the stream (zeroed = true).
int launch_device(gpuai_ctx *ctx, const gpuai_board *d_pos, const uint32_t *d_off, uint32_t npos,
                  uint32_t uniform_reps, uint32_t total, uint64_t seed, uint64_t stream_base,
                  int32_t policy, int8_t *d_out, cudaStream_t s, Control *ctl, bool zeroed) {
  if (!zeroed) CK(cudaMemsetAsync(ctl, 0, sizeof(Control), s), "reset work counter");
  ga::PlayoutArgs a;
  a.pos = reinterpret_cast<const ga::Board *>(d_pos);
  a.offsets = d_off;
  a.npos = npos;
  a.uniform_reps = uniform_reps;
  a.total = total;
  a.seed = seed;
  a.stream_base = stream_base;
  a.out = d_out;
  a.counter = &ctl->counter;
  a.status = &ctl->status;
  a.plies = &ctl->plies;
  CK(ga::launch_playouts(a, policy, ctx->block[policy], grid_for(ctx, policy, total), s, ctx->layout[policy]),
     "playout kernel launch");
  return GPUAI_OK;
}

}  // namespace

extern "C" {

const char *gpuai_last_error(void) { return g_last_error.c_str(); }

int gpuai_create(int device, gpuai_ctx **out) {
  if (!out) return fail(GPUAI_ERR_INVALID, "gpuai_create: out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(GPUAI_ERR_NO_DEVICE, "no CUDA device available (%s)",
                e != cudaSuccess ? cudaGetErrorString(e) : "device count 0");
  if (device < 0 || device >= count)
    return fail(GPUAI_ERR_NO_DEVICE, "device %d out of range (%d devices)", device, count);
  gpuai_ctx *ctx = new (std::nothrow) gpuai_ctx;
  if (!ctx) return fail(GPUAI_ERR_OOM, "gpuai_create: host allocation failed");
  ctx->device = device;
  int rc = set_device(ctx);
  if (rc == GPUAI_OK) {
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaGetDeviceProperties");
    else ctx->sms = prop.multiProcessorCount;
  }
  for (int p = 0; rc == GPUAI_OK && p < 3; p++) {
    e = ga::playout_occupancy(p, ctx->block[p], &ctx->max_blocks_per_sm[p]);
    if (e != cudaSuccess) rc = cuda_fail(e, "occupancy query");
    else if (ctx->max_blocks_per_sm[p] < 1) ctx->max_blocks_per_sm[p] = 1;
    ctx->blocks_per_sm[p] = ctx->max_blocks_per_sm[p];
  }
  if (rc == GPUAI_OK) {
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
  }
  if (rc == GPUAI_OK) {
    e = cudaMalloc(&ctx->ctl, sizeof(Control));
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc control block");
  }
  if (rc != GPUAI_OK) {
    gpuai_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return GPUAI_OK;
}

void gpuai_destroy(gpuai_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->d_in.release();
  ctx->d_aux.release();
  ctx->h_in.release();
  if (ctx->ctl) cudaFree(ctx->ctl);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int gpuai_device_info(gpuai_ctx *ctx, int32_t *sms, int32_t *blocks_per_sm, int32_t *block_threads) {
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_device_info: ctx is NULL");
  if (sms) *sms = ctx->sms;
  if (blocks_per_sm) *blocks_per_sm = ctx->blocks_per_sm[0];
  if (block_threads) *block_threads = ctx->block[0];
  return GPUAI_OK;
}

int gpuai_set_launch(gpuai_ctx *ctx, int32_t policy, int32_t block_threads, int32_t blocks_per_sm) {
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_set_launch: ctx is NULL");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_set_launch: unknown policy %d", policy);
  if (!ga::valid_block(block_threads))
    return fail(GPUAI_ERR_INVALID, "gpuai_set_launch: block_threads %d not in {64,128,256,512}", block_threads);
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = set_device(ctx);
  if (rc) return rc;
  int maxb = 0;
  CK(ga::playout_occupancy(policy, block_threads, &maxb, ctx->layout[policy]), "occupancy query");
  if (maxb < 1) return fail(GPUAI_ERR_INVALID, "gpuai_set_launch: block of %d threads cannot be resident", block_threads);
  if (blocks_per_sm < 0) return fail(GPUAI_ERR_INVALID, "gpuai_set_launch: negative blocks_per_sm");
  ctx->block[policy] = block_threads;
  ctx->max_blocks_per_sm[policy] = maxb;
  ctx->blocks_per_sm[policy] = (blocks_per_sm == 0 || blocks_per_sm > maxb) ? maxb : blocks_per_sm;
  return GPUAI_OK;
}

int gpuai_set_layout(gpuai_ctx *ctx, int32_t policy, int32_t layout) {
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_set_layout: ctx is NULL");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_set_layout: unknown policy %d", policy);
  if (layout != GPUAI_LAYOUT_THREAD && layout != GPUAI_LAYOUT_WARP && layout != GPUAI_LAYOUT_POOLED)
    return fail(GPUAI_ERR_INVALID, "gpuai_set_layout: unknown layout %d", layout);
  if (layout == GPUAI_LAYOUT_WARP && policy != GPUAI_POLICY_RANDOM)
    return fail(GPUAI_ERR_INVALID, "gpuai_set_layout: the warp layout plays the uniform random policy only");
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = set_device(ctx);
  if (rc) return rc;
  int maxb = 0;
  CK(ga::playout_occupancy(policy, ctx->block[policy], &maxb, layout), "occupancy query");
  if (maxb < 1) return fail(GPUAI_ERR_INVALID, "gpuai_set_layout: the kernel cannot be resident");
  ctx->layout[policy] = layout;
  ctx->max_blocks_per_sm[policy] = maxb;
  ctx->blocks_per_sm[policy] = maxb;
  return GPUAI_OK;
}

int gpuai_get_layout(gpuai_ctx *ctx, int32_t policy, int32_t *layout) {
  if (!ctx || !layout) return fail(GPUAI_ERR_INVALID, "gpuai_get_layout: NULL");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_get_layout: unknown policy %d", policy);
  *layout = ctx->layout[policy];
  return GPUAI_OK;
}

int gpuai_get_launch(gpuai_ctx *ctx, int32_t policy, int32_t *block_threads, int32_t *blocks_per_sm,
                     int32_t *max_blocks_per_sm) {
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_get_launch: ctx is NULL");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_get_launch: unknown policy %d", policy);
  if (block_threads) *block_threads = ctx->block[policy];
  if (blocks_per_sm) *blocks_per_sm = ctx->blocks_per_sm[policy];
  if (max_blocks_per_sm) *max_blocks_per_sm = ctx->max_blocks_per_sm[policy];
  return GPUAI_OK;
}

int gpuai_playouts(gpuai_ctx *ctx, const gpuai_board *pos, const uint32_t *reps, uint32_t npos,
                   uint64_t seed, uint64_t stream_base, int32_t policy, int8_t *out) {
  GPUAI_RANGE("gpuai_playouts");
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_playouts: ctx is NULL");
  if (npos == 0) return GPUAI_OK;
  if (!pos || !out) return fail(GPUAI_ERR_INVALID, "gpuai_playouts: NULL buffer");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_playouts: unknown policy %d", policy);
  int rc = check_boards(pos, npos);
  if (rc) return rc;
  uint64_t total = 0;
  if (reps) {
    for (uint32_t p = 0; p < npos; p++) total += reps[p];
  } else {
    total = npos;
  }
  if (total > 0x7fffffffull) return fail(GPUAI_ERR_INVALID, "gpuai_playouts: %llu playouts exceed 2^31-1",
                                         (unsigned long long)total);
  if (total == 0) return GPUAI_OK;

  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((rc = set_device(ctx))) return rc;
  cudaStream_t s = ctx->stream;
  // Device layout [boards | offsets | control | outcomes]: the control block
  // (work counter, status, plies) travels zeroed with the inputs in one copy
  // from pinned staging; the outcomes are copied straight into the caller's
  // buffer (a device-to-host copy into pageable memory is as fast as into
  // pinned memory on a coherent CPU-GPU link, and spares a host memcpy).
  // Equal repetitions (or none) need no offsets: the kernel divides instead.
  uint32_t uniform = 1;
  if (reps) {
    uniform = reps[0];
    for (uint32_t p = 1; p < npos && uniform; p++)
      if (reps[p] != uniform) uniform = 0;
    if (uniform) reps = nullptr;
  }
  const size_t bytes_pos = sizeof(gpuai_board) * (size_t)npos;
  const size_t bytes_off = reps ? sizeof(uint32_t) * ((size_t)npos + 1) : 0;
  const size_t ctl_at = (bytes_pos + bytes_off + 15) & ~(size_t)15;
  const size_t out_at = ctl_at + sizeof(Control);
  const size_t bytes_all = out_at + (size_t)total;
  CK(ctx->h_in.reserve(out_at), "pinned staging");
  CK(ctx->d_in.reserve(bytes_all), "device buffer");
  char *h = static_cast<char *>(ctx->h_in.p);
  char *d = static_cast<char *>(ctx->d_in.p);
  std::memcpy(h, pos, bytes_pos);
  if (reps) {
    uint32_t *h_off = reinterpret_cast<uint32_t *>(h + bytes_pos);
    h_off[0] = 0;
    for (uint32_t p = 0; p < npos; p++) h_off[p + 1] = h_off[p] + reps[p];
  }
  std::memset(h + bytes_pos + bytes_off, 0, out_at - (bytes_pos + bytes_off));
  CK(cudaMemcpyAsync(d, h, out_at, cudaMemcpyHostToDevice, s), "H2D boards");
  Control *d_ctl = reinterpret_cast<Control *>(d + ctl_at);
  rc = launch_device(ctx, reinterpret_cast<const gpuai_board *>(d),
                     reps ? reinterpret_cast<const uint32_t *>(d + bytes_pos) : nullptr, npos, uniform, (uint32_t)total,
                     seed, stream_base, policy, reinterpret_cast<int8_t *>(d + out_at), s, d_ctl, true);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, d + out_at, (size_t)total, cudaMemcpyDeviceToHost, s), "D2H outcomes");
  CK(cudaMemcpyAsync(h + ctl_at, d + ctl_at, sizeof(Control), cudaMemcpyDeviceToHost, s), "D2H status");
  CK(cudaStreamSynchronize(s), "playout kernel");
  Control ctl_h;
  std::memcpy(&ctl_h, h + ctl_at, sizeof ctl_h);
  ctx->last_host = ctl_h;
  ctx->last_was_host = true;
  if (ctl_h.status)
    return fail(GPUAI_ERR_LIMIT, "playout kernel status 0x%x (capture depth / ply limit)", ctl_h.status);
  return GPUAI_OK;
}

int gpuai_playouts_device(gpuai_ctx *ctx, const gpuai_board *d_pos, const uint32_t *d_offsets,
                          uint32_t npos, uint32_t uniform_reps, uint32_t total, uint64_t seed,
                          uint64_t stream_base, int32_t policy, int8_t *d_out, void *stream) {
  GPUAI_RANGE("gpuai_playouts_device");
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_playouts_device: ctx is NULL");
  if (total == 0) return GPUAI_OK;
  if (npos == 0 || !d_pos || !d_out) return fail(GPUAI_ERR_INVALID, "gpuai_playouts_device: empty or NULL input");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_playouts_device: unknown policy %d", policy);
  if (total > 0x7fffffffu) return fail(GPUAI_ERR_INVALID, "gpuai_playouts_device: total exceeds 2^31-1");
  if (!d_offsets && (uniform_reps == 0 || (uint64_t)uniform_reps * npos != total))
    return fail(GPUAI_ERR_INVALID, "gpuai_playouts_device: total != npos * uniform_reps");
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
  ctx->last_was_host = false;
  return launch_device(ctx, d_pos, d_offsets, npos, uniform_reps, total, seed, stream_base, policy,
                       d_out, s, ctx->ctl, false);
}

int gpuai_status(gpuai_ctx *ctx, uint32_t *status, uint64_t *plies) {
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_status: ctx is NULL");
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = set_device(ctx);
  if (rc) return rc;
  Control c;
  CK(cudaDeviceSynchronize(), "synchronise before status read");
  if (ctx->last_was_host) c = ctx->last_host;
  else CK(cudaMemcpy(&c, ctx->ctl, sizeof c, cudaMemcpyDeviceToHost), "D2H status");
  if (status) *status = c.status;
  if (plies) *plies = c.plies;
  return GPUAI_OK;
}

int gpuai_genmoves(gpuai_ctx *ctx, const gpuai_board *pos, uint32_t n, gpuai_move *out,
                   uint32_t max_moves, uint8_t *counts) {
  GPUAI_RANGE("gpuai_genmoves");
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_genmoves: ctx is NULL");
  if (n == 0) return GPUAI_OK;
  if (!pos || !out || !counts || max_moves == 0) return fail(GPUAI_ERR_INVALID, "gpuai_genmoves: NULL buffer");
  int rc = check_boards(pos, n);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if ((rc = set_device(ctx))) return rc;
  cudaStream_t s = ctx->stream;
  const size_t bytes_pos = sizeof(gpuai_board) * (size_t)n;
  const size_t bytes_mv = sizeof(gpuai_move) * (size_t)n * max_moves;
  CK(ctx->d_in.reserve(bytes_pos), "device buffer");
  CK(ctx->d_aux.reserve(bytes_mv + n), "device buffer");
  CK(cudaMemcpyAsync(ctx->d_in.p, pos, bytes_pos, cudaMemcpyHostToDevice, s), "H2D boards");
  CK(cudaMemsetAsync(ctx->ctl, 0, sizeof(Control), s), "reset status");
  uint8_t *d_counts = static_cast<uint8_t *>(ctx->d_aux.p) + bytes_mv;
  CK(cudaMemsetAsync(ctx->d_aux.p, 0, bytes_mv, s), "clear move buffer");
  CK(ga::launch_genmoves(static_cast<const ga::Board *>(ctx->d_in.p), n, ctx->d_aux.p, max_moves,
                         d_counts, &ctx->ctl->status, s),
     "genmoves kernel launch");
  Control c;
  CK(cudaMemcpyAsync(out, ctx->d_aux.p, bytes_mv, cudaMemcpyDeviceToHost, s), "D2H moves");
  CK(cudaMemcpyAsync(counts, d_counts, n, cudaMemcpyDeviceToHost, s), "D2H counts");
  CK(cudaMemcpyAsync(&c, ctx->ctl, sizeof c, cudaMemcpyDeviceToHost, s), "D2H status");
  CK(cudaStreamSynchronize(s), "genmoves kernel");
  if (c.status & ga::kStatusDepth) return fail(GPUAI_ERR_LIMIT, "gpuai_genmoves: capture deeper than %d jumps", ga::kMaxDepth);
  if (c.status & ga::kStatusOverflow) return fail(GPUAI_ERR_LIMIT, "gpuai_genmoves: a move list exceeds max_moves=%u", max_moves);
  return GPUAI_OK;
}

int gpuai_random_positions(gpuai_ctx *ctx, uint64_t seed, uint32_t n, uint32_t min_plies,
                           uint32_t max_plies, gpuai_board *out) {
  GPUAI_RANGE("gpuai_random_positions");
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_random_positions: ctx is NULL");
  if (n == 0) return GPUAI_OK;
  if (!out) return fail(GPUAI_ERR_INVALID, "gpuai_random_positions: out is NULL");
  if (min_plies > max_plies) return fail(GPUAI_ERR_INVALID, "gpuai_random_positions: min_plies > max_plies");
  if (max_plies - min_plies == 0xffffffffu) return fail(GPUAI_ERR_INVALID, "gpuai_random_positions: ply range too wide");
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = set_device(ctx);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  const size_t bytes = sizeof(gpuai_board) * (size_t)n;
  CK(ctx->d_aux.reserve(bytes), "device buffer");
  CK(ga::launch_random_positions(seed, n, min_plies, max_plies, static_cast<ga::Board *>(ctx->d_aux.p), s),
     "random positions kernel launch");
  CK(cudaMemcpyAsync(out, ctx->d_aux.p, bytes, cudaMemcpyDeviceToHost, s), "D2H boards");
  CK(cudaStreamSynchronize(s), "random positions kernel");
  return GPUAI_OK;
}

int gpuai_selfplay_positions(gpuai_ctx *ctx, uint64_t seed, uint32_t n, uint32_t min_plies, uint32_t max_plies,
                             int32_t policy, gpuai_board *d_out, void *stream) {
  GPUAI_RANGE("gpuai_selfplay_positions");
  if (!ctx) return fail(GPUAI_ERR_INVALID, "gpuai_selfplay_positions: ctx is NULL");
  if (n == 0) return GPUAI_OK;
  if (!d_out) return fail(GPUAI_ERR_INVALID, "gpuai_selfplay_positions: d_out is NULL");
  if (policy < 0 || policy > 2) return fail(GPUAI_ERR_INVALID, "gpuai_selfplay_positions: unknown policy %d", policy);
  if (min_plies > max_plies || max_plies - min_plies == 0xffffffffu)
    return fail(GPUAI_ERR_INVALID, "gpuai_selfplay_positions: bad ply range");
  std::lock_guard<std::mutex> lock(ctx->mu);
  int rc = set_device(ctx);
  if (rc) return rc;
  CK(ga::launch_random_positions(seed, n, min_plies, max_plies, reinterpret_cast<ga::Board *>(d_out),
                                 static_cast<cudaStream_t>(stream), policy),
     "self-play positions kernel launch");
  return GPUAI_OK;
}

int gpuai_apply_move(const gpuai_board *board, const gpuai_move *move, gpuai_board *out) {
  if (!board || !move || !out) return fail(GPUAI_ERR_INVALID, "gpuai_apply_move: NULL");
  if (move->from >= 32 || move->to >= 32 || move->jumps > 12)
    return fail(GPUAI_ERR_INVALID, "gpuai_apply_move: malformed move record");
  uint32_t removed = 0;
  for (int j = 0; j < move->jumps; j++) {
    if (move->removed[j] >= 32) return fail(GPUAI_ERR_INVALID, "gpuai_apply_move: malformed move record");
    removed |= 1u << move->removed[j];
  }
  const uint32_t mover = (board->meta & 1u) ? board->p2 : board->p1;
  if (!((mover >> move->from) & 1u) || (((board->p1 | board->p2) >> move->to) & 1u && move->to != move->from))
    return fail(GPUAI_ERR_INVALID, "gpuai_apply_move: move does not fit the board");
  ga::Board b{board->p1, board->p2, board->kings, board->meta};
  ga::apply_move(b, move->from, move->to, removed);
  *out = gpuai_board{b.p1, b.p2, b.kings, b.meta};
  return GPUAI_OK;
}

}  // extern "C"
