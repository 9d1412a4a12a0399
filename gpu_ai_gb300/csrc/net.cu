// net.cu -- the policy/value MLP on the sm_103a tensor cores, its training
// kernels, training labels from GPU playouts, and their C ABI (gpuai_net_*,
// gpuai_label_positions).  The reference has no learned evaluation; this is
// the project's own component (its heuristic, src/heuristic.cu:20-49, is the
// only evaluation function there).
//
// Every matrix product is one kernel, gemm_kernel: C = A * B^T with A (M x K)
// and B (N x K) BF16 and K-major in global memory.  A CTA of eight warps
// computes one 128 x BN tile (BN = 64..256): warp 0 streams 64-wide K blocks of
// A and B through a shared-memory ring with TMA (128-byte swizzle), warp 1
// issues tcgen05.mma (M = 128, N = BN, K = 16 per instruction, FP32
// accumulators in TMEM), then all eight warps read the accumulators back
// (warp w owns TMEM lanes 32(w%4).. , i.e. 32 tile rows, and half of the
// columns) and apply a fused epilogue, whose stores go through a per-warp
// staging area in the (by then idle) ring so that every store instruction
// writes whole sectors.  The ring is sized so that two CTAs fit on an SM: one
// CTA's epilogue overlaps the other's loads and MMAs; a product of the
// training chain whose grid is at most one CTA per SM gets twice the ring.
//
// Training step on a batch of B rows (a multiple of 128; rows past n are zero):
//   features      X (B x 192), X^T
//   F1  X  W1^T  -> H1 = bf16(relu(. + b1)), H1^T
//   F2  H1 W2^T  -> H2 = bf16(relu(. + b2)), H2^T, H2 . wv over each 128-column tile
//   F3  H2 W3^T  -> logits = . + b3 (FP32); vraw = the two tiles' sums + bv
//   loss          dZ3 = (softmax - target) / n on the legal (from, to), dZ3^T, dv
//   B1  dZ3 W3   -> dZ2 = bf16((. + dv wv^T) * [H2 > 0]), dZ2^T
//   B3  dZ2 W2   -> dZ1^T = bf16(. * [H1 > 0])
//   B2  dZ3^T H2 -> dW3 partial sums (K = the batch, split over CTAs)
//   B4  dZ2^T H1 -> dW2 partial sums
//   B5  dZ1^T X  -> dW1 partial sums
//   row sums      db1, db2, db3, dwv = H2^T dv, dbv
//   adam          sums the partials in a fixed order, updates the FP32 master
//                 parameters, writes the BF16 copies W1..W3 and W2^T, W3^T
// Every reduction has a fixed order, so a training run is reproducible.
// The chain features .. F3, loss, B1, B3, B5 runs on the network's stream,
// each kernel launched while the one before it drains (programmatic
// dependent launch); B2 and its row sums run on a second stream, B4 and the
// remaining row sums on a third.  dZ3 and dZ3^T are all zero between steps:
// the loss writes at most 32 entries of a row and clear_dz3_kernel zeroes
// them again once B1 and B2 have read them.
#include "net.h"

#include "launch.h"
#include "rules.cuh"
#include "tc.cuh"

#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <vector>
#include <utility>
#include <string>

using bf16 = __nv_bfloat16;

struct gpuai_net {
  int device = 0;
  cudaStream_t stream = nullptr;
  // the backward pass's second and third streams: the products and sums off
  // the critical path overlap the chain loss -> dZ2 -> dZ1 -> dW1 on
  // `stream`; `side` takes dW3, db3, dwv, the loss means and dbv once the loss
  // is known, `side2` dW2 and db2 once dZ2 is, and db1 once dZ1 is
  cudaStream_t side = nullptr, side2 = nullptr;
  cudaEvent_t ev_loss = nullptr, ev_b1 = nullptr, ev_b3 = nullptr, ev_side = nullptr, ev_side2 = nullptr,
              ev_clear = nullptr;
  // dZ3 and dZ3^T hold zeros between steps: the loss kernel writes at most 32
  // entries per row and clear_dz3_kernel zeroes them again once both readers
  // are done.  Set when a step stopped between the two (both are then cleared
  // in full before the next step).
  bool dz_dirty = false;
  uint32_t rows = 0;  // training batch capacity (multiple of 128)
  std::vector<void *> allocs;
  float *params = nullptr, *adam_m = nullptr, *adam_v = nullptr, *grad = nullptr;
  bf16 *W1b = nullptr, *W2b = nullptr, *W3b = nullptr, *W2T = nullptr, *W3T = nullptr;
  CUtensorMap mW1, mW2, mW3, mW2T, mW3T, mW2Tn, mW3Tn, mW2w;  // ..Tn: 64-row boxes; mW2w: 256-row boxes
  uint64_t step = 0;
  ga::net::Fwd fw;
  bf16 *Xt = nullptr, *H1t = nullptr, *H2t = nullptr, *dZ3 = nullptr, *dZ3t = nullptr, *dZ2 = nullptr,
       *dZ2t = nullptr, *dZ1t = nullptr;
  float *dv = nullptr, *rowloss = nullptr, *loss2 = nullptr, *p1 = nullptr, *p2 = nullptr, *p3 = nullptr;
  float *gout = nullptr, *value = nullptr;
  CUtensorMap mXt, mH1t, mH2t, mdZ3, mdZ3t, mdZ2, mdZ2t, mdZ1t;
  uint32_t *status = nullptr;
  gpuai_board *in_boards = nullptr;  // staging for host-buffer calls
  float *in_z = nullptr, *in_q = nullptr;
  // learned-proposal playouts: a forward workspace with BF16 logits and the
  // playouts' boards, grown to the largest call so far
  ga::net::Fwd prop_fw;
  std::vector<void *> prop_allocs;
  ga::Board *prop_cur = nullptr;
  size_t prop_cur_cap = 0;
  // the training step as one CUDA graph (for its batch size, tau and value
  // coefficient), and its kernel nodes whose arguments change from step to
  // step: the ones that read the rows, and Adam's (learning rate, bias
  // corrections)
  cudaGraph_t train_g = nullptr;
  cudaGraphExec_t train_graph = nullptr;
  cudaGraphNode_t node_features = nullptr, node_loss = nullptr, node_clear = nullptr, node_adam = nullptr;
  uint32_t graph_n = 0;
  float graph_tau = 0.0f, graph_vcoef = 0.0f;
  std::mutex mu;
};

namespace ga {
namespace net {
namespace {

enum : uint32_t {
  kEpiBias = 1u,      // + bias[col]
  kEpiRelu = 2u,      // max(., 0)
  kEpiF32 = 4u,       // FP32 row-major store
  kEpiB16 = 8u,       // BF16 row-major store
  kEpiB16T = 16u,     // BF16 transposed store: out_t[col * ld_t + row]
  kEpiMask = 32u,     // * [mask[row][col] > 0] (mask: BF16 ReLU output)
  kEpiRank1 = 64u,    // + r1_row[row] * r1_col[col]
  kEpiVdot = 128u,    // vdot_part[t][row] = sum over columns 128t .. 128t+127 of bf16(.) * vdot_w[col]
  kEpiPartial = 256u, // FP32 row-major store into split-K partial blockIdx.z
  kEpiVsum = 512u     // vdot_out[row] = (vdot_part[0][row] + vdot_part[1][row]) + vdot_b (first column tile)
};

struct Epi {
  uint32_t flags = 0;
  const float *bias = nullptr;
  float *out_f32 = nullptr;
  uint32_t ld_f32 = 0;
  uint64_t partial_stride = 0;
  bf16 *out_b = nullptr;
  uint32_t ld_b = 0;
  bf16 *out_t = nullptr;
  uint32_t ld_t = 0;
  const bf16 *mask = nullptr;
  uint32_t ld_mask = 0;
  const float *r1_row = nullptr, *r1_col = nullptr;
  const float *vdot_w = nullptr, *vdot_b = nullptr;
  float *vdot_out = nullptr;
  float *vdot_part = nullptr;  // [2][vdot_ld] per-tile partial sums of the value head
  uint32_t vdot_ld = 0;
};

struct GemmArgs {
  uint32_t m_rows;        // rows of A (multiple of 128)
  uint32_t bn;            // tile width = MMA N (64, 128, 192 or 256)
  uint32_t tmem_cols;     // TMEM columns allocated (power of two >= bn)
  uint32_t kb_per_split;  // 64-wide K blocks per CTA
  uint32_t stages;        // shared-memory ring depth
  const uint32_t *dev_rows;  // optional device row count: tiles past it do nothing
  uint32_t *status;
  Epi e;
  uint64_t wait_ns;     // limit of every barrier wait (tc::kWaitLimitNs)
  uint32_t skip_loads;  // self-test of the bounded waits: issue no TMA load, so the MMA warp's wait runs out
};

constexpr uint32_t kBM = 128, kBK = 64, kMaxStages = 8;
constexpr uint32_t kThreads = 256;            // 8 warps: two per TMEM lane quadrant in the epilogue
constexpr uint32_t kABytes = kBM * kBK * 2;   // one A stage: 16 KiB
constexpr uint32_t kSmemLimit = 227u * 1024u;
constexpr uint32_t kRingBudget = 100u * 1024u;  // ring size that leaves room for two CTAs per SM
constexpr uint32_t kBarBytes = 256u;  // full[] and empty[] (kMaxStages each), accf, TMEM slot, error flag
constexpr uint32_t kSmemExtra = 1024u + kBarBytes + 1024u;  // alignment slack, barriers, value-head partials
static_assert((2u * kMaxStages + 1u) * 8u + 8u <= kBarBytes, "barriers outgrow their slot");
static_assert(2u * kRingBudget + kSmemExtra <= kSmemLimit, "doubled ring above the shared-memory limit");

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // a in the low half
  return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ float lo_bf(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float hi_bf(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }
__device__ __forceinline__ bool positive_bf(uint32_t h16) { return (h16 & 0x8000u) == 0 && (h16 & 0x7fffu) != 0; }

// Epilogue arithmetic on 32 consecutive columns col0.. of one row (lane's own
// row): bias, rank-1 term, ReLU, ReLU mask.
__device__ __forceinline__ void epilogue_math(const Epi &e, float (&v)[32], uint32_t row, uint32_t col0) {
  const uint32_t f = e.flags;
  if (f & kEpiBias) {  // column vectors are 16-byte aligned: col0 is a multiple of 32
    const float4 *bp = reinterpret_cast<const float4 *>(e.bias + col0);
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float4 t = __ldg(bp + q);
      v[4 * q] += t.x;
      v[4 * q + 1] += t.y;
      v[4 * q + 2] += t.z;
      v[4 * q + 3] += t.w;
    }
  }
  if (f & kEpiRank1) {
    const float r = e.r1_row[row];
    const float4 *cp = reinterpret_cast<const float4 *>(e.r1_col + col0);
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float4 t = __ldg(cp + q);
      v[4 * q] = fmaf(r, t.x, v[4 * q]);
      v[4 * q + 1] = fmaf(r, t.y, v[4 * q + 1]);
      v[4 * q + 2] = fmaf(r, t.z, v[4 * q + 2]);
      v[4 * q + 3] = fmaf(r, t.w, v[4 * q + 3]);
    }
  }
  if (f & kEpiRelu) {
#pragma unroll
    for (int j = 0; j < 32; j++) v[j] = fmaxf(v[j], 0.0f);
  }
  if (f & kEpiMask) {
    const uint4 *mp = reinterpret_cast<const uint4 *>(e.mask + (size_t)row * e.ld_mask + col0);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint4 m = mp[q];
      const uint32_t w[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
      for (int t = 0; t < 4; t++) {
        if (!positive_bf(w[t] & 0xffffu)) v[8 * q + 2 * t] = 0.0f;
        if (!positive_bf(w[t] >> 16)) v[8 * q + 2 * t + 1] = 0.0f;
      }
    }
  }
}

// Per-warp staging area of the epilogue stores (reuses the operand ring once
// the MMAs are done): 32 rows x 36 floats, or 32 rows x 20 words of BF16
// pairs, or 32 columns x 40 BF16 values of the transpose.  The padding keeps
// each row 16-byte aligned and spreads a phase's accesses over the banks.
constexpr uint32_t kStageF32 = 36, kStageB16 = 20, kStageB16T = 40;
constexpr uint32_t kStageBytesPerWarp = 32u * kStageF32 * 4u;  // 4608
constexpr uint32_t kStageBytes = 8u * kStageBytesPerWarp;      // eight warps

// Stores of the 32 x 32 chunk at rows rbase.., columns col0.., whose values
// lane l holds for row rbase + l.  The chunk goes through the warp's staging
// area, so that a store instruction writes whole 32-byte sectors: 4 FP32
// rows x 128 bytes, 8 BF16 rows x 64 bytes, or 8 columns x 64 bytes of the
// BF16 transpose (instead of 16 bytes in each of 32 rows).  Rows >= `rows`
// are not written.  Warp-collective.
__device__ __forceinline__ void epilogue_store(const Epi &e, const float (&v)[32], uint8_t *stage, uint32_t rbase,
                                               uint32_t rows, uint32_t lane, uint32_t col0, uint32_t split,
                                               float &vsum) {
  const uint32_t f = e.flags;
  if (f & (kEpiF32 | kEpiPartial)) {
    float *st = reinterpret_cast<float *>(stage);
#pragma unroll
    for (int q = 0; q < 8; q++)
      reinterpret_cast<float4 *>(st + lane * kStageF32)[q] =
          make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    __syncwarp();
    float *o = e.out_f32 + ((f & kEpiPartial) ? (uint64_t)split * e.partial_stride : 0ull) + col0 + 4u * (lane & 7u);
#pragma unroll
    for (uint32_t k = 0; k < 8; k++) {
      const uint32_t r = 4u * k + (lane >> 3);
      const float4 t = reinterpret_cast<const float4 *>(st + r * kStageF32)[lane & 7u];
      if (rbase + r < rows) *reinterpret_cast<float4 *>(o + (size_t)(rbase + r) * e.ld_f32) = t;
    }
    __syncwarp();
  }
  if (f & (kEpiB16 | kEpiB16T | kEpiVdot)) {
    uint32_t p[16];
#pragma unroll
    for (int t = 0; t < 16; t++) p[t] = pack2(v[2 * t], v[2 * t + 1]);
    if (f & kEpiB16) {
      uint32_t *st = reinterpret_cast<uint32_t *>(stage);
#pragma unroll
      for (int q = 0; q < 4; q++)
        reinterpret_cast<uint4 *>(st + lane * kStageB16)[q] = make_uint4(p[4 * q], p[4 * q + 1], p[4 * q + 2], p[4 * q + 3]);
      __syncwarp();
#pragma unroll
      for (uint32_t k = 0; k < 4; k++) {
        const uint32_t r = 8u * k + (lane >> 2), j = lane & 3u;
        const uint4 t = reinterpret_cast<const uint4 *>(st + r * kStageB16)[j];
        if (rbase + r < rows) reinterpret_cast<uint4 *>(e.out_b + (size_t)(rbase + r) * e.ld_b + col0)[j] = t;
      }
      __syncwarp();
    }
    if (f & kEpiB16T) {
      uint16_t *st = reinterpret_cast<uint16_t *>(stage);  // [column][row]
#pragma unroll
      for (int t = 0; t < 16; t++) {
        st[(2 * t) * kStageB16T + lane] = (uint16_t)(p[t] & 0xffffu);
        st[(2 * t + 1) * kStageB16T + lane] = (uint16_t)(p[t] >> 16);
      }
      __syncwarp();
#pragma unroll
      for (uint32_t k = 0; k < 4; k++) {
        const uint32_t c = 8u * k + (lane >> 2), r0 = 8u * (lane & 3u);
        const uint4 t = *reinterpret_cast<const uint4 *>(st + c * kStageB16T + r0);
        uint16_t *o = reinterpret_cast<uint16_t *>(e.out_t) + (size_t)(col0 + c) * e.ld_t + rbase + r0;
        if (rbase + r0 + 8u <= rows) {
          *reinterpret_cast<uint4 *>(o) = t;
        } else {
          const uint32_t w[4] = {t.x, t.y, t.z, t.w};
          for (uint32_t i = 0; i < 8u && rbase + r0 + i < rows; i++) o[i] = (uint16_t)(w[i >> 1] >> (16u * (i & 1u)));
        }
      }
      __syncwarp();
    }
    if (f & kEpiVdot) {
      const float4 *wp = reinterpret_cast<const float4 *>(e.vdot_w + col0);
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const float4 t = __ldg(wp + q);
        vsum = fmaf(lo_bf(p[2 * q]), t.x, vsum);
        vsum = fmaf(hi_bf(p[2 * q]), t.y, vsum);
        vsum = fmaf(lo_bf(p[2 * q + 1]), t.z, vsum);
        vsum = fmaf(hi_bf(p[2 * q + 1]), t.w, vsum);
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads, 2)
    gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const GemmArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023u) & ~(uintptr_t)1023u);
  const uint32_t bn = g.bn, stage_bytes = kABytes + bn * 128u, nst = g.stages;
  // [ring of nst stages, reused by the epilogue's staging][barriers][value-head partials]
  const uint32_t area = nst * stage_bytes > kStageBytes ? nst * stage_bytes : kStageBytes;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + area);
  uint64_t *empty = full + nst;
  uint64_t *accf = empty + nst;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(accf + 1);
  uint32_t *s_err = tslot + 1;
  float *vpart = reinterpret_cast<float *>(smem + area + kBarBytes);  // [2][128] value-head partial sums
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t row0 = blockIdx.x * kBM;
  tc::grid_dep_wait();  // the operands come from the kernel before this one
  tc::grid_dep_trigger();
  uint32_t rows = g.m_rows;
  if (g.dev_rows) {
    const uint32_t d = *g.dev_rows;
    rows = d < rows ? d : rows;
    if (row0 >= rows) return;  // uniform over the CTA, before any barrier or TMEM use
  }
  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < nst; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accf, 1);
    *s_err = 0;
    tc::fence_mbar_init();
    tc::tma_prefetch_map(&tmA);
    tc::tma_prefetch_map(&tmB);
  }
  if (warp == 2) tc::tmem_alloc(tslot, g.tmem_cols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t nkb = g.kb_per_split, kb0 = blockIdx.z * nkb;
  uint32_t issued = 0;

  if (warp == 0) {
    if (lane == 0 && !g.skip_loads) {  // TMA producer
      for (uint32_t i = 0; i < nkb; i++) {
        const uint32_t s = i % nst;
        if (i >= nst && !tc::mbar_wait(&empty[s], ((i / nst) - 1u) & 1u, g.wait_ns)) {
          atomicOr(s_err, 1u);
          break;
        }
        uint8_t *sa = smem + s * stage_bytes;
        tc::mbar_arrive_expect_tx(&full[s], stage_bytes);
        tc::tma_load_2d(sa, &tmA, &full[s], (int32_t)((kb0 + i) * kBK), (int32_t)row0);
        tc::tma_load_2d(sa + kABytes, &tmB, &full[s], (int32_t)((kb0 + i) * kBK), (int32_t)(blockIdx.y * bn));
        issued = i + 1;
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idesc = tc::idesc_bf16_f32(kBM, bn);
      for (uint32_t i = 0; i < nkb; i++) {
        const uint32_t s = i % nst;
        if (!tc::mbar_wait(&full[s], (i / nst) & 1u, g.wait_ns)) {
          atomicOr(s_err, 1u);
          break;
        }
        tc::fence_after_sync();
        const uint32_t sa = tc::smem_u32(smem + s * stage_bytes), sb = sa + kABytes;
#pragma unroll
        for (uint32_t kk = 0; kk < kBK / 16; kk++)
          tc::mma_bf16(tmem, tc::sdesc_sw128(sa + kk * 32u), tc::sdesc_sw128(sb + kk * 32u), idesc,
                       (i | kk) != 0u ? 1u : 0u);
        tc::mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
      }
      tc::mma_commit(accf);
    }
    __syncwarp();
  }

  // epilogue: warp w reads TMEM lane quadrant w % 4 (tile rows 32(w%4)..) and
  // column half w / 4 of the tile
  if (!tc::mbar_wait(accf, 0, g.wait_ns)) atomicOr(s_err, 1u);
  __syncwarp();  // lanes leave the wait one by one; tcgen05.ld needs the whole warp
  tc::fence_after_sync();
  const uint32_t quad = warp & 3u, half = warp >> 2;
  const uint32_t trow = quad * 32u + lane, row = row0 + trow;
  // uniform over the warp: the staged stores below are warp-collective
  const bool warp_ok = __all_sync(0xffffffffu, *s_err == 0u);
  const bool row_ok = row < rows && warp_ok;
  uint8_t *stage = smem + warp * kStageBytesPerWarp;  // the ring is free: every MMA has read its stage
  // value head: one FP32 chain per 64 columns (the first and the second 64
  // of a 128-column half-tile), so that a 128-column tile's sum is the same
  // whether the tile is a CTA of its own (two warp halves) or half of a
  // 256-column CTA (one warp half)
  float vs0 = 0.0f, vs1 = 0.0f;
  const uint32_t c_lo = half * (bn / 2), c_hi = c_lo + bn / 2;
  for (uint32_t c = c_lo; c < c_hi; c += 32) {
    float v[32];
    tc::tmem_load32(tmem + ((quad * 32u) << 16) + c, v);  // warp-collective: every lane takes part
    const uint32_t col0 = blockIdx.y * bn + c;
    if (row_ok) epilogue_math(g.e, v, row, col0);
    if (warp_ok)
      epilogue_store(g.e, v, stage, row0 + quad * 32u, rows, lane, col0, blockIdx.z, c - c_lo < 64u ? vs0 : vs1);
  }
  if (g.e.flags & kEpiVdot) vpart[half * kBM + trow] = vs0;

  tc::fence_before_sync();
  __syncthreads();
  if ((g.e.flags & kEpiVdot) && row_ok) {  // each 128-column tile: its two 64-column chains, in order
    if (bn == 256u) g.e.vdot_part[(size_t)half * g.e.vdot_ld + row] = vs0 + vs1;
    else if (half == 0) g.e.vdot_part[(size_t)blockIdx.y * g.e.vdot_ld + row] = vpart[trow] + vpart[kBM + trow];
  }
  if ((g.e.flags & kEpiVsum) && blockIdx.y == 0 && half == 0 && row_ok)  // the two tiles' sums, in order
    g.e.vdot_out[row] = (g.e.vdot_part[row] + g.e.vdot_part[g.e.vdot_ld + row]) + g.e.vdot_b[0];
  if (*s_err) {
    if (threadIdx.x == 0) {
      atomicOr(g.status, kStatusNetWait);
      // let loads still in flight land before the CTA's shared memory goes away
      for (uint32_t i = issued > nst ? issued - nst : 0u; i < issued; i++) tc::mbar_wait(&full[i % nst], (i / nst) & 1u);
    }
    __syncthreads();
  }
  if (warp == 2) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, g.tmem_cols);
  }
}

// ---- small kernels

__device__ __forceinline__ uint32_t one_pair(uint32_t bits, int t) {
  return (((bits >> (2 * t)) & 1u) ? 0x3F80u : 0u) | (((bits >> (2 * t + 1)) & 1u) ? 0x3F800000u : 0u);
}

constexpr uint32_t kChunks = kInPad / 8;  // 8-feature chunks of a row of X
constexpr uint32_t kXtChunks = 17;        // chunks holding a feature: 128 piece bits and the side to move

// The four piece planes (own men, own kings, opponent men, opponent kings)
// and the side to move of board r; all zero for r >= nn.
__device__ __forceinline__ void board_planes(const gpuai_board *boards, uint32_t r, uint32_t nn, uint32_t (&pl)[4],
                                             uint32_t &side) {
  pl[0] = pl[1] = pl[2] = pl[3] = 0u;
  side = 0u;
  if (r >= nn) return;
  const uint4 b = __ldg(reinterpret_cast<const uint4 *>(boards) + r);
  side = b.w & 1u;
  const uint32_t own = side ? b.y : b.x, opp = side ? b.x : b.y;
  pl[0] = own & ~b.z;
  pl[1] = own & b.z;
  pl[2] = opp & ~b.z;
  pl[3] = opp & b.z;
}

// X[r] = the 192 features of board r (zero rows past n), one 8-feature chunk
// per thread (thread t: row t / 24, chunk t % 24).  With Xt, thread t also
// writes features 8c .. 8c+7 of column r of X^T for c = t / rows, r = t % rows
// (consecutive threads, consecutive columns); rows 136.. of X^T hold no
// feature and stay zero from the network's creation.
__global__ void features_kernel(const gpuai_board *boards, uint32_t n, const uint32_t *dev_n, uint32_t rows, bf16 *X,
                                bf16 *Xt, uint32_t ldt) {
  tc::grid_dep_wait();
  tc::grid_dep_trigger();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t nn = n;
  if (dev_n) nn = *dev_n < rows ? *dev_n : rows;
  uint32_t pl[4], side;
  if (t < rows * kChunks) {
    const uint32_t r = t / kChunks, c = t - r * kChunks;
    board_planes(boards, r, nn, pl, side);
    uint32_t bits = 0;
    if (c < 16) bits = (pl[c >> 2] >> ((c & 3u) * 8u)) & 0xffu;
    else if (c == 16) bits = side;
    reinterpret_cast<uint4 *>(X + (size_t)r * kInPad)[c] =
        make_uint4(one_pair(bits, 0), one_pair(bits, 1), one_pair(bits, 2), one_pair(bits, 3));
  }
  if (Xt && t < rows * kXtChunks) {
    const uint32_t c = t / rows, r = t - c * rows;
    board_planes(boards, r, nn, pl, side);
    uint16_t *xt = reinterpret_cast<uint16_t *>(Xt);
#pragma unroll
    for (uint32_t j = 0; j < 8; j++) {
      const uint32_t f = 8u * c + j;
      const uint32_t bit = f < 128 ? (pl[f >> 5] >> (f & 31u)) & 1u : (f == 128 ? side : 0u);
      xt[(size_t)f * ldt + r] = bit ? 0x3F80u : 0u;
    }
  }
}

// The (from, to) pair of move `lane` of the list of board b (k moves,
// 1 <= k <= 32), as from * 32 + to; lanes >= k get `none`.  Positions where no
// capture can continue (nearly all) take each lane's move straight from the
// move masks; the others walk the list.  Warp-collective: one board per warp.
__device__ __forceinline__ uint32_t lane_pair(const Side &sd, uint32_t J, int &k, uint32_t lane, uint32_t none) {
  uint32_t M[4];
  bool capture;
  if (simple_move_masks(sd, M, capture)) {
    k = popc(M[0]) + popc(M[1]) + popc(M[2]) + popc(M[3]);
    if (lane >= (uint32_t)k || k > (int)kMaxMoves) return none;
    int from, to;
    uint32_t removed;
    nth_move(M[0], M[1], M[2], M[3], lane, capture, sd.own & ~sd.ownK, from, to, removed);
    return (uint32_t)(from * 32 + to);
  }
  k = count_moves(sd, J);
  if (k < 1 || k > (int)kMaxMoves) return none;
  uint32_t pi = none, m = 0;
  for_each_move(sd, J, [&](int from, int to, uint32_t, int, uint32_t) {
    if (m == lane) pi = (uint32_t)(from * 32 + to);
    m++;
    return false;
  });
  return pi;
}

// One warp per row: value and policy loss terms and their gradients.  Lane m
// holds move m of the reference move list; moves with the same (from, to)
// share one logit (the lowest such lane speaks for the pair).
__global__ void loss_kernel(const gpuai_board *boards, const float *z, const float *q, uint32_t n, uint32_t rows,
                            float tau, float vcoef, const float *logits, const float *vraw, bf16 *dZ3, bf16 *dZ3t,
                            uint32_t ldt, float *dv, float *rowloss) {
  tc::grid_dep_wait();  // the logits and the value come from the kernel before this one
  tc::grid_dep_trigger();
  const uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
  constexpr uint32_t kFull = 0xffffffffu;
  if (r >= rows) return;
  if (r >= n) {
    if (lane == 0) {
      dv[r] = 0.0f;
      rowloss[2 * r] = rowloss[2 * r + 1] = 0.0f;
    }
    return;
  }
  const float inv_n = 1.0f / (float)n;
  if (lane == 0) {
    const float th = tanhf(vraw[r]);
    const float e = th - z[r];
    dv[r] = vcoef * 2.0f * e * (1.0f - th * th) * inv_n;
    rowloss[2 * r + 1] = e * e;
  }
  const uint4 bv = __ldg(reinterpret_cast<const uint4 *>(boards) + r);
  const Board b{bv.x, bv.y, bv.z, bv.w};
  Side sd;
  make_side(b, sd);
  const uint32_t J = jumpers(sd);
  int k = 0;
  // distinct placeholder for lanes without a move
  const uint32_t pi = lane_pair(sd, J, k, lane, 0x10000u + lane);
  float ce = 0.0f;
  if (k >= 1 && k <= (int)kMaxMoves) {  // uniform over the warp
    const bool act = lane < (uint32_t)k;
    const float qm = act ? q[(size_t)r * kMaxMoves + lane] : -3.0e38f;
    float qmax = qm;
    for (int o = 16; o; o >>= 1) qmax = fmaxf(qmax, __shfl_xor_sync(kFull, qmax, o));
    const float et = act ? expf((qm - qmax) / tau) : 0.0f;
    float tsum = et;
    for (int o = 16; o; o >>= 1) tsum += __shfl_xor_sync(kFull, tsum, o);
    const float t = et / tsum;
    const uint32_t grp = __match_any_sync(kFull, pi);
    const bool leader = act && (uint32_t)(__ffs(grp) - 1) == lane;
    float tp = t;  // target of this lane's pair: sum over the lanes sharing it, in lane order
    if (__any_sync(kFull, (grp & (grp - 1u)) != 0u)) {  // some pair has two moves (king captures)
      tp = 0.0f;
      for (int j = 0; j < 32; j++) {
        const float tj = __shfl_sync(kFull, t, j);
        if ((grp >> j) & 1u) tp += tj;
      }
    }
    const float lg = leader ? logits[(size_t)r * kOut + pi] : -3.0e38f;
    float lmax = lg;
    for (int o = 16; o; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(kFull, lmax, o));
    float sum = leader ? expf(lg - lmax) : 0.0f;
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
    const float logz = lmax + logf(sum);
    if (leader) {
      const float lp = lg - logz;
      ce = -tp * lp;
      const bf16 gq = __float2bfloat16_rn((expf(lp) - tp) * inv_n);
      dZ3[(size_t)r * kOut + pi] = gq;
      dZ3t[(size_t)pi * ldt + r] = gq;
    }
    for (int o = 16; o; o >>= 1) ce += __shfl_xor_sync(kFull, ce, o);
  }
  if (lane == 0) rowloss[2 * r] = ce;
}

// The terms of loss_kernel for row r on a segment of W lanes of the warp:
// lane l of the segment holds move l of the row's list (pair pi) or none, k
// moves in all; the segment's first lane writes the row's terms.  Same
// arithmetic as loss_kernel's (its 32-lane reductions only add the neutral
// values of lanes without a move).  Warp-collective: every lane of the warp
// calls it, with W = 32 (one row) or W = 16 (two rows, one per half).
template <uint32_t W>
__device__ __forceinline__ void row_loss(uint32_t r, bool row_ok, int k, uint32_t pi, const float *z, const float *q,
                                         uint32_t n, float tau, float vcoef, const float *logits, const float *vraw,
                                         bf16 *dZ3, bf16 *dZ3t, uint32_t ldt, float *dv, float *rowloss) {
  constexpr uint32_t kFull = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u, sl = lane & (W - 1u), base = lane & ~(W - 1u);
  const float inv_n = 1.0f / (float)n;
  if (sl == 0) {
    float dvr = 0.0f, ve = 0.0f;
    if (row_ok) {
      const float th = tanhf(vraw[r]);
      const float e = th - z[r];
      dvr = vcoef * 2.0f * e * (1.0f - th * th) * inv_n;
      ve = e * e;
    }
    dv[r] = dvr;
    rowloss[2 * r + 1] = ve;
  }
  const bool act = row_ok && k >= 1 && k <= (int)kMaxMoves && sl < (uint32_t)k;
  const float qm = act ? q[(size_t)r * kMaxMoves + sl] : -3.0e38f;
  float qmax = qm;
  for (uint32_t o = W / 2; o; o >>= 1) qmax = fmaxf(qmax, __shfl_xor_sync(kFull, qmax, o));
  const float et = act ? expf((qm - qmax) / tau) : 0.0f;
  float tsum = et;
  for (uint32_t o = W / 2; o; o >>= 1) tsum += __shfl_xor_sync(kFull, tsum, o);
  const float t = act ? et / tsum : 0.0f;
  const uint32_t grp = __match_any_sync(kFull, pi | (base << 20));  // pairs of the lane's own row
  const bool leader = act && (uint32_t)(__ffs(grp) - 1) == lane;
  float tp = t;  // target of this lane's pair: sum over the lanes sharing it, in lane order
  if (__any_sync(kFull, (grp & (grp - 1u)) != 0u)) {  // some pair has two moves (king captures)
    tp = 0.0f;
    for (uint32_t j = 0; j < W; j++) {
      const float tj = __shfl_sync(kFull, t, base + j);
      if ((grp >> (base + j)) & 1u) tp += tj;
    }
  }
  const float lg = leader ? logits[(size_t)r * kOut + pi] : -3.0e38f;
  float lmax = lg;
  for (uint32_t o = W / 2; o; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(kFull, lmax, o));
  float sum = leader ? expf(lg - lmax) : 0.0f;
  for (uint32_t o = W / 2; o; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
  float ce = 0.0f;
  if (leader) {
    const float lp = lg - (lmax + logf(sum));
    ce = -tp * lp;
    const bf16 gq = __float2bfloat16_rn((expf(lp) - tp) * inv_n);
    dZ3[(size_t)r * kOut + pi] = gq;
    dZ3t[(size_t)pi * ldt + r] = gq;
  }
  for (uint32_t o = W / 2; o; o >>= 1) ce += __shfl_xor_sync(kFull, ce, o);
  if (sl == 0) rowloss[2 * r] = ce;
}

// loss_kernel for batches of several waves of warps, two rows per warp (rows
// 2w and 2w+1): when both list at most 16 moves, none of them a capture that
// can continue, each half of the warp takes one row and each lane its move
// straight from the move masks; otherwise the warp takes the two rows one
// after the other on all 32 lanes.  Half the warps and about half the
// instructions of one row per warp, which pays where the rows fill several
// waves; where they fit in one, loss_kernel's shorter warps are faster.
__global__ void loss_pairs_kernel(const gpuai_board *boards, const float *z, const float *q, uint32_t n,
                                  uint32_t rows, float tau, float vcoef, const float *logits, const float *vraw,
                                  bf16 *dZ3, bf16 *dZ3t, uint32_t ldt, float *dv, float *rowloss) {
  tc::grid_dep_wait();  // the logits and the value come from the kernel before this one
  tc::grid_dep_trigger();
  constexpr uint32_t kFull = 0xffffffffu;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
  const uint32_t r0 = 2u * w;
  if (r0 >= rows) return;  // uniform over the warp; rows is even
  const uint32_t r = r0 + (lane >> 4), hl = lane & 15u;
  Side sd{};
  uint32_t M[4] = {0u, 0u, 0u, 0u};
  bool capture = false, simple = true;
  int k = 0;
  if (r < n) {
    const uint4 bv = __ldg(reinterpret_cast<const uint4 *>(boards) + r);
    make_side(Board{bv.x, bv.y, bv.z, bv.w}, sd);
    simple = simple_move_masks(sd, M, capture);
    k = simple ? popc(M[0]) + popc(M[1]) + popc(M[2]) + popc(M[3]) : 0;
  }
  if (__all_sync(kFull, simple && k <= 16)) {
    uint32_t pi = 0x10000u + lane;  // distinct placeholder for lanes without a move
    if (hl < (uint32_t)k) {
      int from, to;
      uint32_t removed;
      nth_move(M[0], M[1], M[2], M[3], hl, capture, sd.own & ~sd.ownK, from, to, removed);
      pi = (uint32_t)(from * 32 + to);
    }
    row_loss<16>(r, r < n, k, pi, z, q, n, tau, vcoef, logits, vraw, dZ3, dZ3t, ldt, dv, rowloss);
    return;
  }
  for (uint32_t h = 0; h < 2; h++) {
    const uint32_t rr = r0 + h;
    int kk = 0;
    uint32_t pi = 0x10000u + lane;
    if (rr < n) {
      const uint4 bv = __ldg(reinterpret_cast<const uint4 *>(boards) + rr);
      Side s2;
      make_side(Board{bv.x, bv.y, bv.z, bv.w}, s2);
      pi = lane_pair(s2, jumpers(s2), kk, lane, 0x10000u + lane);
    }
    row_loss<32>(rr, rr < n, kk, pi, z, q, n, tau, vcoef, logits, vraw, dZ3, dZ3t, ldt, dv, rowloss);
  }
}

// Zeroes the entries of dZ3 and dZ3^T that the loss (loss_kernel or
// loss_pairs_kernel) wrote for rows [0, n):
// the (from, to) pairs of each row's legal moves, found the same way.
__global__ void clear_dz3_kernel(const gpuai_board *boards, uint32_t n, bf16 *dZ3, bf16 *dZ3t, uint32_t ldt) {
  const uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
  if (r >= n) return;
  const uint4 bv = __ldg(reinterpret_cast<const uint4 *>(boards) + r);
  const Board b{bv.x, bv.y, bv.z, bv.w};
  Side sd;
  make_side(b, sd);
  int k = 0;
  const uint32_t pi = lane_pair(sd, jumpers(sd), k, lane, ~0u);
  if (pi == ~0u) return;
  const bf16 zero = __float2bfloat16_rn(0.0f);
  dZ3[(size_t)r * kOut + pi] = zero;
  dZ3t[(size_t)pi * ldt + r] = zero;
}

// out[row] = sum over the first ncols columns of M[row] (times vec[col] if
// given); one block of 256 threads per row, fixed order.
__global__ void __launch_bounds__(256) rowsum_kernel(const bf16 *M, uint32_t ncols, uint32_t ld, const float *vec,
                                                     float *out) {
  __shared__ float red[256];
  const uint32_t row = blockIdx.x, tid = threadIdx.x;
  const bf16 *p = M + (size_t)row * ld;
  float s = 0.0f;
  for (uint32_t c = tid * 8u; c < ncols; c += 2048u) {
    const uint4 u = *reinterpret_cast<const uint4 *>(p + c);
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const float a = lo_bf(w[t]), b = hi_bf(w[t]);
      s += vec ? a * vec[c + 2 * t] : a;
      s += vec ? b * vec[c + 2 * t + 1] : b;
    }
  }
  red[tid] = s;
  __syncthreads();
  for (uint32_t o = 128; o; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) out[row] = red[0];
}

// One block of 256: loss2 = {mean policy cross entropy, mean squared value
// error} over the n rows, and dbv = sum of dv over all rows (fixed order).
__global__ void loss_reduce_kernel(const float *rowloss, const float *dv, uint32_t n, uint32_t rows, float *loss2,
                                   float *dbv) {
  __shared__ float sp[256], sv[256], sd[256];
  float a = 0.0f, b = 0.0f, c = 0.0f;
  for (uint32_t i = threadIdx.x; i < n; i += 256) {
    a += rowloss[2 * i];
    b += rowloss[2 * i + 1];
  }
  for (uint32_t i = threadIdx.x; i < rows; i += 256) c += dv[i];
  sp[threadIdx.x] = a;
  sv[threadIdx.x] = b;
  sd[threadIdx.x] = c;
  __syncthreads();
  for (uint32_t o = 128; o; o >>= 1) {
    if (threadIdx.x < o) {
      sp[threadIdx.x] += sp[threadIdx.x + o];
      sv[threadIdx.x] += sv[threadIdx.x + o];
      sd[threadIdx.x] += sd[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    loss2[0] = n ? sp[0] / (float)n : 0.0f;
    loss2[1] = n ? sv[0] / (float)n : 0.0f;
    dbv[0] = sd[0];
  }
}

struct AdamArgs {
  float *w, *m, *v;
  const float *g_direct;  // bias / value-head gradients (parameter layout)
  const float *p1, *p2, *p3;
  uint32_t s1, s2, s3;    // split-K partial counts of dW1, dW2, dW3
  float lr, bc1, bc2;
  uint32_t mode;          // 0 update, 1 write the gradient to g_out, 2 refresh the BF16 copies only
  float *g_out;
  bf16 *W1b, *W2b, *W3b, *W2T, *W3T;
};

constexpr float kBeta1 = 0.9f, kBeta2 = 0.999f, kAdamEps = 1e-8f;

// p[0] + p[stride] + ... + p[(count - 1) * stride], added in that order; the
// loads are issued eight at a time.
__device__ __forceinline__ float sum_partials(const float *p, size_t stride, uint32_t count) {
  float g = 0.0f;
  uint32_t s = 0;
  for (; s + 8u <= count; s += 8u) {
    float t[8];
#pragma unroll
    for (uint32_t j = 0; j < 8; j++) t[j] = __ldg(p + (size_t)(s + j) * stride);
#pragma unroll
    for (uint32_t j = 0; j < 8; j++) g += t[j];
  }
  for (; s < count; s++) g += __ldg(p + (size_t)s * stride);
  return g;
}

__global__ void adam_kernel(AdamArgs a) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  float w = a.w[i];
  if (a.mode != 2) {
    float g = 0.0f;
    if (i < oB1) {
      g = sum_partials(a.p1 + (i - oW1), (size_t)kH * kInPad, a.s1);
    } else if (i >= oW2 && i < oB2) {
      g = sum_partials(a.p2 + (i - oW2), (size_t)kH * kH, a.s2);
    } else if (i >= oW3 && i < oB3) {
      g = sum_partials(a.p3 + (i - oW3), (size_t)kOut * kH, a.s3);
    } else {
      g = a.g_direct[i];
    }
    if (a.mode == 1) {
      a.g_out[i] = g;
      return;
    }
    const float lr = a.lr, bc1 = a.bc1, bc2 = a.bc2;
    const float m = kBeta1 * a.m[i] + (1.0f - kBeta1) * g;
    const float v = kBeta2 * a.v[i] + (1.0f - kBeta2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    w -= lr * (m / bc1) / (sqrtf(v / bc2) + kAdamEps);
    a.w[i] = w;
  }
  const bf16 wb = __float2bfloat16_rn(w);
  if (i < oB1) {
    a.W1b[i - oW1] = wb;
  } else if (i >= oW2 && i < oB2) {
    const size_t j = i - oW2, r = j / kH, c = j % kH;
    a.W2b[j] = wb;
    a.W2T[c * kH + r] = wb;
  } else if (i >= oW3 && i < oB3) {
    const size_t j = i - oW3, r = j / kH, c = j % kH;
    a.W3b[j] = wb;
    a.W3T[c * kOut + r] = wb;
  }
}

__global__ void tanh_kernel(const float *x, uint32_t n, float *y) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = tanhf(x[i]);
}

// ---- training labels

constexpr uint32_t kLabelSlots = kMaxMoves;  // child slots per position

// Child boards and playout offsets: position i owns playouts
// [i*P, (i+1)*P); move m of its k moves gets P/k (+1 for m < P%k) of them.  A
// position that is over (or has more than 32 moves) gives all P playouts to
// slot 0, a copy of itself, and is marked with nmoves 0.
__global__ void label_children_kernel(const gpuai_board *pos, uint32_t n, uint32_t P, Board *children,
                                      uint32_t *offsets, uint8_t *nmoves) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 bv = __ldg(reinterpret_cast<const uint4 *>(pos) + i);
  const Board b{bv.x, bv.y, bv.z, bv.w};
  Side sd;
  make_side(b, sd);
  const uint32_t J = jumpers(sd);
  int k = ((b.meta >> 8) & 0xffu) >= (uint32_t)kDrawPlies ? 0 : count_moves(sd, J);
  if (k < 0 || k > (int)kLabelSlots) k = 0;
  Board *ch = children + (size_t)i * kLabelSlots;
  uint32_t *off = offsets + (size_t)i * kLabelSlots;
  const uint32_t base = i * P;
  int m = 0;
  if (k > 0) {
    for_each_move(sd, J, [&](int from, int to, uint32_t removed, int, uint32_t) {
      Board c = b;
      apply_move(c, from, to, removed);
      ch[m++] = c;
      return false;
    });
  }
  for (; m < (int)kLabelSlots; m++) ch[m] = b;
  const uint32_t uk = (uint32_t)k;
  for (uint32_t s = 0; s < kLabelSlots; s++) {
    uint32_t o;
    if (uk == 0) o = s == 0 ? base : base + P;
    else o = s >= uk ? base + P : base + s * (P / uk) + (s < P % uk ? s : P % uk);
    off[s] = o;
  }
  nmoves[i] = (uint8_t)uk;
  if (i == n - 1) offsets[(size_t)n * kLabelSlots] = n * P;
}

// One warp per position: move values and the position value for its side to move.
__global__ void label_reduce_kernel(const gpuai_board *pos, const int8_t *out, const uint32_t *offsets,
                                    const uint8_t *nmoves, uint32_t n, uint32_t P, float *value, float *q) {
  const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
  if (i >= n) return;
  const uint32_t k = nmoves[i];
  const float sign = (pos[i].meta & 1u) ? -1.0f : 1.0f;  // outcome +1 = PLAYER_1 won
  int total = 0;
  for (uint32_t m = 0; m < kLabelSlots; m++) {
    float qm = 0.0f;
    if (m < k) {
      const uint32_t a = offsets[(size_t)i * kLabelSlots + m], e = offsets[(size_t)i * kLabelSlots + m + 1];
      int s = 0;
      for (uint32_t j = a + lane; j < e; j += 32) s += out[j];
      for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      total += s;
      qm = sign * (float)s / (float)(e - a);
    }
    if (lane == 0) q[(size_t)i * kMaxMoves + m] = qm;
  }
  if (lane == 0) value[i] = k ? sign * (float)total / (float)P : 0.0f;
}

// ---- host side

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Tensor map of a K-major BF16 matrix (rows x k, row pitch k elements) read
// in boxes of 64 x box_rows with the 128-byte swizzle.
cudaError_t make_map(CUtensorMap *m, const void *base, uint64_t rows, uint64_t k, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  if (k % kBK || box_rows == 0 || box_rows > 256 || reinterpret_cast<uintptr_t>(base) % 16)
    return cudaErrorInvalidValue;
  const cuuint64_t dims[2] = {k, rows};
  const cuuint64_t strides[1] = {k * 2};
  const cuuint32_t box[2] = {kBK, box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Multiprocessors of the current device (read once).
uint32_t sm_count() {
  static uint32_t n = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) ==
                                                  cudaSuccess)
      n = (uint32_t)v;
  });
  return n;
}

// Launches `kernel`; with `pdl` it may start before the kernel ahead of it in
// the stream has finished (the kernel then waits for it with grid_dep_wait).
template <class... Params, class... Args>
cudaError_t launch(void (*kernel)(Params...), dim3 grid, uint32_t threads, uint32_t smem, cudaStream_t s, bool pdl,
                   Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1u : 0u;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

cudaError_t gemm(const CUtensorMap &a, const CUtensorMap &b, uint32_t m_rows, uint32_t n_total, uint32_t bn,
                 uint32_t kb_total, uint32_t splits, const uint32_t *dev_rows, uint32_t *status, const Epi &e,
                 cudaStream_t s, bool pdl = false, uint64_t wait_ns = tc::kWaitLimitNs, bool skip_loads = false) {
  if (m_rows % kBM || bn % 64 || bn == 0 || bn > 256 || n_total % bn || splits == 0 || kb_total % splits)
    return cudaErrorInvalidValue;
  if ((e.flags & kEpiVdot) && !(n_total == 256u && (bn == 128u || bn == 256u)))  // the value head's two tiles
    return cudaErrorInvalidValue;
  GemmArgs g;
  g.m_rows = m_rows;
  g.bn = bn;
  g.tmem_cols = bn <= 64 ? 64u : (bn <= 128 ? 128u : 256u);
  g.kb_per_split = kb_total / splits;
  const uint32_t stage_bytes = kABytes + bn * 128u;
  // A product of the training step's critical chain (the launches with
  // `pdl`) whose grid is at most one CTA per SM gets twice the ring: more
  // loads in flight.  The side streams' products keep room for a second CTA
  // on each SM, where they run beside the chain.
  const uint32_t ctas = (m_rows / kBM) * (n_total / bn) * splits;
  const uint32_t budget = pdl && ctas <= sm_count() ? 2u * kRingBudget : kRingBudget;
  uint32_t st = budget / stage_bytes;
  st = st < 2 ? 2 : (st > kMaxStages ? kMaxStages : st);
  g.stages = g.kb_per_split < st ? g.kb_per_split : st;
  g.dev_rows = dev_rows;
  g.status = status;
  g.e = e;
  g.wait_ns = wait_ns;
  g.skip_loads = skip_loads ? 1u : 0u;
  const uint32_t ring = g.stages * stage_bytes;
  const uint32_t smem = (ring > kStageBytes ? ring : kStageBytes) + kSmemExtra;
  if (smem > kSmemLimit) return cudaErrorInvalidValue;
  return launch(gemm_kernel, dim3(m_rows / kBM, n_total / bn, splits), kThreads, smem, s, pdl, a, b, g);
}

uint32_t pick_splits(uint32_t kb, uint32_t target) {
  for (uint32_t s = target; s > 1; s--)
    if (kb % s == 0 && kb / s >= 2) return s;
  return 1;
}

// Split-K factors of the weight-gradient products (K = the batch): dW3, dW2,
// dW1 above 16,384 rows; up to 16,384 rows dW1 takes more splits (more CTAs
// for the last product of the chain) and dW2 fewer (fewer partials for Adam
// to sum), 2 % faster at 8192 rows and 0.7 % slower at 32,768.
constexpr uint32_t kSplit3 = 8, kSplit2 = 32, kSplit1 = 16;
constexpr uint32_t kSmallBatch = 16384, kSplit2Small = 16, kSplit1Small = 32;
constexpr uint32_t kMaxSplit2 = kSplit2 > kSplit2Small ? kSplit2 : kSplit2Small;
constexpr uint32_t kMaxSplit1 = kSplit1 > kSplit1Small ? kSplit1 : kSplit1Small;
// N tile of each product (the B operand's tensor-map box height)
// B1 and B3 take 128-wide tiles when that fills the SMs, else 64-wide (twice
// the CTAs, two per SM); F2 takes two 128-wide tiles per row block while
// that leaves SMs idle, else one 256-wide tile (the value-head sums of its two
// halves are the same either way, and F3 adds them).
constexpr uint32_t kBnF1 = 128, kBnF2 = 128, kBnF3 = 256, kBnB1 = 128, kBnB3 = 128, kBnNarrow = 64,
                   kBnB2 = 128, kBnB4 = 128, kBnB5 = 64;

template <class T>
cudaError_t dalloc(std::vector<void *> &allocs, T **p, size_t n) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T) + 256);
  if (e == cudaSuccess) {
    allocs.push_back(q);
    *p = static_cast<T *>(q);
  }
  return e;
}

uint32_t round128(uint32_t n) { return (n + 127u) / 128u * 128u; }

}  // namespace

cudaError_t fwd_alloc(Fwd &w, uint32_t rows, std::vector<void *> &allocs, bool bf16_logits) {
  w.rows = round128(rows ? rows : 1);
  cudaError_t e = dalloc(allocs, &w.X, (size_t)w.rows * kInPad);
  if (e == cudaSuccess) e = dalloc(allocs, &w.H1, (size_t)w.rows * kH);
  if (e == cudaSuccess) e = dalloc(allocs, &w.H2, (size_t)w.rows * kH);
  if (e == cudaSuccess && bf16_logits) e = dalloc(allocs, &w.logits_b, (size_t)w.rows * kOut);
  if (e == cudaSuccess && !bf16_logits) e = dalloc(allocs, &w.logits, (size_t)w.rows * kOut);
  if (e == cudaSuccess) e = dalloc(allocs, &w.vraw, (size_t)w.rows);
  if (e == cudaSuccess) e = dalloc(allocs, &w.vpart, 2 * (size_t)w.rows);
  if (e == cudaSuccess) e = make_map(&w.mX, w.X, w.rows, kInPad, kBM);
  if (e == cudaSuccess) e = make_map(&w.mH1, w.H1, w.rows, kH, kBM);
  if (e == cudaSuccess) e = make_map(&w.mH2, w.H2, w.rows, kH, kBM);
  return e;
}

namespace {

// Forward through the three layers; with `train`, also the transposed
// activations the backward pass reads.
cudaError_t forward_impl(const gpuai_net *net, Fwd &w, const gpuai_board *boards, uint32_t n, const uint32_t *dev_n,
                         uint32_t rows, uint32_t *status, bool train, cudaStream_t s) {
  const float *P = net->params;
  features_kernel<<<(rows * kChunks + 255) / 256, 256, 0, s>>>(boards, n, dev_n, rows, w.X, train ? net->Xt : nullptr,
                                                     net->rows);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  Epi e1;
  e1.flags = kEpiBias | kEpiRelu | kEpiB16 | (train ? kEpiB16T : 0u);
  e1.bias = P + oB1;
  e1.out_b = w.H1;
  e1.ld_b = kH;
  e1.out_t = net->H1t;
  e1.ld_t = net->rows;
  if ((e = gemm(w.mX, net->mW1, rows, kH, kBnF1, kInPad / kBK, 1, dev_n, status, e1, s, train)) != cudaSuccess)
    return e;
  Epi e2 = e1;
  e2.flags |= kEpiVdot;
  e2.bias = P + oB2;
  e2.out_b = w.H2;
  e2.out_t = net->H2t;
  e2.vdot_w = P + oWV;
  e2.vdot_part = w.vpart;
  e2.vdot_ld = w.rows;
  // F2 in 128-column tiles (two CTAs per row block) while that leaves SMs
  // idle, in 256-column tiles once the row blocks alone fill the SMs
  const bool wide2 = rows / kBM >= sm_count();
  if ((e = gemm(w.mH1, wide2 ? net->mW2w : net->mW2, rows, kH, wide2 ? 2u * kBnF2 : kBnF2, kH / kBK, 1, dev_n, status,
                e2, s, train)) != cudaSuccess)
    return e;
  Epi e3;
  e3.flags = kEpiBias | kEpiVsum | (w.logits_b ? kEpiB16 : kEpiF32);
  e3.bias = P + oB3;
  e3.vdot_part = w.vpart;
  e3.vdot_ld = w.rows;
  e3.vdot_b = P + oBV;
  e3.vdot_out = w.vraw;
  e3.out_f32 = w.logits;
  e3.ld_f32 = kOut;
  e3.out_b = w.logits_b;
  e3.ld_b = kOut;
  return gemm(w.mH2, net->mW3, rows, kOut, kBnF3, kH / kBK, 1, dev_n, status, e3, s, train);
}

// Forward + backward on rows [0, n) of the training workspace; gradients are
// left in the partial buffers and net->grad.
cudaError_t backward_impl(gpuai_net *net, const gpuai_board *boards, const float *z, const float *q, uint32_t n,
                          float tau, float vcoef, uint32_t *splits, cudaStream_t s) {
  const uint32_t B = round128(n), L = net->rows;
  const float *P = net->params;
  cudaError_t e = forward_impl(net, net->fw, boards, n, nullptr, B, net->status, true, s);
  if (e != cudaSuccess) return e;
  // The chain forward -> loss -> dZ2 -> dZ1 -> dW1 launches each kernel while
  // the one before it drains (programmatic dependent launch); dZ3 and dZ3^T
  // are zero on entry apart from what this step's loss kernel writes.
  net->dz_dirty = true;  // until clear_dz3_kernel is queued
  // one row per warp while the rows fit one wave of resident warps (64 per
  // SM with these 128-thread blocks), two per warp above that
  const bool pairs = B > 64u * sm_count();
  if ((e = launch(pairs ? loss_pairs_kernel : loss_kernel, dim3(pairs ? B / 8 : B / 4), 128, 0, s, true, boards, z,
                  q, n, B, tau, vcoef, net->fw.logits, net->fw.vraw, net->dZ3, net->dZ3t, L, net->dv,
                  net->rowloss)) != cudaSuccess)
    return e;
  const uint32_t kb = B / kBK;
  const bool small = B <= kSmallBatch;
  splits[2] = pick_splits(kb, kSplit3);
  splits[1] = pick_splits(kb, small ? kSplit2Small : kSplit2);
  splits[0] = pick_splits(kb, small ? kSplit1Small : kSplit1);
  const cudaStream_t t = net->side, u = net->side2;
  // side stream, after the loss: dW3 partials, db3, dwv, the loss means and dbv
  if ((e = cudaEventRecord(net->ev_loss, s)) != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(t, net->ev_loss, 0)) != cudaSuccess) return e;
  Epi b2;
  b2.flags = kEpiPartial;
  b2.out_f32 = net->p3;
  b2.ld_f32 = kH;
  b2.partial_stride = (uint64_t)kOut * kH;
  if ((e = gemm(net->mdZ3t, net->mH2t, kOut, kH, kBnB2, kb, splits[2], nullptr, net->status, b2, t)) != cudaSuccess)
    return e;
  rowsum_kernel<<<kOut, 256, 0, t>>>(net->dZ3t, B, L, nullptr, net->grad + oB3);
  rowsum_kernel<<<kH, 256, 0, t>>>(net->H2t, B, L, net->dv, net->grad + oWV);
  loss_reduce_kernel<<<1, 256, 0, t>>>(net->rowloss, net->dv, n, B, net->loss2, net->grad + oBV);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(net->ev_side, t)) != cudaSuccess) return e;
  Epi b1;
  b1.flags = kEpiRank1 | kEpiMask | kEpiB16 | kEpiB16T;
  b1.r1_row = net->dv;
  b1.r1_col = P + oWV;
  b1.mask = net->fw.H2;
  b1.ld_mask = kH;
  b1.out_b = net->dZ2;
  b1.ld_b = kH;
  b1.out_t = net->dZ2t;
  b1.ld_t = L;
  const bool wide = (B / kBM) * (kH / kBnB1) >= sm_count();  // 128-wide tiles of B1 and B3 fill the SMs
  if ((e = gemm(net->mdZ3, wide ? net->mW3T : net->mW3Tn, B, kH, wide ? kBnB1 : kBnNarrow, kOut / kBK, 1, nullptr,
                net->status, b1, s, true)) != cudaSuccess)
    return e;
  // third stream, after dZ2: dW2 partials and db2; side stream: dZ3 (read
  // by dZ2's product) and dZ3^T (dW3's) back to zero, which nothing in the
  // step waits for (the main stream joins it at the end of the step)
  if ((e = cudaEventRecord(net->ev_b1, s)) != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(u, net->ev_b1, 0)) != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(t, net->ev_b1, 0)) != cudaSuccess) return e;
  clear_dz3_kernel<<<B / 4, 128, 0, t>>>(boards, n, net->dZ3, net->dZ3t, L);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(net->ev_clear, t)) != cudaSuccess) return e;
  net->dz_dirty = false;
  Epi b4;
  b4.flags = kEpiPartial;
  b4.out_f32 = net->p2;
  b4.ld_f32 = kH;
  b4.partial_stride = (uint64_t)kH * kH;
  if ((e = gemm(net->mdZ2t, net->mH1t, kH, kH, kBnB4, kb, splits[1], nullptr, net->status, b4, u)) != cudaSuccess)
    return e;
  rowsum_kernel<<<kH, 256, 0, u>>>(net->dZ2t, B, L, nullptr, net->grad + oB2);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  Epi b3;
  b3.flags = kEpiMask | kEpiB16T;
  b3.mask = net->fw.H1;
  b3.ld_mask = kH;
  b3.out_t = net->dZ1t;
  b3.ld_t = L;
  if ((e = gemm(net->mdZ2, wide ? net->mW2T : net->mW2Tn, B, kH, wide ? kBnB3 : kBnNarrow, kH / kBK, 1, nullptr,
                net->status, b3, s, true)) != cudaSuccess)
    return e;
  // third stream, after dZ1: db1; then the main stream waits for both side streams
  if ((e = cudaEventRecord(net->ev_b3, s)) != cudaSuccess) return e;
  if ((e = cudaStreamWaitEvent(u, net->ev_b3, 0)) != cudaSuccess) return e;
  rowsum_kernel<<<kH, 256, 0, u>>>(net->dZ1t, B, L, nullptr, net->grad + oB1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(net->ev_side2, u)) != cudaSuccess) return e;
  Epi b5;
  b5.flags = kEpiPartial;
  b5.out_f32 = net->p1;
  b5.ld_f32 = kInPad;
  b5.partial_stride = (uint64_t)kH * kInPad;
  if ((e = gemm(net->mdZ1t, net->mXt, kH, kInPad, kBnB5, kb, splits[0], nullptr, net->status, b5, s, true)) !=
      cudaSuccess)
    return e;
  if ((e = cudaStreamWaitEvent(s, net->ev_side, 0)) != cudaSuccess) return e;
  return cudaStreamWaitEvent(s, net->ev_side2, 0);
}

// Joins the side stream's clearing of dZ3 / dZ3^T into `s` (after the
// step's last kernel on `s`, so nothing there waits for it).
cudaError_t join_clear(gpuai_net *net, cudaStream_t s) { return cudaStreamWaitEvent(s, net->ev_clear, 0); }

// dZ3 and dZ3^T in full back to zero after a step that stopped half-way.
cudaError_t clear_dz3_full(gpuai_net *net, cudaStream_t s) {
  if (!net->dz_dirty) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(net->dZ3, 0, (size_t)net->rows * kOut * sizeof(bf16), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->dZ3t, 0, (size_t)kOut * net->rows * sizeof(bf16), s);
  if (e == cudaSuccess) net->dz_dirty = false;
  return e;
}

cudaError_t run_adam(gpuai_net *net, uint32_t mode, const uint32_t *splits, float lr, cudaStream_t s) {
  AdamArgs a;
  a.w = net->params;
  a.m = net->adam_m;
  a.v = net->adam_v;
  a.g_direct = net->grad;
  a.p1 = net->p1;
  a.p2 = net->p2;
  a.p3 = net->p3;
  a.s1 = splits ? splits[0] : 0;
  a.s2 = splits ? splits[1] : 0;
  a.s3 = splits ? splits[2] : 0;
  a.lr = lr;
  a.bc1 = (float)(1.0 - std::pow(0.9, (double)net->step));
  a.bc2 = (float)(1.0 - std::pow(0.999, (double)net->step));
  a.mode = mode;
  a.g_out = net->gout;
  a.W1b = net->W1b;
  a.W2b = net->W2b;
  a.W3b = net->W3b;
  a.W2T = net->W2T;
  a.W3T = net->W3T;
  adam_kernel<<<(uint32_t)((kParams + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

template <class... P>
constexpr uint32_t nparams(void (*)(P...)) {
  return (uint32_t)sizeof...(P);
}

// The one kernel node of graph g that runs `func`.
cudaError_t find_kernel_node(cudaGraph_t g, const void *func, cudaGraphNode_t *out) {
  size_t count = 0;
  cudaError_t e = cudaGraphGetNodes(g, nullptr, &count);
  std::vector<cudaGraphNode_t> nodes(count);
  if (e == cudaSuccess && count) e = cudaGraphGetNodes(g, nodes.data(), &count);
  if (e != cudaSuccess) return e;
  *out = nullptr;
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType t;
    cudaKernelNodeParams p;
    if (cudaGraphNodeGetType(node, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
    if ((e = cudaGraphKernelNodeGetParams(node, &p)) != cudaSuccess) return e;
    if (p.func != func) continue;
    if (*out) return cudaErrorInvalidValue;  // more than one
    *out = node;
  }
  return *out ? cudaSuccess : cudaErrorInvalidValue;
}

// Replaces arguments of kernel node `node` (nargs in all) of the instantiated
// graph x: argument r.first by *r.second; the others keep their captured
// values.  The next launch of x uses them.
cudaError_t set_node_args(cudaGraphExec_t x, cudaGraphNode_t node, uint32_t nargs,
                          std::initializer_list<std::pair<uint32_t, void *>> repl) {
  cudaKernelNodeParams p;
  cudaError_t e = cudaGraphKernelNodeGetParams(node, &p);
  if (e != cudaSuccess) return e;
  if (!p.kernelParams || p.extra || nargs > 16) return cudaErrorNotSupported;
  void *args[16];
  for (uint32_t i = 0; i < nargs; i++) args[i] = p.kernelParams[i];
  for (const auto &r : repl) {
    if (r.first >= nargs) return cudaErrorInvalidValue;
    args[r.first] = r.second;
  }
  p.kernelParams = args;
  return cudaGraphExecKernelNodeSetParams(x, node, &p);
}

int err(int code, const std::string &m) { return ga::record_error(code, m.c_str()); }
int cuda_err(cudaError_t e, const char *what) {
  return err(e == cudaErrorMemoryAllocation ? GPUAI_ERR_OOM : GPUAI_ERR_CUDA,
             std::string("net: ") + what + ": " + cudaGetErrorString(e));
}

#define NCK(call, what)                               \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_err(e_, what); \
  } while (0)

int check_status(gpuai_net *net) {
  uint32_t st = 0;
  NCK(cudaMemcpyAsync(&st, net->status, sizeof st, cudaMemcpyDeviceToHost, net->stream), "status read");
  NCK(cudaStreamSynchronize(net->stream), "net kernels");
  if (st) {
    NCK(cudaMemsetAsync(net->status, 0, sizeof(uint32_t), net->stream), "status clear");
    return err(GPUAI_ERR_LIMIT, "net: a tensor-core kernel gave up waiting (status " + std::to_string(st) + ")");
  }
  return GPUAI_OK;
}

// Glorot-uniform initial parameters from Philox stream (seed, i, 7).
void init_params(std::vector<float> &p, uint64_t seed) {
  p.assign(kParams, 0.0f);
  auto fill = [&](size_t off, uint32_t rows, uint32_t cols, uint32_t used_cols, uint32_t fan_in, uint32_t fan_out) {
    const double bound = std::sqrt(6.0 / (double)(fan_in + fan_out));
    for (uint32_t r = 0; r < rows; r++)
      for (uint32_t c = 0; c < used_cols; c++) {
        const size_t i = off + (size_t)r * cols + c;
        uint32_t ctr[4] = {0u, (uint32_t)i, (uint32_t)(i >> 32), 7u};
        philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
        const double u = (double)(ctr[0] >> 8) * (1.0 / 16777216.0);
        p[i] = (float)((2.0 * u - 1.0) * bound);
      }
  };
  fill(oW1, kH, kInPad, kIn, kIn, kH);
  fill(oW2, kH, kH, kH, kH, kH);
  fill(oW3, kOut, kH, kH, kH, kOut);
  fill(oWV, 1, kH, kH, kH, 1);
}

struct Header {
  char magic[8];
  uint32_t version, features, in_pad, hidden, logits, nparams;
  uint64_t step;
  uint8_t reserved[24];
};
static_assert(sizeof(Header) == 64, "header size");

}  // namespace

int device_of(const gpuai_net *net) { return net->device; }

cudaError_t forward(const gpuai_net *net, Fwd &w, const gpuai_board *boards, uint32_t n, const uint32_t *dev_n,
                    uint32_t *status, cudaStream_t s) {
  return forward_impl(net, w, boards, n, dev_n, dev_n ? w.rows : round128(n), status, false, s);
}

}  // namespace net
}  // namespace ga

using namespace ga::net;

extern "C" {

int gpuai_net_create(int device, uint32_t max_batch, uint64_t init_seed, gpuai_net **out) {
  if (!out) return err(GPUAI_ERR_INVALID, "gpuai_net_create: out is NULL");
  *out = nullptr;
  if (max_batch == 0 || max_batch > (1u << 20))
    return err(GPUAI_ERR_INVALID, "gpuai_net_create: max_batch must be in 1..2^20");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    return err(GPUAI_ERR_NO_DEVICE, "gpuai_net_create: no such CUDA device");
  if (!encode_fn()) return err(GPUAI_ERR_CUDA, "gpuai_net_create: cuTensorMapEncodeTiled unavailable");
  gpuai_net *net = new gpuai_net;
  net->device = device;
  auto fail = [&](int rc) {
    gpuai_net_destroy(net);
    return rc;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(err(GPUAI_ERR_CUDA, "cudaSetDevice failed"));
  // the GEMM's shared-memory ring needs the opt-in limit (set here, outside any stream capture)
  if (cudaFuncSetAttribute(gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit) != cudaSuccess)
    return fail(err(GPUAI_ERR_CUDA, "gpuai_net_create: cannot enable 227 KiB shared memory for the GEMM kernel"));
  const uint32_t L = round128(max_batch);
  net->rows = L;
  auto &A = net->allocs;
  cudaError_t e = cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&net->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&net->side2, cudaStreamNonBlocking);
  for (cudaEvent_t *ev : {&net->ev_loss, &net->ev_b1, &net->ev_b3, &net->ev_side, &net->ev_side2, &net->ev_clear})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = dalloc(A, &net->params, kParams);
  if (e == cudaSuccess) e = dalloc(A, &net->adam_m, kParams);
  if (e == cudaSuccess) e = dalloc(A, &net->adam_v, kParams);
  if (e == cudaSuccess) e = dalloc(A, &net->grad, kParams);
  if (e == cudaSuccess) e = dalloc(A, &net->gout, kParams);
  if (e == cudaSuccess) e = dalloc(A, &net->W1b, (size_t)kH * kInPad);
  if (e == cudaSuccess) e = dalloc(A, &net->W2b, (size_t)kH * kH);
  if (e == cudaSuccess) e = dalloc(A, &net->W3b, (size_t)kOut * kH);
  if (e == cudaSuccess) e = dalloc(A, &net->W2T, (size_t)kH * kH);
  if (e == cudaSuccess) e = dalloc(A, &net->W3T, (size_t)kH * kOut);
  if (e == cudaSuccess) e = fwd_alloc(net->fw, L, A, false);
  if (e == cudaSuccess) e = dalloc(A, &net->Xt, (size_t)kInPad * L);
  if (e == cudaSuccess) e = dalloc(A, &net->H1t, (size_t)kH * L);
  if (e == cudaSuccess) e = dalloc(A, &net->H2t, (size_t)kH * L);
  if (e == cudaSuccess) e = dalloc(A, &net->dZ3, (size_t)L * kOut);
  if (e == cudaSuccess) e = dalloc(A, &net->dZ3t, (size_t)kOut * L);
  if (e == cudaSuccess) e = dalloc(A, &net->dZ2, (size_t)L * kH);
  if (e == cudaSuccess) e = dalloc(A, &net->dZ2t, (size_t)kH * L);
  if (e == cudaSuccess) e = dalloc(A, &net->dZ1t, (size_t)kH * L);
  if (e == cudaSuccess) e = dalloc(A, &net->dv, L);
  if (e == cudaSuccess) e = dalloc(A, &net->rowloss, 2 * (size_t)L);
  if (e == cudaSuccess) e = dalloc(A, &net->loss2, 2);
  if (e == cudaSuccess) e = dalloc(A, &net->value, L);
  if (e == cudaSuccess) e = dalloc(A, &net->p3, (size_t)kSplit3 * kOut * kH);
  if (e == cudaSuccess) e = dalloc(A, &net->p2, (size_t)kMaxSplit2 * kH * kH);
  if (e == cudaSuccess) e = dalloc(A, &net->p1, (size_t)kMaxSplit1 * kH * kInPad);
  if (e == cudaSuccess) e = dalloc(A, &net->status, 1);
  if (e == cudaSuccess) e = dalloc(A, &net->in_boards, L);
  if (e == cudaSuccess) e = dalloc(A, &net->in_z, L);
  if (e == cudaSuccess) e = dalloc(A, &net->in_q, (size_t)L * kMaxMoves);
  if (e != cudaSuccess) return fail(cuda_err(e, "gpuai_net_create: allocation"));
  e = make_map(&net->mW1, net->W1b, kH, kInPad, kBnF1);
  if (e == cudaSuccess) e = make_map(&net->mW2, net->W2b, kH, kH, kBnF2);
  if (e == cudaSuccess) e = make_map(&net->mW2w, net->W2b, kH, kH, 2u * kBnF2);
  if (e == cudaSuccess) e = make_map(&net->mW3, net->W3b, kOut, kH, kBnF3);
  if (e == cudaSuccess) e = make_map(&net->mW2T, net->W2T, kH, kH, kBnB3);
  if (e == cudaSuccess) e = make_map(&net->mW3T, net->W3T, kH, kOut, kBnB1);
  if (e == cudaSuccess) e = make_map(&net->mW2Tn, net->W2T, kH, kH, kBnNarrow);
  if (e == cudaSuccess) e = make_map(&net->mW3Tn, net->W3T, kH, kOut, kBnNarrow);
  if (e == cudaSuccess) e = make_map(&net->mXt, net->Xt, kInPad, L, kBnB5);
  if (e == cudaSuccess) e = make_map(&net->mH1t, net->H1t, kH, L, kBnB4);
  if (e == cudaSuccess) e = make_map(&net->mH2t, net->H2t, kH, L, kBnB2);
  if (e == cudaSuccess) e = make_map(&net->mdZ3, net->dZ3, L, kOut, kBM);
  if (e == cudaSuccess) e = make_map(&net->mdZ3t, net->dZ3t, kOut, L, kBM);
  if (e == cudaSuccess) e = make_map(&net->mdZ2, net->dZ2, L, kH, kBM);
  if (e == cudaSuccess) e = make_map(&net->mdZ2t, net->dZ2t, kH, L, kBM);
  if (e == cudaSuccess) e = make_map(&net->mdZ1t, net->dZ1t, kH, L, kBM);
  if (e != cudaSuccess) return fail(cuda_err(e, "gpuai_net_create: tensor maps"));
  // the transposed activations are read up to the padded batch: start them at zero
  e = cudaMemsetAsync(net->status, 0, sizeof(uint32_t), net->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->Xt, 0, (size_t)kInPad * L * sizeof(bf16), net->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->H1t, 0, (size_t)kH * L * sizeof(bf16), net->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->H2t, 0, (size_t)kH * L * sizeof(bf16), net->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->dZ3, 0, (size_t)L * kOut * sizeof(bf16), net->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(net->dZ3t, 0, (size_t)kOut * L * sizeof(bf16), net->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
  if (e != cudaSuccess) return fail(cuda_err(e, "gpuai_net_create: clear"));
  std::vector<float> p;
  init_params(p, init_seed);
  const int rc = gpuai_net_set_params(net, p.data());
  if (rc) return fail(rc);
  *out = net;
  return GPUAI_OK;
}

void gpuai_net_destroy(gpuai_net *net) {
  if (!net) return;
  cudaSetDevice(net->device);
  if (net->stream) cudaStreamSynchronize(net->stream);
  if (net->side) cudaStreamSynchronize(net->side);
  if (net->side2) cudaStreamSynchronize(net->side2);
  if (net->train_graph) cudaGraphExecDestroy(net->train_graph);
  if (net->train_g) cudaGraphDestroy(net->train_g);
  for (void *p : net->prop_allocs) cudaFree(p);
  if (net->prop_cur) cudaFree(net->prop_cur);
  for (void *p : net->allocs) cudaFree(p);
  for (cudaEvent_t ev : {net->ev_loss, net->ev_b1, net->ev_b3, net->ev_side, net->ev_side2, net->ev_clear})
    if (ev) cudaEventDestroy(ev);
  if (net->side) cudaStreamDestroy(net->side);
  if (net->side2) cudaStreamDestroy(net->side2);
  if (net->stream) cudaStreamDestroy(net->stream);
  delete net;
}

int gpuai_net_get_params(gpuai_net *net, float *params) {
  if (!net || !params) return err(GPUAI_ERR_INVALID, "gpuai_net_get_params: NULL");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  NCK(cudaMemcpyAsync(params, net->params, kParams * sizeof(float), cudaMemcpyDeviceToHost, net->stream), "D2H");
  NCK(cudaStreamSynchronize(net->stream), "D2H");
  return GPUAI_OK;
}

int gpuai_net_set_params(gpuai_net *net, const float *params) {
  if (!net || !params) return err(GPUAI_ERR_INVALID, "gpuai_net_set_params: NULL");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  const cudaStream_t s = net->stream;
  NCK(cudaMemcpyAsync(net->params, params, kParams * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
  NCK(cudaMemsetAsync(net->adam_m, 0, kParams * sizeof(float), s), "clear Adam state");
  NCK(cudaMemsetAsync(net->adam_v, 0, kParams * sizeof(float), s), "clear Adam state");
  net->step = 0;
  NCK(run_adam(net, 2, nullptr, 0.0f, s), "BF16 copies");
  NCK(cudaStreamSynchronize(s), "set params");
  return GPUAI_OK;
}

int gpuai_net_save(gpuai_net *net, const char *path) {
  if (!net || !path) return err(GPUAI_ERR_INVALID, "gpuai_net_save: NULL");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  std::vector<float> buf(3 * kParams);
  const cudaStream_t s = net->stream;
  NCK(cudaMemcpyAsync(buf.data(), net->params, kParams * 4, cudaMemcpyDeviceToHost, s), "D2H");
  NCK(cudaMemcpyAsync(buf.data() + kParams, net->adam_m, kParams * 4, cudaMemcpyDeviceToHost, s), "D2H");
  NCK(cudaMemcpyAsync(buf.data() + 2 * kParams, net->adam_v, kParams * 4, cudaMemcpyDeviceToHost, s), "D2H");
  NCK(cudaStreamSynchronize(s), "D2H");
  Header h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, "GPUAINET", 8);
  h.version = 1;
  h.features = kIn;
  h.in_pad = kInPad;
  h.hidden = kH;
  h.logits = kOut;
  h.nparams = (uint32_t)kParams;
  h.step = net->step;
  FILE *f = std::fopen(path, "wb");
  if (!f) return err(GPUAI_ERR_INVALID, std::string("gpuai_net_save: cannot open ") + path);
  const bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && std::fwrite(buf.data(), 4, buf.size(), f) == buf.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed) return err(GPUAI_ERR_INVALID, std::string("gpuai_net_save: write failed: ") + path);
  return GPUAI_OK;
}

int gpuai_net_load(gpuai_net *net, const char *path) {
  if (!net || !path) return err(GPUAI_ERR_INVALID, "gpuai_net_load: NULL");
  FILE *f = std::fopen(path, "rb");
  if (!f) return err(GPUAI_ERR_INVALID, std::string("gpuai_net_load: cannot open ") + path);
  Header h;
  std::vector<float> buf(3 * kParams);
  const bool ok = std::fread(&h, sizeof h, 1, f) == 1 && std::fread(buf.data(), 4, buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok || std::memcmp(h.magic, "GPUAINET", 8) != 0 || h.version != 1 || h.features != kIn ||
      h.in_pad != kInPad || h.hidden != kH || h.logits != kOut || h.nparams != kParams)
    return err(GPUAI_ERR_INVALID, std::string("gpuai_net_load: not a network file of this layout: ") + path);
  int rc = gpuai_net_set_params(net, buf.data());
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(net->mu);
  const cudaStream_t s = net->stream;
  NCK(cudaMemcpyAsync(net->adam_m, buf.data() + kParams, kParams * 4, cudaMemcpyHostToDevice, s), "H2D");
  NCK(cudaMemcpyAsync(net->adam_v, buf.data() + 2 * kParams, kParams * 4, cudaMemcpyHostToDevice, s), "H2D");
  NCK(cudaStreamSynchronize(s), "H2D");
  net->step = h.step;
  return GPUAI_OK;
}

int gpuai_net_forward(gpuai_net *net, const gpuai_board *boards, uint32_t n, float *value, float *logits) {
  GPUAI_RANGE("gpuai_net_forward");
  if (!net || (n && (!boards || !value))) return err(GPUAI_ERR_INVALID, "gpuai_net_forward: NULL");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  const cudaStream_t s = net->stream;
  for (uint32_t done = 0; done < n;) {
    const uint32_t c = n - done < net->rows ? n - done : net->rows;
    NCK(cudaMemcpyAsync(net->in_boards, boards + done, c * sizeof(gpuai_board), cudaMemcpyHostToDevice, s), "H2D");
    NCK(forward(net, net->fw, net->in_boards, c, nullptr, net->status, s), "forward");
    tanh_kernel<<<(c + 255) / 256, 256, 0, s>>>(net->fw.vraw, c, net->value);
    NCK(cudaGetLastError(), "tanh");
    NCK(cudaMemcpyAsync(value + done, net->value, c * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
    if (logits)
      NCK(cudaMemcpyAsync(logits + (size_t)done * kOut, net->fw.logits, (size_t)c * kOut * sizeof(float),
                          cudaMemcpyDeviceToHost, s),
          "D2H");
    const int rc = check_status(net);
    if (rc) return rc;
    done += c;
  }
  return GPUAI_OK;
}

int gpuai_net_gradients(gpuai_net *net, const gpuai_board *boards, const float *value_target, const float *move_q,
                        uint32_t n, float tau, float value_coef, float *grads, float *loss2) {
  GPUAI_RANGE("gpuai_net_gradients");
  if (!net || !boards || !value_target || !move_q || !grads) return err(GPUAI_ERR_INVALID, "gpuai_net_gradients: NULL");
  if (n == 0 || n > net->rows) return err(GPUAI_ERR_INVALID, "gpuai_net_gradients: n outside 1..max_batch");
  if (!(tau > 0.0f)) return err(GPUAI_ERR_INVALID, "gpuai_net_gradients: tau must be > 0");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  const cudaStream_t s = net->stream;
  NCK(cudaMemcpyAsync(net->in_boards, boards, n * sizeof(gpuai_board), cudaMemcpyHostToDevice, s), "H2D");
  NCK(cudaMemcpyAsync(net->in_z, value_target, n * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
  NCK(cudaMemcpyAsync(net->in_q, move_q, (size_t)n * kMaxMoves * sizeof(float), cudaMemcpyHostToDevice, s), "H2D");
  uint32_t splits[3];
  NCK(clear_dz3_full(net, s), "clear");
  NCK(backward_impl(net, net->in_boards, net->in_z, net->in_q, n, tau, value_coef, splits, s), "backward");
  NCK(run_adam(net, 1, splits, 0.0f, s), "gradient gather");
  NCK(join_clear(net, s), "join");
  NCK(cudaMemcpyAsync(grads, net->gout, kParams * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
  if (loss2) NCK(cudaMemcpyAsync(loss2, net->loss2, 2 * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
  return check_status(net);
}

int gpuai_net_train_step(gpuai_net *net, const gpuai_board *d_boards, const float *d_value_target,
                         const float *d_move_q, uint32_t n, float lr, float tau, float value_coef, float *loss2) {
  GPUAI_RANGE("gpuai_net_train_step");
  if (!net || !d_boards || !d_value_target || !d_move_q) return err(GPUAI_ERR_INVALID, "gpuai_net_train_step: NULL");
  if (n == 0 || n > net->rows) return err(GPUAI_ERR_INVALID, "gpuai_net_train_step: n outside 1..max_batch");
  if (!(tau > 0.0f) || !(lr >= 0.0f)) return err(GPUAI_ERR_INVALID, "gpuai_net_train_step: bad tau or lr");
  if (reinterpret_cast<uintptr_t>(d_boards) % 16 || reinterpret_cast<uintptr_t>(d_value_target) % 4 ||
      reinterpret_cast<uintptr_t>(d_move_q) % 4)
    return err(GPUAI_ERR_INVALID, "gpuai_net_train_step: rows not aligned (boards 16 bytes, values 4)");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  const cudaStream_t s = net->stream;
  // The step's ~25 launches are replayed as one CUDA graph, captured again
  // only when the batch size, tau or the value coefficient change.  Before
  // each replay the graph's kernels that read the rows (features, loss, the
  // clearing of dZ3) get this step's row pointers, and Adam this step's
  // learning rate and bias corrections, as new arguments of their nodes in the
  // instantiated graph: no copy and no launch besides the graph itself.  Same
  // kernels in the same order: same results.
  NCK(clear_dz3_full(net, s), "clear");
  net->step++;
  if (!net->train_graph || net->graph_n != n || net->graph_tau != tau || net->graph_vcoef != value_coef) {
    if (net->train_graph) cudaGraphExecDestroy(net->train_graph);
    if (net->train_g) cudaGraphDestroy(net->train_g);
    net->train_graph = nullptr;
    net->train_g = nullptr;
    cudaGraph_t g = nullptr;
    uint32_t splits[3];
    NCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = backward_impl(net, d_boards, d_value_target, d_move_q, n, tau, value_coef, splits, s);
    if (e == cudaSuccess) e = run_adam(net, 0, splits, lr, s);
    if (e == cudaSuccess) e = join_clear(net, s);
    // nothing ran during the capture: dZ3 / dZ3^T are as the last replay left them
    net->dz_dirty = false;
    const cudaError_t ec = cudaStreamEndCapture(s, &g);
    if (e == cudaSuccess) e = ec;
    if (e == cudaSuccess) e = find_kernel_node(g, (const void *)features_kernel, &net->node_features);
    if (e == cudaSuccess)
      e = find_kernel_node(g, round128(n) > 64u * sm_count() ? (const void *)loss_pairs_kernel : (const void *)loss_kernel,
                           &net->node_loss);
    if (e == cudaSuccess) e = find_kernel_node(g, (const void *)clear_dz3_kernel, &net->node_clear);
    if (e == cudaSuccess) e = find_kernel_node(g, (const void *)adam_kernel, &net->node_adam);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&net->train_graph, g, 0);
    if (e != cudaSuccess && g) cudaGraphDestroy(g);
    NCK(e, "training step graph");
    net->train_g = g;
    net->graph_n = n;
    net->graph_tau = tau;
    net->graph_vcoef = value_coef;
  }
  {
    cudaKernelNodeParams p;
    NCK(cudaGraphKernelNodeGetParams(net->node_adam, &p), "graph update");
    AdamArgs a = *static_cast<const AdamArgs *>(p.kernelParams[0]);
    a.lr = lr;
    a.bc1 = (float)(1.0 - std::pow(0.9, (double)net->step));
    a.bc2 = (float)(1.0 - std::pow(0.999, (double)net->step));
    const cudaGraphExec_t x = net->train_graph;
    NCK(set_node_args(x, net->node_features, nparams(features_kernel), {{0u, &d_boards}}), "graph update");
    NCK(set_node_args(x, net->node_loss, nparams(loss_kernel),
                      {{0u, &d_boards}, {1u, &d_value_target}, {2u, &d_move_q}}),
        "graph update");
    NCK(set_node_args(x, net->node_clear, nparams(clear_dz3_kernel), {{0u, &d_boards}}), "graph update");
    NCK(set_node_args(x, net->node_adam, nparams(adam_kernel), {{0u, &a}}), "graph update");
  }
  NCK(cudaGraphLaunch(net->train_graph, s), "training step");
  if (loss2) {
    NCK(cudaMemcpyAsync(loss2, net->loss2, 2 * sizeof(float), cudaMemcpyDeviceToHost, s), "D2H");
    return check_status(net);
  }
  return GPUAI_OK;
}

int gpuai_net_wait_selftest(gpuai_net *net, uint32_t wait_limit_us, uint32_t *status) {
  if (!net || !status) return err(GPUAI_ERR_INVALID, "gpuai_net_wait_selftest: NULL");
  if (wait_limit_us == 0 || wait_limit_us > 1000000u)
    return err(GPUAI_ERR_INVALID, "gpuai_net_wait_selftest: wait_limit_us must be in 1..1000000");
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  const cudaStream_t s = net->stream;
  // the first layer's GEMM on one 128-row tile, with no TMA load issued: the
  // MMA warp's wait for the first stage runs out after wait_limit_us
  Epi e1;
  e1.flags = kEpiBias | kEpiRelu | kEpiB16;
  e1.bias = net->params + oB1;
  e1.out_b = net->fw.H1;
  e1.ld_b = kH;
  NCK(gemm(net->fw.mX, net->mW1, kBM, kH, kBnF1, kInPad / kBK, 1, nullptr, net->status, e1, s, false,
           (uint64_t)wait_limit_us * 1000u, true),
      "self-test launch");
  uint32_t st = 0;
  NCK(cudaMemcpyAsync(&st, net->status, sizeof st, cudaMemcpyDeviceToHost, s), "status read");
  NCK(cudaStreamSynchronize(s), "self-test kernel");
  NCK(cudaMemsetAsync(net->status, 0, sizeof(uint32_t), s), "status clear");
  NCK(cudaStreamSynchronize(s), "status clear");
  *status = st;
  return GPUAI_OK;
}

int gpuai_playouts_learned(gpuai_ctx *ctx, gpuai_net *net, const gpuai_board *d_pos, const uint32_t *d_offsets,
                           uint32_t npos, uint32_t uniform_reps, uint32_t total, uint64_t seed, uint64_t stream_base,
                           uint32_t guided_plies, float temperature, int8_t *d_out, void *stream,
                           gpuai_board *d_trace_boards, uint16_t *d_trace_logits) {
  GPUAI_RANGE("gpuai_playouts_learned");
  if (!ctx || !net) return err(GPUAI_ERR_INVALID, "gpuai_playouts_learned: ctx or net is NULL");
  if (npos == 0 || total == 0) return GPUAI_OK;
  if (!d_pos || !d_out) return err(GPUAI_ERR_INVALID, "gpuai_playouts_learned: NULL buffer");
  if (guided_plies > kMaxGuidedPlies)
    return err(GPUAI_ERR_INVALID, "gpuai_playouts_learned: guided_plies above " + std::to_string(kMaxGuidedPlies));
  if (!(temperature > 0.0f && temperature < 1.0e6f))
    return err(GPUAI_ERR_INVALID, "gpuai_playouts_learned: temperature must be positive");
  if (!d_offsets && (uint64_t)npos * uniform_reps != total)
    return err(GPUAI_ERR_INVALID, "gpuai_playouts_learned: total != npos * uniform_reps");
  if (total > 0x7fffffffu) return err(GPUAI_ERR_INVALID, "gpuai_playouts_learned: more than 2^31-1 playouts");
  if (guided_plies == 0)
    return gpuai_playouts_device(ctx, d_pos, d_offsets, npos, uniform_reps, total, seed, stream_base,
                                 GPUAI_POLICY_RANDOM, d_out, stream);
  std::lock_guard<std::mutex> lock(net->mu);
  NCK(cudaSetDevice(net->device), "cudaSetDevice");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  // workspace: logits for the positions (first guided ply) and for the playouts (later plies)
  const uint32_t need_rows = round128(guided_plies > 1 && total > npos ? total : npos);
  if (net->prop_fw.rows < need_rows || net->prop_cur_cap < total) {
    NCK(cudaDeviceSynchronize(), "workspace");
    for (void *p : net->prop_allocs) cudaFree(p);
    net->prop_allocs.clear();
    net->prop_fw = Fwd();
    if (net->prop_cur) cudaFree(net->prop_cur);
    net->prop_cur = nullptr;
    net->prop_cur_cap = 0;
    NCK(fwd_alloc(net->prop_fw, need_rows, net->prop_allocs, true), "proposal workspace");
    NCK(cudaMalloc(&net->prop_cur, (size_t)total * sizeof(ga::Board)), "proposal boards");
    net->prop_cur_cap = total;
  }
  Fwd &W = net->prop_fw;
  NCK(forward(net, W, d_pos, npos, nullptr, net->status, s), "forward on the positions");
  ga::ProposalArgs a{};
  a.in = reinterpret_cast<const ga::Board *>(d_pos);
  a.offsets = d_offsets;
  a.npos = npos;
  a.uniform_reps = uniform_reps;
  a.total = total;
  a.per_position = true;
  a.logits = reinterpret_cast<const uint16_t *>(W.logits_b);
  a.seed = seed;
  a.stream_base = stream_base;
  a.inv_temperature = 1.0f / temperature;
  a.out = net->prop_cur;
  for (uint32_t g = 0; g < guided_plies; g++) {
    if (g > 0) {
      NCK(forward(net, W, reinterpret_cast<const gpuai_board *>(net->prop_cur), total, nullptr, net->status, s),
          "forward on the playouts");
      a.in = net->prop_cur;
      a.per_position = false;
      a.offsets = nullptr;
    }
    a.ply = g;
    a.trace_boards = d_trace_boards ? reinterpret_cast<ga::Board *>(d_trace_boards) + (size_t)g * total : nullptr;
    a.trace_logits = d_trace_logits ? d_trace_logits + (size_t)g * total * kOut : nullptr;
    NCK(ga::launch_proposal_ply(a, s), "guided ply");
  }
  return gpuai_playouts_device(ctx, reinterpret_cast<const gpuai_board *>(net->prop_cur), nullptr, total, 1, total,
                               seed, stream_base, GPUAI_POLICY_RANDOM, d_out, stream);
}

int gpuai_label_positions(gpuai_ctx *ctx, const gpuai_board *d_pos, uint32_t n, uint32_t playouts_per_position,
                          uint64_t seed, uint64_t stream_base, int32_t policy, float *d_value, float *d_move_q,
                          uint8_t *d_nmoves, void *stream) {
  GPUAI_RANGE("gpuai_label_positions");
  if (!ctx) return err(GPUAI_ERR_INVALID, "gpuai_label_positions: ctx is NULL");
  if (n == 0) return GPUAI_OK;
  if (!d_pos || !d_value || !d_move_q || !d_nmoves) return err(GPUAI_ERR_INVALID, "gpuai_label_positions: NULL");
  const uint32_t P = playouts_per_position;
  if (P < kMaxMoves) return err(GPUAI_ERR_INVALID, "gpuai_label_positions: playouts_per_position must be >= 32");
  if ((uint64_t)n * P >= 0x7fffffffull || (uint64_t)n * kLabelSlots >= 0x7fffffffull)
    return err(GPUAI_ERR_INVALID, "gpuai_label_positions: n * playouts_per_position must stay below 2^31");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  ga::Board *children = nullptr;
  uint32_t *offsets = nullptr;
  int8_t *out = nullptr;
  const size_t nc = (size_t)n * kLabelSlots;
  NCK(cudaMallocAsync(reinterpret_cast<void **>(&children), nc * sizeof(ga::Board), s), "label scratch");
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&offsets), (nc + 1) * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void **>(&out), (size_t)n * P, s);
  int rc = GPUAI_OK;
  if (e != cudaSuccess) {
    rc = cuda_err(e, "label scratch");
  } else {
    label_children_kernel<<<(n + 127) / 128, 128, 0, s>>>(d_pos, n, P, children, offsets, d_nmoves);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_err(e, "label children");
  }
  if (rc == GPUAI_OK)
    rc = gpuai_playouts_device(ctx, reinterpret_cast<const gpuai_board *>(children), offsets, (uint32_t)nc, 0,
                               n * P, seed, stream_base, policy, out, stream);
  if (rc == GPUAI_OK) {
    label_reduce_kernel<<<(n + 3) / 4, 128, 0, s>>>(d_pos, out, offsets, d_nmoves, n, P, d_value, d_move_q);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_err(e, "label reduce");
  }
  if (out) cudaFreeAsync(out, s);
  if (offsets) cudaFreeAsync(offsets, s);
  if (children) cudaFreeAsync(children, s);
  return rc;
}

}  // extern "C"
