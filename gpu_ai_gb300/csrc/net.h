// net.h -- the policy/value network inside libgpuai: sizes, parameter
// layout, and the forward pass other translation units (the learned
// searches) run on their own workspaces.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/gpuai.h"

namespace ga {
namespace net {

constexpr uint32_t kIn = 129;      // features
constexpr uint32_t kInPad = 192;   // padded to whole 64-wide K blocks
constexpr uint32_t kH = 256;       // hidden units per layer
constexpr uint32_t kOut = 1024;    // move logits, index from*32 + to
constexpr uint32_t kMaxMoves = 32; // moves per position the policy covers

// FP32 parameter layout (gpuai.h, GPUAI_NET_PARAMS).
constexpr size_t oW1 = 0;
constexpr size_t oB1 = oW1 + (size_t)kH * kInPad;
constexpr size_t oW2 = oB1 + kH;
constexpr size_t oB2 = oW2 + (size_t)kH * kH;
constexpr size_t oW3 = oB2 + kH;
constexpr size_t oB3 = oW3 + (size_t)kOut * kH;
constexpr size_t oWV = oB3 + kOut;
constexpr size_t oBV = oWV + kH;
constexpr size_t kParams = oBV + 1;
static_assert(kParams == GPUAI_NET_PARAMS, "parameter count");

constexpr uint32_t kMaxGuidedPlies = 32;  // learned-proposal plies per playout at most
constexpr uint32_t kStatusNetWait = 16u;  // a tensor-core kernel gave up waiting (status bit)

// Forward workspace for up to `rows` boards (a multiple of 128).
struct Fwd {
  uint32_t rows = 0;
  __nv_bfloat16 *X = nullptr, *H1 = nullptr, *H2 = nullptr;
  float *logits = nullptr, *vraw = nullptr;  // FP32 logits (training, host forward) ...
  __nv_bfloat16 *logits_b = nullptr;         // ... or BF16 logits (search leaves: priors only)
  float *vpart = nullptr;                    // [2][rows] value-head sums of F2's two column tiles
  CUtensorMap mX, mH1, mH2;
};

// CUDA device the network lives on.
int device_of(const gpuai_net *net);

// Allocates a workspace (device allocations appended to `allocs`); the logits
// are stored in BF16 when bf16_logits is set, else in FP32.
cudaError_t fwd_alloc(Fwd &w, uint32_t rows, std::vector<void *> &allocs, bool bf16_logits);

// Features, three GEMMs: w.logits or w.logits_b (rows x 1024, bias added) and w.vraw (the
// value before tanh) for boards[0..n).  With dev_n set, n is read from device
// memory (launches inside a CUDA graph); tiles past it do no work.
cudaError_t forward(const gpuai_net *net, Fwd &w, const gpuai_board *boards, uint32_t n, const uint32_t *dev_n,
                    uint32_t *status, cudaStream_t s);

}  // namespace net
}  // namespace ga
