// curand_pin.cu -- TEST INFRASTRUCTURE: the project's Philox4x32-10 against
// cuRAND's Philox4_32_10 generator on the GPU.
//
// Draw k of the project's stream (seed, id, tag) is word k & 3 of
// philox4x32_10(counter = {k >> 2, id_lo, id_hi, tag}, key = {seed_lo, seed_hi})
// (gpu_ai_gb300/csrc/rules.cuh).  cuRAND's generator initialised with
// curand_init(seed, subsequence, offset) starts at the counter whose low 64
// bits are offset / 4 and whose high 64 bits are the subsequence, with the key
// taken from the seed; so subsequence = tag << 32 | id_hi and an offset of
// 4 * (id_lo << 32 | k >> 2) draws (reached with skipahead, as it can exceed
// 64 bits) put the two on the same block, and curand4() returns that block's
// four words.
//
//   curand_pin [cases]   prints "cases N mismatches M" and exits 1 if M > 0
#include <curand_kernel.h>

#include <cstdio>
#include <cstdlib>

#include "rules.cuh"

__device__ __forceinline__ unsigned long long mix(unsigned long long z) {  // splitmix64
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void pin_kernel(unsigned n, unsigned *mismatches, unsigned *first) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long seed = mix(3 * i), id = mix(3 * i + 1);
  const unsigned long long r = mix(3 * i + 2);
  const unsigned block = (unsigned)(r & 0xffffffu), tag = (unsigned)((r >> 32) & 3u);
  unsigned c[4] = {block, (unsigned)id, (unsigned)(id >> 32), tag};
  ga::philox4x32_10(c, (unsigned)seed, (unsigned)(seed >> 32));
  curandStatePhilox4_32_10_t st;
  curand_init(seed, ((unsigned long long)tag << 32) | (id >> 32), 0ull, &st);
  // offset 4 * (id_lo << 32 | block) draws, which can exceed 64 bits: id_lo << 32
  // draws four times (each adds id_lo << 30 blocks), then 4 * block
  const unsigned long long hi = ((unsigned long long)(unsigned)id) << 32;
  for (int q = 0; q < 4; q++) skipahead(hi, &st);
  skipahead(4ull * block, &st);
  const uint4 v = curand4(&st);
  if (v.x != c[0] || v.y != c[1] || v.z != c[2] || v.w != c[3]) {
    if (atomicAdd(mismatches, 1u) == 0u) *first = i;
  }
}

int main(int argc, char **argv) {
  const unsigned n = argc > 1 ? (unsigned)strtoul(argv[1], nullptr, 10) : (1u << 20);
  unsigned *d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned)) != cudaSuccess) return 2;
  cudaMemset(d, 0, 2 * sizeof(unsigned));
  pin_kernel<<<(n + 255) / 256, 256>>>(n, d, d + 1);
  unsigned h[2] = {0, 0};
  if (cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) {
    printf("CUDA error: %s\n", cudaGetErrorString(cudaGetLastError()));
    return 2;
  }
  cudaFree(d);
  printf("cases %u mismatches %u first %u\n", n, h[0], h[0] ? h[1] : 0u);
  return h[0] ? 1 : 0;
}
