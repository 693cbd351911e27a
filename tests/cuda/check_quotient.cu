// div_by_recip (graph_gb300/csrc/common.cuh) against __fdiv_rn on sampled
// operand pairs of the ranges the kernels use it for: |a| in [2^-100, 2^94]
// log-uniform, b in [1, 2^26] log-uniform plus exact powers of two, y = RN(1/b).
// Prints "pairs=<n> mismatches=<m>"; exit status 0 when it ran.
#include <cstdio>
#include <cstdint>

#include "../../graph_gb300/csrc/common.cuh"

__device__ uint32_t mix(uint32_t x) { return cgl::lowbias32(x * 0x9E3779B9u + 0x7F4A7C15u); }
__device__ float unit(uint32_t k) { return (mix(k) >> 8) * (1.0f / 16777216.0f); }

__global__ void check(unsigned long long* bad, uint32_t salt, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = salt * n + i;
  float a = exp2f(-100.f + 194.f * unit(4 * k));
  if (mix(4 * k + 3) & 1) a = -a;
  float b = exp2f(26.f * unit(4 * k + 1));
  if ((mix(4 * k + 2) & 63) == 0) b = exp2f((float)(mix(k) % 27));
  const float y = __frcp_rn(b);
  if (__float_as_uint(cgl::div_by_recip(a, b, y)) != __float_as_uint(__fdiv_rn(a, b))) atomicAdd(bad, 1ull);
}

int main(int argc, char** argv) {
  const uint32_t n = 1u << 24;
  const int rounds = argc > 1 ? atoi(argv[1]) : 16;
  unsigned long long* bad;
  if (cudaMalloc(&bad, 8) != cudaSuccess) return 1;
  cudaMemset(bad, 0, 8);
  for (int r = 0; r < rounds; ++r) check<<<n / 256, 256>>>(bad, (uint32_t)r, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 1;
  unsigned long long h = 0;
  cudaMemcpy(&h, bad, 8, cudaMemcpyDeviceToHost);
  printf("pairs=%llu mismatches=%llu\n", (unsigned long long)n * rounds, h);
  return 0;
}
