// div_by_recip (graph_gb300/csrc/common.cuh) against __fdiv_rn on sampled
// operand pairs of the ranges the kernels use it for: |a| in [2^-100, 2^94]
// log-uniform, b in [1, 2^26] log-uniform plus exact powers of two, y = RN(1/b).
// The spring quotient (l - d) / l, the same where spring_quotient_in_range
// holds: l log-uniform in [2^-4, 2^30], the rest length d = l * u with u in
// [0.5, 1.0101) or d = l (a zero numerator).
// Prints "pairs=<n> mismatches=<m> spring=<in range>/<m>"; exit status 0 when
// it ran.
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

__global__ void check_spring(unsigned long long* bad, uint32_t salt, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = salt * n + i;
  const float l = exp2f(-4.f + 34.f * unit(3 * k));
  const float dd = (mix(3 * k + 2) & 31) == 0 ? l : __fmul_rn(l, 0.5f + 0.5101f * unit(3 * k + 1));
  const float a = __fsub_rn(l, dd);
  if (!cgl::spring_quotient_in_range(a, l)) return;
  atomicAdd(&bad[1], 1ull);   // pairs in range
  if (__float_as_uint(cgl::div_by_recip(a, l, cgl::recip_in_range(l))) != __float_as_uint(__fdiv_rn(a, l)))
    atomicAdd(&bad[0], 1ull);
}

int main(int argc, char** argv) {
  const uint32_t n = 1u << 24;
  const int rounds = argc > 1 ? atoi(argv[1]) : 16;
  unsigned long long* bad;
  if (cudaMalloc(&bad, 24) != cudaSuccess) return 1;
  cudaMemset(bad, 0, 24);
  for (int r = 0; r < rounds; ++r) check<<<n / 256, 256>>>(bad, (uint32_t)r, n);
  for (int r = 0; r < rounds; ++r) check_spring<<<n / 256, 256>>>(bad + 1, (uint32_t)r, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 1;
  unsigned long long h[3] = {0, 0, 0};
  cudaMemcpy(h, bad, 24, cudaMemcpyDeviceToHost);
  printf("pairs=%llu mismatches=%llu spring=%llu/%llu\n", (unsigned long long)n * rounds, h[0], h[2], h[1]);
  return 0;
}
