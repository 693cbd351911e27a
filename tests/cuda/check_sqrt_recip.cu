// sqrt_in_range and recip_in_range (graph_gb300/csrc/common.cuh) against
// __fsqrt_rn and __frcp_rn on EVERY float of the ranges the many-body kernels
// use them for: l in [1, 2^52] and b in [1, 2^26], end points included.
// Prints "sqrt=<checked>/<mismatches> recip=<checked>/<mismatches>"; exit
// status 0 when it ran.
#include <cstdio>
#include <cstdint>

#include "../../graph_gb300/csrc/common.cuh"

__global__ void check(unsigned long long* bad, uint32_t n_sqrt, uint32_t n_recip) {
  unsigned long long bs = 0, br = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_sqrt; i += stride) {
    const float l = __uint_as_float(0x3F800000u + i);
    if (__float_as_uint(cgl::sqrt_in_range(l)) != __float_as_uint(__fsqrt_rn(l))) ++bs;
    if (i < n_recip && __float_as_uint(cgl::recip_in_range(l)) != __float_as_uint(__frcp_rn(l))) ++br;
  }
  if (bs) atomicAdd(&bad[0], bs);
  if (br) atomicAdd(&bad[1], br);
}

int main() {
  const uint32_t n_sqrt = (52u << 23) + 1, n_recip = (26u << 23) + 1;   // through 2^52 and 2^26
  unsigned long long* bad;
  if (cudaMalloc(&bad, 16) != cudaSuccess) return 1;
  cudaMemset(bad, 0, 16);
  check<<<152 * 16, 256>>>(bad, n_sqrt, n_recip);
  if (cudaDeviceSynchronize() != cudaSuccess) return 1;
  unsigned long long h[2] = {0, 0};
  cudaMemcpy(h, bad, 16, cudaMemcpyDeviceToHost);
  printf("sqrt=%u/%llu recip=%u/%llu\n", n_sqrt, h[0], n_recip, h[1]);
  return 0;
}
