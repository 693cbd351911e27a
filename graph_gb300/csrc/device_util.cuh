// device_util.cuh — warp/block primitives and the near-field slot selection
// shared by the plain and the batched tick kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace cgl {

constexpr int kBlock = 256;

// Streaming multiprocessors of the current device.
inline uint32_t sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? (uint32_t)sms : 1u;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

static __device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_tot[kBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < (kBlock / 32) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < (kBlock / 32)) warp_tot[lane] = t;
  }
  __syncthreads();
  const uint32_t before = w > 0 ? warp_tot[w - 1] : 0;
  *total = warp_tot[kBlock / 32 - 1];
  __syncthreads();
  return before + x - v;
}

// The same for 64-bit values (the scan of packed (count, pairs) cell words).
static __device__ unsigned long long block_exclusive_scan64(unsigned long long v, unsigned long long* total) {
  __shared__ unsigned long long warp_tot64[kBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot64[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned long long t = lane < (kBlock / 32) ? warp_tot64[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < (kBlock / 32)) warp_tot64[lane] = t;
  }
  __syncthreads();
  const unsigned long long before = w > 0 ? warp_tot64[w - 1] : 0;
  *total = warp_tot64[kBlock / 32 - 1];
  __syncthreads();
  return before + x - v;
}

// Single-pass scans (decoupled look-back, Merrill and Garland 2016): each
// block takes the next chunk in the order blocks start (a ticket), so every
// chunk before its own belongs to a block that has already started.  The block publishes
// its chunk's total, then warp 0 walks back over the status words of the
// chunks before it, adding totals until it meets a chunk whose inclusive
// prefix is known; the block then publishes its own inclusive prefix.  A
// status word holds the value in its low 60 bits, a flag for "total" or
// "inclusive prefix", and the parity of the pass (the ticket / blocks), so a
// word left from the previous tick never reads as current.
constexpr unsigned long long kScanTotal = 1ull << 61, kScanInclusive = 1ull << 62, kScanParity = 1ull << 63;
constexpr unsigned long long kScanValue = (1ull << 60) - 1;
constexpr uint32_t kScanPollLimit = 1u << 20;   // ~0.1 s of polls: far beyond any wait on a started block

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// The exclusive prefix of chunk `vb` (> 0) from the status words of chunks
// [0, vb); warp 0 of the block, every lane gets it.  A wait that outlasts
// kScanPollLimit polls sets `error_bit` in *error and returns what it has.
static __device__ unsigned long long scan_look_back(const unsigned long long* status, uint32_t vb,
                                                    unsigned long long parity, uint32_t* error, uint32_t error_bit) {
  const int lane = threadIdx.x & 31;
  unsigned long long prefix = 0;
  int end = (int)vb;   // this round looks at chunks end - 1 - lane
  for (uint32_t polls = 0;;) {
    const int i = end - 1 - lane;
    const unsigned long long w = i >= 0 ? ld_relaxed_u64(&status[i]) : (parity | kScanInclusive);
    const bool current = (w & kScanParity) == parity && (w & (kScanTotal | kScanInclusive));
    const unsigned ready = __ballot_sync(0xffffffffu, current);
    const unsigned incl = __ballot_sync(0xffffffffu, current && (w & kScanInclusive));
    // the lanes up to and including the nearest chunk with an inclusive prefix
    const unsigned need = incl ? (incl ^ (incl - 1u)) : 0xffffffffu;
    if ((ready & need) == need) {
      unsigned long long x = ((need >> lane) & 1u) ? (w & kScanValue) : 0ull;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      prefix += x;
      if (incl) return prefix;
      end -= 32;
      continue;
    }
    if (++polls > kScanPollLimit) {
      if (lane == 0) atomicOr(error, error_bit);
      return prefix;
    }
    __nanosleep(64);
  }
}

// Insert (hash bits, index) into a sorted list of the 8 smallest DISTINCT
// hashes, each kept with its lowest index (the peel's tie rule,
// build-nearfield-slots.vert:146-162); `at` tracks segment positions.
__device__ __forceinline__ void top8_insert(unsigned long long (&best)[kSlots], uint32_t (&at)[kSlots],
                                            unsigned long long key, uint32_t pos) {
  const uint32_t hb = (uint32_t)(key >> 32);
  bool dup = false;
#pragma unroll
  for (int q = 0; q < kSlots; ++q) {
    if ((uint32_t)(best[q] >> 32) == hb && best[q] != ~0ull) {
      dup = true;
      if (key < best[q]) { best[q] = key; at[q] = pos; }
    }
  }
  if (!dup && key < best[kSlots - 1]) {
#pragma unroll
    for (int q = 0; q < kSlots; ++q) {
      if (key < best[q]) {
        unsigned long long tk = best[q]; best[q] = key; key = tk;
        uint32_t ta = at[q]; at[q] = pos; pos = ta;
      }
    }
  }
}

// The slot selection of one warp cell from candidates held in registers, up
// to 4 per lane: hash bits (~0u: none; hashes lie in [0, 1), so no hash has
// those bits), point index and segment position.  Round k takes the smallest
// hash above the last one taken, then the lowest index among the keys with
// that hash: the order of the keys (hash << 32 | index) that top8_insert
// keeps, found with two 32-bit warp minimums (redux) per round.
__device__ __forceinline__ int warp_select_slots(const uint32_t (&hb)[4], const uint32_t (&ix)[4],
                                                 const uint32_t (&at)[4], uint32_t (&sel)[kSlots]) {
  int ns = 0;
  uint32_t last = 0;
#pragma unroll
  for (int k = 0; k < kSlots; ++k) sel[k] = 0;
#pragma unroll
  for (int k = 0; k < kSlots; ++k) {
    uint32_t mh = ~0u;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if ((k == 0 || hb[u] > last) && hb[u] < mh) mh = hb[u];
    const uint32_t gh = __reduce_min_sync(0xffffffffu, mh);
    if (gh == ~0u) break;   // warp-uniform: no hash left
    uint32_t mi = ~0u;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (hb[u] == gh && ix[u] < mi) mi = ix[u];
    const uint32_t gi = __reduce_min_sync(0xffffffffu, mi);
    uint32_t mp = 0;
    bool has = false;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (hb[u] == gh && ix[u] == gi) { mp = at[u]; has = true; }
    sel[k] = __shfl_sync(0xffffffffu, mp, __ffs(__ballot_sync(0xffffffffu, has)) - 1);
    ns = k + 1;
    last = gh;
  }
  return ns;
}

__device__ __forceinline__ unsigned long long peel_key(uint32_t idx, uint32_t seed_bits) {
  return ((unsigned long long)__float_as_uint(peel_hash(idx, seed_bits)) << 32) | idx;
}

}  // namespace cgl
