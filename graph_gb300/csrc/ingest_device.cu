// ingest_device.cu — ForceLink.create for both directions built on the device
// from the raw setLinks array: the same CSR, random draws, bias and strength as
// the host build in ingest.h (ForceLink/index.ts:40-83, GraphData/index.ts:
// 525-568), bit for bit.
//
// The host build visits links in index order; here:
//   1. one pass over the links marks the valid ones (GraphData.isPointIndex)
//      and counts each point's incoming and outgoing list (integer atomics,
//      order-free);
//   2. a stable compaction keeps the valid links in index order;
//   3. a stable LSD radix sort by row (8-bit digits) puts each direction's
//      entries in row order, link-index order within a row — the list order
//      of GraphData._createAdjacencyLists;
//   4. one pass fills the entries: entry `at` of the incoming CSR takes random
//      draw base + at, of the outgoing CSR base + M + at (SplitMix64 is
//      counter-based, so a draw needs no predecessor); bias and strength are
//      the same FP64 expressions, correctly rounded (__ddiv_rn, __dsqrt_rn),
//      rounded to f32;
//   5. the rows ordered by list length, longest first, ties by index (the
//      launch order of the link kernel), by the same stable sort.
// The many-body jitter texture is drawn the same way (draws 2t and 2t + 1 of
// texel t), so it too needs no sequential pass.
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "device_util.cuh"
#include "ingest_device.cuh"

namespace cgl {
namespace dingest {

namespace {

constexpr uint32_t kScanPer = kBlock * 4;             // elements per scan block
constexpr int kSortItems = 8;                          // items per thread per tile
constexpr uint32_t kSortTile = kBlock * kSortItems;    // 2048
constexpr int kWarps = kBlock / 32;

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

// ------------------------------------------------------------------ scan --
__global__ void __launch_bounds__(kBlock) k_scan_local(uint32_t* d, uint32_t n, uint32_t* sums) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanPer + threadIdx.x * 4u;
  uint32_t v[4], s = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    v[j] = base + j < n ? d[base + j] : 0u;
    s += v[j];
  }
  uint32_t total;
  uint32_t ex = block_exclusive_scan(s, &total);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (base + j < n) d[base + j] = ex;
    ex += v[j];
  }
  if (threadIdx.x == 0 && sums) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kBlock) k_scan_add(uint32_t* d, uint32_t n, const uint32_t* sums) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanPer + threadIdx.x * 4u;
  const uint32_t add = sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (base + j < n) d[base + j] += add;
}

// ----------------------------------------------------------- radix sort --
// Digit counts of each tile, digit-major: hist[digit * tiles + tile], so that
// one exclusive scan gives every (digit, tile) its first output position.
__global__ void __launch_bounds__(kBlock) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                    uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const uint64_t i = base + (uint64_t)r * kBlock + threadIdx.x;
    const bool valid = i < n;
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const uint32_t dgt = (keys[i] >> shift) & 255u;
      const unsigned peers = __match_any_sync(vm, dgt);
      if (lane == __ffs(peers) - 1) atomicAdd(&h[dgt], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: item i of a tile goes to (first position of its digit in
// this tile) + (items of the same digit before it in the tile).  A tile is
// processed in kSortItems rounds of kBlock consecutive items; within a round
// the lanes of a warp rank by __match_any_sync and the warps by a prefix over
// per-warp digit counts.
__global__ void __launch_bounds__(kBlock) k_rs_scatter(const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                                                       uint32_t* __restrict__ vout, uint32_t n, int shift,
                                                       const uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t off[256];
  __shared__ uint32_t wcnt[kWarps][256];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  off[t] = hist[(size_t)t * tiles + blockIdx.x];
  const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
    const uint64_t i = base + (uint64_t)r * kBlock + t;
    const bool valid = i < n;
    uint32_t k = 0, v = 0, dgt = 0, rank = 0;
    if (valid) {
      k = kin[i];
      v = vin[i];
      dgt = (k >> shift) & 255u;
    }
#pragma unroll
    for (int x = 0; x < kWarps; ++x) wcnt[x][t] = 0;
    __syncthreads();
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const unsigned peers = __match_any_sync(vm, dgt);
      rank = __popc(peers & ((1u << lane) - 1u));
      if (lane == __ffs(peers) - 1) wcnt[w][dgt] = __popc(peers);
    }
    __syncthreads();
    {   // thread t owns digit t: exclusive prefix over the warps, then the tile's running offset
      uint32_t run = off[t];
#pragma unroll
      for (int x = 0; x < kWarps; ++x) {
        const uint32_t c = wcnt[x][t];
        wcnt[x][t] = run;
        run += c;
      }
      off[t] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = wcnt[w][dgt] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------- links --
// GraphData.isPointIndex (GraphData/index.ts:286-289) on an f32 value: finite,
// integral, 0 <= v < n (n <= 2^24 is exact in f32).
__device__ __forceinline__ bool point_index(float v, uint32_t n) {
  return v == floorf(v) && v >= 0.f && v < (float)n;
}

__global__ void __launch_bounds__(kBlock) k_links_count(const float2* __restrict__ links, uint32_t E, uint32_t N,
                                                        uint32_t* __restrict__ valid, uint32_t* __restrict__ len_in,
                                                        uint32_t* __restrict__ len_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  const float2 l = links[i];
  const bool ok = point_index(l.x, N) && point_index(l.y, N);
  valid[i] = ok;
  if (ok) {
    atomicAdd(&len_in[(uint32_t)l.x], 1u);    // incoming list of the source (:534-547)
    atomicAdd(&len_out[(uint32_t)l.y], 1u);   // outgoing list of the target
  }
}

// pos[0..E] = exclusive scan of the valid flags with a trailing 0, so link i
// is valid exactly when pos[i + 1] != pos[i]; valid links keep index order.
__global__ void __launch_bounds__(kBlock) k_links_compact(const float2* __restrict__ links, uint32_t E,
                                                          const uint32_t* __restrict__ pos,
                                                          uint32_t* __restrict__ key_in, uint32_t* __restrict__ key_out,
                                                          uint32_t* __restrict__ val_in, uint32_t* __restrict__ val_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  const uint32_t p = pos[i];
  if (pos[i + 1] == p) return;
  const float2 l = links[i];
  key_in[p] = (uint32_t)l.x;
  key_out[p] = (uint32_t)l.y;
  val_in[p] = i;
  val_out[p] = i;
}

__device__ __forceinline__ uint64_t splitmix_draw(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One entry of a direction's CSR (ForceLink/index.ts:57-76): neighbour (or the
// absent sentinel), the f32 random rest-length draw, bias and strength.  The
// draw is draws[at] when the host drew the graph's values (the reference's
// sequential stream), else counter draw draw_base + at of `seed`.
__global__ void __launch_bounds__(kBlock) k_csr_fill(const uint32_t* __restrict__ rows, const uint32_t* __restrict__ lidx,
                                                     uint32_t M, const float2* __restrict__ links, int incoming,
                                                     const uint32_t* __restrict__ len_in,
                                                     const uint32_t* __restrict__ len_out,
                                                     const float* __restrict__ strength,
                                                     const uint8_t* __restrict__ flags,
                                                     const float* __restrict__ draws, uint64_t seed,
                                                     uint64_t draw_base, uint32_t point_off, uint4* __restrict__ ent) {
  const uint32_t at = blockIdx.x * blockDim.x + threadIdx.x;
  if (at >= M) return;
  const uint32_t i = lidx[at], p = rows[at];
  const float2 l = links[i];
  const uint32_t q = (uint32_t)(incoming ? l.y : l.x);
  const double degree = (double)(len_in[q] + len_out[q]), connected = (double)(len_in[p] + len_out[p]);
  const double sum = __dadd_rn(degree, connected);
  const double bias = sum != 0.0 ? __ddiv_rn(degree, sum) : 0.5;
  const double mind = degree < connected ? degree : connected;
  const double si = strength ? (double)strength[i] : 0.0;
  double st;
  if (!strength || !isfinite(si) || si < 0.0) st = __ddiv_rn(1.0, mind < 1.0 ? 1.0 : mind);
  else st = si;
  st = __dsqrt_rn(st);
  float r;
  if (draws) {
    r = draws[at];
  } else {
    // Random.float(0, 1) = u * (1 - 0) + 0, u = top 53 bits / 2^53 (exact), rounded to f32
    const double u = (double)(splitmix_draw(seed, draw_base + at) >> 11) * 0x1.0p-53;
    r = __double2float_rn(u);
  }
  ent[at] = make_uint4((flags[q] & kAbsent) ? kAbsentTarget : q + point_off, __float_as_uint(r),
                       __float_as_uint(__double2float_rn(bias)), __float_as_uint(__double2float_rn(st)));
}

// key = longest - length (so that a stable ascending sort lists the longest
// first), value = point; plus the longest list and the rows above kHeavyDegree.
__global__ void __launch_bounds__(kBlock) k_len_stats(const uint32_t* __restrict__ len, uint32_t N,
                                                      uint32_t* __restrict__ stats /* [max, heavy] */) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t m = 0, h = 0;
  if (p < N) {
    m = len[p];
    h = m > kHeavyDegree;
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    h += __shfl_xor_sync(0xffffffffu, h, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (m) atomicMax(&stats[0], m);
    if (h) atomicAdd(&stats[1], h);
  }
}

__global__ void __launch_bounds__(kBlock) k_len_keys(const uint32_t* __restrict__ len, uint32_t N,
                                                     const uint32_t* __restrict__ stats, uint32_t* __restrict__ key,
                                                     uint32_t* __restrict__ val) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  key[p] = stats[0] - len[p];
  val[p] = p;
}

// ForceManyBody.create jitter (ForceManyBody/index.ts:133-138): texel t takes
// draws base + 2t and base + 2t + 1, each Random.float(-1, 1) * 0.00001 in FP64
// (-1 + 2u, then the product), rounded to f32.
__global__ void __launch_bounds__(kBlock) k_jitter(uint64_t seed, uint64_t base, uint32_t n, float2* __restrict__ out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float r[2];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const double u = (double)(splitmix_draw(seed, base + 2ull * t + c) >> 11) * 0x1.0p-53;
    r[c] = __double2float_rn(__dmul_rn(__dadd_rn(-1.0, __dmul_rn(2.0, u)), 0.00001));
  }
  out[t] = make_float2(r[0], r[1]);
}

__global__ void k_copy_u32(const uint32_t* __restrict__ a, uint32_t* __restrict__ b, uint32_t n, uint32_t add) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i] + add;
}

}  // namespace

// ------------------------------------------------------------ host side --
size_t scan_temp_words(uint64_t n) {
  size_t w = 0;
  while (n > kScanPer) {
    n = ceil_div(n, kScanPer);
    w += n;
  }
  return w + 4;
}

void scan_exclusive(uint32_t* d, uint32_t n, uint32_t* tmp, cudaStream_t st) {
  if (n == 0) return;
  const uint32_t nb = ceil_div(n, kScanPer);
  if (nb == 1) {
    k_scan_local<<<1, kBlock, 0, st>>>(d, n, nullptr);
    return;
  }
  k_scan_local<<<nb, kBlock, 0, st>>>(d, n, tmp);
  scan_exclusive(tmp, nb, tmp + nb, st);
  k_scan_add<<<nb, kBlock, 0, st>>>(d, n, tmp);
}

size_t sort_temp_words(uint64_t n) {
  const uint64_t tiles = ceil_div(n, kSortTile);
  return 2 * n + 256 * tiles + scan_temp_words(256 * tiles);
}

int key_bits(uint64_t max_key) {
  int b = 0;
  while (b < 32 && (max_key >> b)) ++b;
  return b;
}

// Stable sort of (keys, vals) by the low `bits` bits of the keys; the result is
// left in (keys, vals).  tmp holds sort_temp_words(n) words.
void sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, uint32_t* tmp, cudaStream_t st) {
  if (n <= 1 || bits <= 0) return;
  const uint32_t tiles = ceil_div(n, kSortTile);
  uint32_t* k2 = tmp;
  uint32_t* v2 = tmp + n;
  uint32_t* hist = tmp + 2 * (size_t)n;
  uint32_t* stmp = hist + 256 * (size_t)tiles;
  uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<tiles, kBlock, 0, st>>>(ka, n, shift, hist, tiles);
    scan_exclusive(hist, 256 * tiles, stmp, st);
    k_rs_scatter<<<tiles, kBlock, 0, st>>>(ka, va, kb, vb, n, shift, hist, tiles);
    uint32_t* t;
    t = ka; ka = kb; kb = t;
    t = va; va = vb; vb = t;
  }
  if (ka != keys) {
    k_copy_u32<<<ceil_div(n, kBlock), kBlock, 0, st>>>(ka, keys, n, 0u);
    k_copy_u32<<<ceil_div(n, kBlock), kBlock, 0, st>>>(va, vals, n, 0u);
  }
}

void count_links(const float2* links, uint32_t E, uint32_t N, uint32_t* valid, uint32_t* len_in, uint32_t* len_out,
                 cudaStream_t st) {
  if (E) k_links_count<<<ceil_div(E, kBlock), kBlock, 0, st>>>(links, E, N, valid, len_in, len_out);
}

void compact_links(const float2* links, uint32_t E, const uint32_t* pos, uint32_t* key_in, uint32_t* key_out,
                   uint32_t* val_in, uint32_t* val_out, cudaStream_t st) {
  if (E) k_links_compact<<<ceil_div(E, kBlock), kBlock, 0, st>>>(links, E, pos, key_in, key_out, val_in, val_out);
}

void fill_csr(const uint32_t* rows, const uint32_t* lidx, uint32_t M, const float2* links, bool incoming,
              const uint32_t* len_in, const uint32_t* len_out, const float* strength, const uint8_t* flags,
              const float* draws, uint64_t seed, uint64_t draw_base, uint32_t point_off, uint4* ent, cudaStream_t st) {
  if (M)
    k_csr_fill<<<ceil_div(M, kBlock), kBlock, 0, st>>>(rows, lidx, M, links, incoming ? 1 : 0, len_in, len_out,
                                                        strength, flags, draws, seed, draw_base, point_off, ent);
}

void len_stats(const uint32_t* len, uint32_t N, uint32_t* stats, cudaStream_t st) {
  if (N) k_len_stats<<<ceil_div(N, kBlock), kBlock, 0, st>>>(len, N, stats);
}

void len_keys(const uint32_t* len, uint32_t N, const uint32_t* stats, uint32_t* key, uint32_t* val, cudaStream_t st) {
  if (N) k_len_keys<<<ceil_div(N, kBlock), kBlock, 0, st>>>(len, N, stats, key, val);
}

void jitter(uint64_t seed, uint64_t base, uint32_t n, float2* out, cudaStream_t st) {
  if (n) k_jitter<<<ceil_div(n, kBlock), kBlock, 0, st>>>(seed, base, n, out);
}

void copy_u32(const uint32_t* a, uint32_t* b, uint32_t n, cudaStream_t st, uint32_t add) {
  if (n) k_copy_u32<<<ceil_div(n, kBlock), kBlock, 0, st>>>(a, b, n, add);
}

}  // namespace dingest
}  // namespace cgl
