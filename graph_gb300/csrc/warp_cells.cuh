// warp_cells.cuh — one warp per dense cell (more than kSmallCell points, at
// most kBigCell): the exact fixed-point sums of its positions and its
// near-field slots, the 8 smallest distinct peel hashes, each with its lowest
// index (build-nearfield-slots.vert:146-162), moved to the head of the cell's
// segment in slot order.  Shared by the plain engine (DeviceView) and the
// batched one (BatchView): both views name the sorted arrays and the per-cell
// results alike.  Hashes and ties use the index minus `koff` (the batched
// engine's per-job point offset; 0 for a single graph).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "device_util.cuh"

namespace cgl {

// The end of a warp cell: move the selected slots to the head [b, b + ns) in
// slot order, in parallel (lane q takes slot q's entry; a head entry that is
// not a slot moves to the place of the r-th slot that lies outside the head,
// r = its rank among them), and write the sums and the slot count.
template <class V>
__device__ __forceinline__ void warp_finish_cell(const V& d, uint32_t c, uint32_t b, int ns,
                                                 const uint32_t (&sel)[kSlots], long long ax, long long ay) {
  const int lane = threadIdx.x & 31;
  uint32_t take_idx = 0, disp_idx = 0, dest = 0;
  float2 take_pos = make_float2(0.f, 0.f), disp_pos = make_float2(0.f, 0.f);
  const uint32_t h = b + (uint32_t)lane;
  bool h_selected = false, sel_outside = false;
#pragma unroll
  for (int k = 0; k < kSlots; ++k) {
    if (k < ns && sel[k] == h) h_selected = true;
    if (k == lane) sel_outside = k < ns && (sel[k] < b || sel[k] >= b + (uint32_t)ns);
  }
  const unsigned out_mask = __ballot_sync(0xffffffffu, sel_outside);
  const bool in_head = lane < ns;
  const bool displaced = in_head && !h_selected;
  const unsigned disp_mask = __ballot_sync(0xffffffffu, displaced);
  if (in_head) {
    uint32_t src = 0;
#pragma unroll
    for (int k = 0; k < kSlots; ++k) if (k == lane) src = sel[k];
    take_idx = d.sorted_idx[src];
    take_pos = d.sorted_pos[src];
  }
  if (displaced) {
    const int r = __popc(disp_mask & ((1u << lane) - 1u));
    unsigned m = out_mask;
    for (int t = 0; t < r; ++t) m &= m - 1u;
    const int k = __ffs(m) - 1;
#pragma unroll
    for (int kk = 0; kk < kSlots; ++kk) if (kk == k) dest = sel[kk];
    disp_idx = d.sorted_idx[h];
    disp_pos = d.sorted_pos[h];
  }
  __syncwarp();
  if (in_head) {
    d.sorted_idx[h] = take_idx;
    d.sorted_pos[h] = take_pos;
    if (d.inv) d.inv[take_idx] = h;
  }
  if (displaced) {
    d.sorted_idx[dest] = disp_idx;
    d.sorted_pos[dest] = disp_pos;
    if (d.inv) d.inv[disp_idx] = dest;
  }
  if (lane == 0) {
    d.big_sx[c] = ax;
    d.big_sy[c] = ay;
    d.big_ns[c] = (uint32_t)ns;
  }
}

// Any warp cell: per-lane sorted top-8 lists (top8_insert), merged in 8 rounds
// of a warp minimum over the keys whose hash is larger than the previous
// slot's.  Every top-8 key of the cell is in the top-8 of the lane that holds
// it, so the merge is exact.
template <class V>
__device__ void warp_cell_lists(const V& d, const FixedScale& fx, uint32_t seed_bits, uint32_t koff, uint32_t c,
                                uint32_t b, uint32_t e) {
  const int lane = threadIdx.x & 31;
  long long ax = 0, ay = 0;
  unsigned long long best[kSlots];
  uint32_t at[kSlots];
#pragma unroll
  for (int q = 0; q < kSlots; ++q) { best[q] = ~0ull; at[q] = 0; }
  uint32_t j = b + lane;
  for (; j + 96 < e; j += 128) {   // loads four points ahead of the selection
    float2 p[4];
    uint32_t ix[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) { p[u] = d.sorted_pos[j + 32 * u]; ix[u] = d.sorted_idx[j + 32 * u]; }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      ax += to_fixed(p[u].x, fx);
      ay += to_fixed(p[u].y, fx);
      top8_insert(best, at, peel_key(ix[u] - koff, seed_bits), j + 32 * u);
    }
  }
  for (; j < e; j += 32) {
    const float2 p = d.sorted_pos[j];
    ax += to_fixed(p.x, fx);
    ay += to_fixed(p.y, fx);
    top8_insert(best, at, peel_key(d.sorted_idx[j] - koff, seed_bits), j);
  }
  ax = warp_sum_ll(ax);
  ay = warp_sum_ll(ay);
  uint32_t sel[kSlots];
  int ns = 0;
  unsigned long long last = 0;
#pragma unroll
  for (int k = 0; k < kSlots; ++k) {
    unsigned long long m = ~0ull;
    uint32_t mp = 0;
#pragma unroll
    for (int q = 0; q < kSlots; ++q)
      if (best[q] != ~0ull && (k == 0 || (best[q] >> 32) > (last >> 32)) && best[q] < m) { m = best[q]; mp = at[q]; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long om = __shfl_xor_sync(0xffffffffu, m, o);
      const uint32_t op = __shfl_xor_sync(0xffffffffu, mp, o);
      if (om < m) { m = om; mp = op; }
    }
    sel[k] = mp;
    if (m != ~0ull) { ns = k + 1; last = m; }
    else last = ~0ull;
  }
  warp_finish_cell(d, c, b, ns, sel, ax, ay);
}

// A cell of at most kWarpSmallCell (128) points: each lane holds at most 4
// keys in registers and the 8 selection rounds are warp minimums over them
// (warp_select_slots).
template <class V>
__device__ void warp_cell_small(const V& d, const FixedScale& fx, uint32_t seed_bits, uint32_t koff, uint32_t c,
                                uint32_t b, uint32_t e) {
  const int lane = threadIdx.x & 31;
  uint32_t hb[4], ix[4], at[4];
  long long ax = 0, ay = 0;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const uint32_t j = b + lane + 32u * u;
    hb[u] = ~0u;
    ix[u] = 0;
    at[u] = j;
    if (j < e) {
      const float2 p = d.sorted_pos[j];
      ax += to_fixed(p.x, fx);
      ay += to_fixed(p.y, fx);
      ix[u] = d.sorted_idx[j] - koff;
      hb[u] = __float_as_uint(peel_hash(ix[u], seed_bits));
    }
  }
  ax = warp_sum_ll(ax);
  ay = warp_sum_ll(ay);
  uint32_t sel[kSlots];
  const int ns = warp_select_slots(hb, ix, at, sel);
  warp_finish_cell(d, c, b, ns, sel, ax, ay);
}

// A cell above kWarpSmallCell points: only points whose hash lies below a
// threshold of about 48 / n stay candidates (about 48 of them), gathered in a
// per-warp buffer and selected as in warp_cell_small.  When at least 8
// distinct hashes lie below the threshold, the 8 smallest of the cell are
// among them, so the slots are exact; otherwise, or when the buffer
// overflows, nothing is written and the function returns false.
constexpr int kCandidates = 128;
template <class V>
__device__ bool warp_cell_filtered(const V& d, const FixedScale& fx, uint32_t seed_bits, uint32_t koff, uint32_t c,
                                   uint32_t b, uint32_t e, uint32_t (&buf)[3][kCandidates]) {
  const int lane = threadIdx.x & 31;
  const uint32_t below = __float_as_uint(__fdiv_rn(48.0f, (float)(e - b)));
  long long ax = 0, ay = 0;
  uint32_t cnt = 0;   // warp-uniform
  __syncwarp();       // the buffer's previous cell is read
  for (uint32_t base = b; base < e; base += 128) {
    float2 p[4];
    uint32_t ix[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t j = base + lane + 32u * u;
      if (j < e) { p[u] = d.sorted_pos[j]; ix[u] = d.sorted_idx[j] - koff; }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t j = base + lane + 32u * u;
      uint32_t h = ~0u;
      if (j < e) {
        ax += to_fixed(p[u].x, fx);
        ay += to_fixed(p[u].y, fx);
        h = __float_as_uint(peel_hash(ix[u], seed_bits));
      }
      const bool cand = h < below;
      const unsigned m = __ballot_sync(0xffffffffu, cand);
      if (cand) {
        const uint32_t slot = cnt + __popc(m & ((1u << lane) - 1u));
        if (slot < (uint32_t)kCandidates) { buf[0][slot] = h; buf[1][slot] = ix[u]; buf[2][slot] = j; }
      }
      cnt += __popc(m);
    }
  }
  if (cnt > (uint32_t)kCandidates) return false;
  __syncwarp();
  uint32_t hb[4], ci[4], cp[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const uint32_t slot = lane + 32u * u;
    const bool in = slot < cnt;
    hb[u] = in ? buf[0][slot] : ~0u;
    ci[u] = in ? buf[1][slot] : 0u;
    cp[u] = in ? buf[2][slot] : 0u;
  }
  uint32_t sel[kSlots];
  const int ns = warp_select_slots(hb, ci, cp, sel);
  if (ns < kSlots) return false;
  ax = warp_sum_ll(ax);
  ay = warp_sum_ll(ay);
  warp_finish_cell(d, c, b, ns, sel, ax, ay);
  return true;
}

// One warp cell of any size up to kBigCell.
template <class V>
__device__ __forceinline__ void warp_cell(const V& d, const FixedScale& fx, uint32_t seed_bits, uint32_t koff,
                                          uint32_t c, uint32_t (&buf)[3][kCandidates]) {
  const uint32_t b = d.cell_start[c], e = d.cell_start[c + 1];
  if (e - b <= kWarpSmallCell) warp_cell_small(d, fx, seed_bits, koff, c, b, e);
  else if (!warp_cell_filtered(d, fx, seed_bits, koff, c, b, e, buf)) warp_cell_lists(d, fx, seed_bits, koff, c, b, e);
}

}  // namespace cgl
