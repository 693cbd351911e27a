// kernels.cu — per-tick force kernels of the GB300 force-layout engine.
//
// One tick (Graph.runSimulationStep, src/index.ts:2006-2099) is:
//   prepass      gravity + update (force-gravity.frag, update-position.frag),
//                optional centroid sums (calculate-centermass.vert), and the
//                finest-cell histogram of the many-body binning
//   center       ForceCenter (force-center.frag) + update + binning   [if on]
//   scan         exclusive scan of the finest-cell histogram
//   scatter      counting-sort scatter of live points into cell order
//   cells        per finest cell: exact sums, the 8-slot near-field peel
//                (build-nearfield-slots.vert), and the pyramid of coarser
//                levels (calculate-level.vert for every level); dense cells
//                get a warp (warp_cells.cuh) or a CTA first (k_bigcells)
//   manybody     level passes + near field + update (force-level.frag,
//                force-nearfield.frag, update-position.frag); one thread per
//                point, or 16 per point for small graphs (k_manybody_split)
//   link in/out  spring force over each direction's link lists + update
//                (force-spring.ts); hub lists get a CTA each, the other
//                lists are read by warps (k_warp_lengths and k_fill_lanes
//                lay them out at render)
//   clusters     centre of mass per cluster + cluster pull + update
//                (calculate-centermass.vert, force-cluster.frag)   [if set]
//   collision    4 offset grids + spatial collision force + update
//                (build-grid.vert, force-collision-spatial.frag)
// Kernels read the tick's alpha and peel seed from device memory so that one
// captured CUDA graph serves every tick.  Outside the tick: the pointer's
// repulsion and drag passes (force-mouse.frag, drag-point.frag) and the
// renderer's position texture.
#include <atomic>

#include "device_util.cuh"
#include "collision.cuh"
#include "kernels.cuh"
#include "manybody_duo.cuh"
#include "warp_cells.cuh"

namespace cgl {

namespace {

__device__ __forceinline__ TickParams tick_params(const DeviceView& d) {
  return d.tick_params[*d.tick_ctr];
}

// Block-reduce three integer sums and add them to dst[0..2] (one atomic each).
__device__ void block_add3(long long a, long long b, long long c, long long* dst) {
  __shared__ long long sm[3][kBlock / 32];
  a = warp_sum_ll(a); b = warp_sum_ll(b); c = warp_sum_ll(c);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sm[0][w] = a; sm[1][w] = b; sm[2][w] = c; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? sm[0][lane] : 0; b = lane < nw ? sm[1][lane] : 0; c = lane < nw ? sm[2][lane] : 0;
    a = warp_sum_ll(a); b = warp_sum_ll(b); c = warp_sum_ll(c);
    if (lane == 0) {
      atomicAdd((unsigned long long*)&dst[0], (unsigned long long)a);
      atomicAdd((unsigned long long*)&dst[1], (unsigned long long)b);
      atomicAdd((unsigned long long*)&dst[2], (unsigned long long)c);
    }
  }
}

__device__ __forceinline__ void bin_point(const DeviceView& d, const SimScalars& s, uint32_t i, float2 p) {
  const int cx = cell_index(p.x, s.csf, s.gf), cy = cell_index(p.y, s.csf, s.gf);
  const uint32_t key = (uint32_t)(cy * s.gf + cx);
  d.key[i] = key;
  d.rank[i] = atomicAdd(&d.counts[key], 1u);
  // a point outside [0, space] (a pinned point, or input positions before
  // their first update) can put a cell's centroid outside its cell
  const bool outside = !(p.x >= 0.f && p.x <= s.space && p.y >= 0.f && p.y <= s.space);
  const unsigned am = __activemask();
  if (__ballot_sync(am, outside) && (threadIdx.x & 31) == (unsigned)(__ffs(am) - 1))
    atomicOr(&d.big_count[kOutsideFlag], 1u);
}

// ---------------------------------------------------------------- prepass --
// force-gravity.frag:24-40 for point p (the velocity, before the update).
__device__ __forceinline__ float2 gravity_velocity(const SimScalars& s, float alpha, float2 p) {
  const float c = __fmul_rn(s.space, 0.5f);
  const float dx = __fsub_rn(c, p.x), dy = __fsub_rn(c, p.y);
  const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  float vx = 0.f, vy = 0.f;
  if (dist > 0.f) {
    const float add = __fmul_rn(__fmul_rn(__fmul_rn(alpha, s.gravity), dist), 0.1f);
    vx = __fadd_rn(vx, __fmul_rn(add, __fdiv_rn(dx, dist)));
    vy = __fadd_rn(vy, __fmul_rn(add, __fdiv_rn(dy, dist)));
  }
  return make_float2(vx, vy);
}

// Binning in the previous tick's cell order (bin_state[0]): points move little
// in a tick, so the lanes of a warp mostly fall in a few cells, and one atomic
// per cell and warp (__match_any_sync) ranks them all.  Keys, ranks, points and
// positions are written by position j; the scatter reads them in that order.
// The order of the points within a cell is free (every use of it is), so the
// ranks need not follow j.  The gravity-updated position is not written back
// to pos: the many-body pass that follows this binning starts from it (through
// the scatter's sorted_pos) and writes every live point that is not pinned,
// and a pinned point does not move.  Without pinned points (s.any_pinned = 0)
// no flag is read either: absent points are not in the cell order.
template <uint32_t MODE>
__device__ __forceinline__ void prepass_in_cell_order(const DeviceView& d, const SimScalars& s, const TickParams& tp) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) d.bin_state[1] = 1;
  if (j >= d.cell_start[s.gf * s.gf]) return;   // the live points, binned last tick
  const uint32_t i = d.sorted_idx[j];
  float2 p = d.pos[i];
  if (MODE & kPreGravity) {
    const float2 v = gravity_velocity(s, tp.alpha, p);
    if (!s.any_pinned || !(d.flags[i] & kPinned)) p = integrate(p, v.x, v.y, s.friction, s.space);
  }
  const int cx = cell_index(p.x, s.csf, s.gf), cy = cell_index(p.y, s.csf, s.gf);
  const uint32_t key = (uint32_t)(cy * s.gf + cx);
  const bool outside = !(p.x >= 0.f && p.x <= s.space && p.y >= 0.f && p.y <= s.space);
  const unsigned am = __activemask();
  const int lane = threadIdx.x & 31;
  if (__ballot_sync(am, outside) && lane == __ffs(am) - 1) atomicOr(&d.big_count[kOutsideFlag], 1u);
  const unsigned peers = __match_any_sync(am, key);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&d.counts[key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  d.key[j] = key;
  d.rank[j] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
  d.idx_s[j] = i;
  d.pos_s[j] = p;
}

template <uint32_t MODE>
__global__ void __launch_bounds__(kBlock) k_prepass(DeviceView d, SimScalars s) {
  const TickParams tp = tick_params(d);
  if ((MODE & kPreBin) && !(MODE & kPreCentroid) && d.bin_state[0]) {
    prepass_in_cell_order<MODE>(d, s, tp);
    return;
  }
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if ((MODE & kPreBin) && i == 0) d.bin_state[1] = 0;
  long long sx = 0, sy = 0, sn = 0;
  if (i < d.n) {
    const uint8_t f = d.flags[i];
    float2 p = d.pos[i];
    if (MODE & kPreGravity) {
      const float2 v = gravity_velocity(s, tp.alpha, p);
      if (!(f & (kPinned | kAbsent))) {
        p = integrate(p, v.x, v.y, s.friction, s.space);
        d.pos[i] = p;
      }
    }
    if (!(f & kAbsent)) {
      if (MODE & kPreCentroid) { sx = to_fixed(p.x, s.fx); sy = to_fixed(p.y, s.fx); sn = 1; }
      if (MODE & kPreBin) bin_point(d, s, i, p);
    } else if (MODE & kPreBin) {
      d.key[i] = kNoCell;
    }
  }
  if (MODE & kPreCentroid) block_add3(sx, sy, sn, d.centroid);
}

// ----------------------------------------------------------------- center --
template <bool BIN>
__global__ void __launch_bounds__(kBlock) k_center(DeviceView d, SimScalars s) {
  // ForceCenter.run (ForceCenter/index.ts:149-199), force-center.frag:22-36
  const TickParams tp = tick_params(d);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const float sx = from_fixed(d.centroid[0], s.fx), sy = from_fixed(d.centroid[1], s.fx);
  const float cnt = (float)d.centroid[2];
  const float cmx = __fdiv_rn(sx, cnt), cmy = __fdiv_rn(sy, cnt);
  const uint8_t f = d.flags[i];
  float2 p = d.pos[i];
  const float dx = __fsub_rn(cmx, p.x), dy = __fsub_rn(cmy, p.y);
  const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  float vx = 0.f, vy = 0.f;
  if (dist > 0.f) {
    const float add = __fmul_rn(__fmul_rn(__fmul_rn(tp.alpha, s.center), dist), 0.01f);
    vx = __fadd_rn(vx, __fmul_rn(add, __fdiv_rn(dx, dist)));
    vy = __fadd_rn(vy, __fmul_rn(add, __fdiv_rn(dy, dist)));
  }
  if (!(f & (kPinned | kAbsent))) {
    p = integrate(p, vx, vy, s.friction, s.space);
    d.pos[i] = p;
  }
  if (BIN) {
    if (i == 0) d.bin_state[1] = 0;
    if (!(f & kAbsent)) bin_point(d, s, i, p);
    else d.key[i] = kNoCell;
  }
}

// ------------------------------------------------------------------- scan --
constexpr int kScanItems = 4;
constexpr int kScanChunk = kBlock * kScanItems;   // cells per scan block

// A cell's scan word: its count, and with PAIRS the number of work items of
// the paired many-body pass, ceil(count / 2), in the high 32 bits (no sum of
// either exceeds 2^32, so one 64-bit add adds both).
template <bool PAIRS>
__device__ __forceinline__ unsigned long long scan_word(uint32_t count) {
  return PAIRS ? ((unsigned long long)((count + 1) >> 1) << 32) | count : count;
}

// Exclusive scan of the cell histogram into cell_start (and, with PAIRS,
// pair_start), the histogram zeroed for the next tick, the dense cells listed.
template <bool PAIRS>
__global__ void __launch_bounds__(kBlock) k_scan(DeviceView d, uint32_t cells) {
  __shared__ unsigned long long s_seq, s_prefix;
  __shared__ uint32_t s_lists[6];   // dense cells of this block per list, then each list's base
  if (threadIdx.x == 0) s_seq = atomicAdd(d.scan_seq, 1ull);
  if (threadIdx.x < 3) s_lists[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t nb = gridDim.x;
  const uint32_t vb = (uint32_t)(s_seq % nb);
  const unsigned long long parity = ((s_seq / nb) & 1ull) << 63;
  // cells is a multiple of 64 (a power-of-two grid of at least 8 x 8) and
  // base of 4: a thread's four cells are all inside or all outside
  const uint32_t base = vb * kScanChunk + threadIdx.x * kScanItems;
  const bool inside = base < cells;
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (inside) v = reinterpret_cast<const uint4*>(d.counts)[base >> 2];
  const unsigned long long w0 = scan_word<PAIRS>(v.x), w1 = scan_word<PAIRS>(v.y), w2 = scan_word<PAIRS>(v.z),
                           w3 = scan_word<PAIRS>(v.w);
  unsigned long long total;
  unsigned long long off = block_exclusive_scan64(w0 + w1 + w2 + w3, &total);
  if (threadIdx.x < 32) {
    unsigned long long prefix = 0;
    if (vb == 0) {
      if (threadIdx.x == 0) st_relaxed_u64(&d.block_sums[0], parity | kScanInclusive | total);
    } else {
      if (threadIdx.x == 0) st_relaxed_u64(&d.block_sums[vb], parity | kScanTotal | total);
      prefix = scan_look_back(d.block_sums, vb, parity, d.error_word, kErrorScan);
      if (threadIdx.x == 0) st_relaxed_u64(&d.block_sums[vb], parity | kScanInclusive | ((prefix + total) & kScanValue));
    }
    if (threadIdx.x == 0) s_prefix = prefix;
  }
  __syncthreads();
  off += s_prefix;
  if (inside) {
    const unsigned long long o1 = off + w0, o2 = o1 + w1, o3 = o2 + w2;
    reinterpret_cast<uint4*>(d.cell_start)[base >> 2] = make_uint4((uint32_t)off, (uint32_t)o1, (uint32_t)o2, (uint32_t)o3);
    if (PAIRS)
      reinterpret_cast<uint4*>(d.pair_start)[base >> 2] =
          make_uint4((uint32_t)(off >> 32), (uint32_t)(o1 >> 32), (uint32_t)(o2 >> 32), (uint32_t)(o3 >> 32));
    reinterpret_cast<uint4*>(d.counts)[base >> 2] = make_uint4(0u, 0u, 0u, 0u);   // ready for the next tick
  }
  // the dense cells' list entries: a slot in the block's share of each list
  // (shared-memory atomics), then one global atomic per list and block
  const uint32_t cnt[4] = {v.x, v.y, v.z, v.w};
  int cls[4];
  uint32_t slot[4];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    cls[k] = cnt[k] > kBigCell ? 0 : cnt[k] > kWarpSmallCell ? 1 : cnt[k] > kSmallCell ? 2 : 3;
    slot[k] = cls[k] < 3 ? atomicAdd(&s_lists[cls[k]], 1u) : 0u;
  }
  __syncthreads();
  if (threadIdx.x < 3 && s_lists[threadIdx.x]) s_lists[3 + threadIdx.x] = atomicAdd(&d.big_count[threadIdx.x], s_lists[threadIdx.x]);
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const uint32_t c = base + k;
    if (cls[k] == 0) d.big_list[s_lists[3] + slot[k]] = c;
    else if (cls[k] == 1) d.big_list[cells + s_lists[4] + slot[k]] = c;
    else if (cls[k] == 2) d.big_list[2 * cells - 1 - (s_lists[5] + slot[k])] = c;
  }
  if (vb == nb - 1 && threadIdx.x == 0) {
    const unsigned long long g = s_prefix + total;
    d.cell_start[cells] = (uint32_t)g;
    if (PAIRS) d.pair_start[cells] = (uint32_t)(g >> 32);
  }
}

// ---------------------------------------------------------------- scatter --
// With PAIRS, the point at an even position of its cell's segment also writes
// the paired pass's work item: positions (dst, dst + 1), or dst alone when it
// is the segment's last point.  Positions, not points: the cell kernel later
// moves the slots to the segment's head, and a pair stays within its cell.
// Keys and ranks by point (index order) or by last tick's position
// (bin_state[1]); either way every live point lands at cell_start + rank, and
// sorted_idx then holds a cell order of the live points (bin_state[0]).
template <bool PAIRS>
__global__ void __launch_bounds__(kBlock) k_scatter(DeviceView d, uint32_t cells) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) d.bin_state[0] = 1;
  uint32_t i, k;
  float2 p;
  if (d.bin_state[1]) {
    if (t >= d.cell_start[cells]) return;
    i = d.idx_s[t];
    k = d.key[t];
    p = d.pos_s[t];
  } else {
    if (t >= d.n) return;
    i = t;
    k = d.key[t];
    if (k == kNoCell) return;
    p = d.pos[t];
  }
  const uint32_t r = d.rank[t];
  const uint32_t b = d.cell_start[k];
  const uint32_t dst = b + r;
  d.sorted_idx[dst] = i;
  d.sorted_pos[dst] = p;
  if (d.inv) d.inv[i] = dst;
  if (PAIRS && !(r & 1u)) {
    const uint32_t m = d.cell_start[k + 1] - b;
    d.pair_list[d.pair_start[k] + (r >> 1)] = dst | (r + 1 == m ? kSingleBit : 0u);
  }
}

// ------------------------------------------------------------------ cells --
// Move the ns selected entries to the head of the segment starting at b, in
// slot (hash) order; the rest of the segment keeps its points in any order.
__device__ __forceinline__ void move_slots_to_head(const DeviceView& d, uint32_t b, int ns, uint32_t (&at)[kSlots]) {
#pragma unroll
  for (int q = 0; q < kSlots; ++q) {
    if (q < ns) {
      const uint32_t tq = b + q, pq = at[q];
      if (pq != tq) {
        const uint32_t i0 = d.sorted_idx[tq], i1 = d.sorted_idx[pq];
        const float2 p0 = d.sorted_pos[tq], p1 = d.sorted_pos[pq];
        d.sorted_idx[tq] = i1; d.sorted_pos[tq] = p1;
        d.sorted_idx[pq] = i0; d.sorted_pos[pq] = p0;
        if (d.inv) { d.inv[i1] = tq; d.inv[i0] = pq; }
#pragma unroll
        for (int r = q + 1; r < kSlots; ++r)
          if (at[r] == tq) at[r] = pq;
      }
    }
  }
}

// Cells holding more than kSmallCell points (lists built by the scan): above
// kBigCell one CTA per cell, otherwise one warp per cell (warp_cells.cuh), so a
// dense hub cell does not serialise on one thread.  The CTA cells: exact sums
// by block reduction; slots by per-thread top-8 lists merged in 8 rounds of a
// block minimum over keys whose hash is larger than the previous slot's.
__global__ void __launch_bounds__(kBlock) k_bigcells(DeviceView d, SimScalars s) {
  __shared__ unsigned long long skey[kBlock * kSlots];
  __shared__ uint32_t spos[kBlock * kSlots];
  __shared__ unsigned long long wmin[kBlock / 32];
  __shared__ uint32_t wpos[kBlock / 32];
  __shared__ unsigned long long sel_key;
  __shared__ uint32_t sel_at[kSlots];
  __shared__ int sel_n;
  const TickParams tp = tick_params(d);
  const uint32_t nbig = d.big_count[0];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint32_t wi = blockIdx.x; wi < nbig; wi += gridDim.x) {
    const uint32_t c = d.big_list[wi];
    const uint32_t b = d.cell_start[c], e = d.cell_start[c + 1];
    long long ax = 0, ay = 0;
    unsigned long long best[kSlots];
    uint32_t at[kSlots];
#pragma unroll
    for (int q = 0; q < kSlots; ++q) { best[q] = ~0ull; at[q] = 0; }
    for (uint32_t j = b + threadIdx.x; j < e; j += blockDim.x) {
      const float2 p = d.sorted_pos[j];
      ax += to_fixed(p.x, s.fx);
      ay += to_fixed(p.y, s.fx);
      top8_insert(best, at, peel_key(d.sorted_idx[j], tp.seed_bits), j);
    }
#pragma unroll
    for (int q = 0; q < kSlots; ++q) { skey[threadIdx.x * kSlots + q] = best[q]; spos[threadIdx.x * kSlots + q] = at[q]; }
    // exact sums: warp then block reduction (integers, order-free)
    ax = warp_sum_ll(ax); ay = warp_sum_ll(ay);
    __shared__ long long rx[kBlock / 32], ry[kBlock / 32];
    if (lane == 0) { rx[w] = ax; ry[w] = ay; }
    if (threadIdx.x == 0) sel_n = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long tx = 0, ty = 0;
      for (int k = 0; k < kBlock / 32; ++k) { tx += rx[k]; ty += ry[k]; }
      d.big_sx[c] = tx;
      d.big_sy[c] = ty;
    }
    unsigned long long last = 0;
    for (int k = 0; k < kSlots; ++k) {
      unsigned long long m = ~0ull;
      uint32_t mp = 0;
#pragma unroll
      for (int q = 0; q < kSlots; ++q) {
        const unsigned long long key = skey[threadIdx.x * kSlots + q];
        if (key != ~0ull && (k == 0 || (key >> 32) > (last >> 32)) && key < m) { m = key; mp = spos[threadIdx.x * kSlots + q]; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long om = __shfl_xor_sync(0xffffffffu, m, o);
        const uint32_t op = __shfl_xor_sync(0xffffffffu, mp, o);
        if (om < m) { m = om; mp = op; }
      }
      if (lane == 0) { wmin[w] = m; wpos[w] = mp; }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long bm = ~0ull;
        uint32_t bp = 0;
        for (int k2 = 0; k2 < kBlock / 32; ++k2)
          if (wmin[k2] < bm) { bm = wmin[k2]; bp = wpos[k2]; }
        sel_key = bm;
        if (bm != ~0ull) { sel_at[sel_n] = bp; sel_n = sel_n + 1; }
      }
      __syncthreads();
      last = sel_key;
      if (last == ~0ull) break;
    }
    if (threadIdx.x == 0) {
      const int ns = sel_n;
      uint32_t pat[kSlots];
#pragma unroll
      for (int q = 0; q < kSlots; ++q) pat[q] = q < ns ? sel_at[q] : 0;
      move_slots_to_head(d, b, ns, pat);
      d.big_ns[c] = (uint32_t)ns;
    }
    __syncthreads();
  }
  // warp cells, one warp each, the heavy ones (above kWarpSmallCell points)
  // first, so the longest start first
  __shared__ uint32_t cand[kBlock / 32][3][kCandidates];
  const uint32_t nheavy = d.big_count[1], nwarp = nheavy + d.big_count[2];
  const uint32_t cells = (uint32_t)(s.gf * s.gf);
  // the first cell by warp id, the next ones from the ticket
  const uint32_t nw_grid = gridDim.x * (blockDim.x >> 5);
  for (uint32_t wi = blockIdx.x * (blockDim.x >> 5) + w; wi < nwarp;) {
    const uint32_t c = wi < nheavy ? d.big_list[cells + wi] : d.big_list[2 * cells - 1 - (wi - nheavy)];
    warp_cell(d, s.fx, tp.seed_bits, 0u, c, cand[w]);
    if (lane == 0) wi = nw_grid + atomicAdd(&d.big_count[3], 1u);
    wi = __shfl_sync(0xffffffffu, wi, 0);
  }
}

// One thread per finest cell, one CTA per tile x tile block of cells.
__global__ void k_cells(DeviceView d, SimScalars s) {
  extern __shared__ long long sm[];   // 3 * tile * tile
  const TickParams tp = tick_params(d);
  const int T = s.tile;
  const int tiles_row = s.gf / T;
  const int tile_x = blockIdx.x % tiles_row, tile_y = blockIdx.x / tiles_row;
  const int tx = threadIdx.x % T, ty = threadIdx.x / T;
  const int cx = tile_x * T + tx, cy = tile_y * T + ty;
  const uint32_t c = (uint32_t)(cy * s.gf + cx);
  const uint32_t b = d.cell_start[c], e = d.cell_start[c + 1];

  // exact sums and the 8 smallest distinct peel hashes (build-nearfield-slots.vert)
  long long ax = 0, ay = 0;
  int ns = 0;
  if (e - b > kSmallCell) {   // done cooperatively by k_bigcells
    ax = d.big_sx[c];
    ay = d.big_sy[c];
    ns = (int)d.big_ns[c];
  } else {
    unsigned long long best[kSlots];
    uint32_t at[kSlots];
#pragma unroll
    for (int q = 0; q < kSlots; ++q) { best[q] = ~0ull; at[q] = 0; }
    for (uint32_t j = b; j < e; ++j) {
      const float2 p = d.sorted_pos[j];
      ax += to_fixed(p.x, s.fx);
      ay += to_fixed(p.y, s.fx);
      top8_insert(best, at, peel_key(d.sorted_idx[j], tp.seed_bits), j);
    }
#pragma unroll
    for (int q = 0; q < kSlots; ++q) ns += best[q] != ~0ull;
    move_slots_to_head(d, b, ns, at);
  }
  const uint32_t cnt = e - b;
  {
    float4 r = make_float4(0.f, 0.f, 0.f, (float)ns);
    if (cnt > 0) {
      const float cf = (float)cnt;
      r.x = __fdiv_rn(from_fixed(ax, s.fx), cf);
      r.y = __fdiv_rn(from_fixed(ay, s.fx), cf);
      r.z = cf;
    }
    d.rec[d.level_off[s.levels - 1] + c] = r;
  }

  // coarser levels inside the tile
  long long* smx = sm;
  long long* smy = sm + T * T;
  long long* smn = sm + 2 * T * T;
  smx[threadIdx.x] = ax; smy[threadIdx.x] = ay; smn[threadIdx.x] = cnt;
  __syncthreads();
  int g = T;
  int lv = s.levels - 1;
  while (g > 1 && lv > 0) {
    g >>= 1;
    --lv;
    long long vx = 0, vy = 0, vn = 0;
    const bool active = tx < g && ty < g;
    if (active) {
      const int i00 = (2 * ty) * T + 2 * tx;
      vx = smx[i00] + smx[i00 + 1] + smx[i00 + T] + smx[i00 + T + 1];
      vy = smy[i00] + smy[i00 + 1] + smy[i00 + T] + smy[i00 + T + 1];
      vn = smn[i00] + smn[i00 + 1] + smn[i00 + T] + smn[i00 + T + 1];
    }
    __syncthreads();
    if (active) {
      smx[ty * T + tx] = vx; smy[ty * T + tx] = vy; smn[ty * T + tx] = vn;
      const int G = 4 << lv;
      const int gx = tile_x * g + tx, gy = tile_y * g + ty;
      float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
      if (vn > 0) {
        const float cf = (float)vn;
        r.x = __fdiv_rn(from_fixed(vx, s.fx), cf);
        r.y = __fdiv_rn(from_fixed(vy, s.fx), cf);
        r.z = cf;
      }
      d.rec[d.level_off[lv] + gy * G + gx] = r;
    }
    __syncthreads();
  }
  if (lv == 0) return;   // the tile reached the coarsest level: no tile is partial
  // levels coarser than the tile: integer atomics, finished by the last CTA
  if (threadIdx.x == 0) {
    const long long tx_ = smx[0], ty_ = smy[0], tn_ = smn[0];
    for (int l = lv - 1; l >= 0; --l) {
      const int sh = lv - l;
      const int G = 4 << l;
      const int gx = tile_x >> sh, gy = tile_y >> sh;
      long long* a = d.acc + 3 * (size_t)(d.acc_off[l] + gy * G + gx);
      atomicAdd((unsigned long long*)&a[0], (unsigned long long)tx_);
      atomicAdd((unsigned long long*)&a[1], (unsigned long long)ty_);
      atomicAdd((unsigned long long*)&a[2], (unsigned long long)tn_);
    }
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(d.cells_ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const uint32_t total_cells = d.acc_off[lv];
  for (uint32_t k = threadIdx.x; k < total_cells; k += blockDim.x) {
    int l = 0;
    while (l + 1 < lv && d.acc_off[l + 1] <= k) ++l;
    const uint32_t cl = k - d.acc_off[l];
    long long* a = d.acc + 3 * (size_t)k;
    const long long vx = __ldcg(&a[0]), vy = __ldcg(&a[1]), vn = __ldcg(&a[2]);
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (vn > 0) {
      const float cf = (float)vn;
      r.x = __fdiv_rn(from_fixed(vx, s.fx), cf);
      r.y = __fdiv_rn(from_fixed(vy, s.fx), cf);
      r.z = cf;
    }
    d.rec[d.level_off[l] + cl] = r;
    a[0] = 0; a[1] = 0; a[2] = 0;
  }
  if (threadIdx.x == 0) *d.cells_ticket = 0;
}

// --------------------------------------------------------------- manybody --
// FAST: the repulsion quotients come from the reciprocals (quotient_by_recip(k),
// the same for every point of a pass, so each launch runs one of the two).

// Level l's sum for the point in finest cell (fcx, fcy).
template <bool FAST, bool UNCHECKED = FAST, bool GUARDED = false>
__device__ __forceinline__ float2 level_sum(const DeviceView& d, int L, int l, int fcx, int fcy, float2 p, float k,
                                            PairUnits pu) {
  const int sh = L - 1 - l;
  return level_terms<FAST, UNCHECKED, GUARDED>(d.rec + d.level_off[l], 4 << l, fcx >> sh, fcy >> sh, p, k, pu);
}

// The level guard of a pass (SimScalars::level_guard) holds this tick: no
// binned point lies outside the space.
__device__ __forceinline__ bool level_guard_holds(const DeviceView& d, const SimScalars& s) {
  return s.level_guard && __ldg(&d.big_count[kOutsideFlag]) == 0;
}

// force-nearfield.frag:151-157 (jitter, step clamp) and the update.  The
// point is left alone when the early pass (early) writes it this tick.
__device__ __forceinline__ void finish_point(const DeviceView& d, const SimScalars& s, uint32_t i, float2 p, float2 rj,
                                             float2 vel, float2 nf, PairUnits pu, bool early = false) {
  nf = add2(nf, mul2(nf, rj, pu), pu);
  const float max_step = __fmul_rn(2.0f, s.csf);
  const float2 nsq = mul2(nf, nf, pu);
  const float speed = __fsqrt_rn(__fadd_rn(nsq.x, nsq.y));
  if (speed > max_step) nf = mul2(nf, splat(__fdiv_rn(max_step, speed)), pu);
  vel = add2(vel, nf, pu);
  const uint8_t f = d.flags[i];
  if (!(f & kPinned) && (early || !(s.skip_early && (f & kEarly))))
    d.pos[i] = integrate(p, vel.x, vel.y, s.friction, s.space);
}

// One point, all of its terms in order on one thread (GUARDED: the level
// terms without the range flag, level_guard_holds).
template <bool FAST, bool GUARDED = false>
__device__ __forceinline__ void manybody_point(const DeviceView& d, const SimScalars& s, uint32_t j, float k,
                                               bool early = false) {
  const uint32_t i = d.sorted_idx[j];
  const float2 p = d.sorted_pos[j];
  const int gf = s.gf, L = s.levels;
  const int fcx = cell_index(p.x, s.csf, gf), fcy = cell_index(p.y, s.csf, gf);
  const PairUnits pu = s.units;
  float2 vel = make_float2(0.f, 0.f);
#pragma unroll 1
  for (int l = 0; l < L; ++l) vel = add2(vel, level_sum<FAST, FAST, GUARDED>(d, L, l, fcx, fcy, p, k, pu), pu);
  const float2 rj = d.jitter[i];
  const float2 nf = near_terms<FAST>(d.rec + d.level_off[L - 1], d.cell_start, d.sorted_pos, gf, fcx, fcy, j, p, rj, k, pu);
  finish_point(d, s, i, p, rj, vel, nf, pu, early);
}

// Small graphs: each point's level sums and near-field cells are independent
// partial sums that the point then adds in the fixed order, so 16 threads can
// share a point: warps 0-3 compute the level sums (8 per point), warps 4-7
// the near-field cells (8 per point; the first also takes cell 8), and one
// thread per point adds them in order.  The operations are those of
// manybody_point, in the same order; only the threads differ.  For graphs that
// do not fill the GPU with one thread per point.
constexpr int kSplitPoints = kBlock / 16;

template <bool FAST, bool GUARDED>
__device__ __forceinline__ void manybody_split(const DeviceView& d, const SimScalars& s, float k,
                                               float2 (&lvs)[kSplitPoints][8], float2 (&nfs)[kSplitPoints][9],
                                               bool (&nfa)[kSplitPoints][9]) {
  const uint32_t total = d.cell_start[s.gf * s.gf];
  const int t = threadIdx.x;
  const bool level_role = t < kBlock / 2;
  const int r = level_role ? t : t - kBlock / 2;
  const int pt = r >> 3, part = r & 7;
  const uint32_t j = blockIdx.x * kSplitPoints + pt;
  const int gf = s.gf, L = s.levels;
  const PairUnits pu = s.units;
  if (j < total) {
    const uint32_t i = d.sorted_idx[j];
    const float2 p = d.sorted_pos[j];
    const int fcx = cell_index(p.x, s.csf, gf), fcy = cell_index(p.y, s.csf, gf);
    if (level_role) {
      if (part < L) lvs[pt][part] = level_sum<FAST, GUARDED, GUARDED>(d, L, part, fcx, fcy, p, k, pu);
    } else {
      const float2 rj = d.jitter[i];
      const float4* fine = d.rec + d.level_off[L - 1];
#pragma unroll 1
      for (int c = part; c < 9; c += 8)
        nfa[pt][c] = near_cell_terms<FAST>(fine, d.cell_start, d.sorted_pos, gf, fcx, fcy, c % 3 - 1, c / 3 - 1, j, p,
                                           rj, k, pu, nfs[pt][c]);
    }
  }
  __syncthreads();
  if (t < kSplitPoints) {
    const uint32_t jt = blockIdx.x * kSplitPoints + t;
    if (jt < total) {
      const uint32_t i = d.sorted_idx[jt];
      const float2 p = d.sorted_pos[jt];
      float2 vel = make_float2(0.f, 0.f);
      for (int l = 0; l < L; ++l) vel = add2(vel, lvs[t][l], pu);
      float2 nf = make_float2(0.f, 0.f);
      for (int c = 0; c < 9; ++c)
        if (nfa[t][c]) nf = add2(nf, nfs[t][c], pu);
      finish_point(d, s, i, p, d.jitter[i], vel, nf, pu);
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_manybody_split(DeviceView d, SimScalars s) {
  __shared__ float2 lvs[kSplitPoints][8];
  __shared__ float2 nfs[kSplitPoints][9];
  __shared__ bool nfa[kSplitPoints][9];
  const TickParams tp = tick_params(d);
  const float k = __fmul_rn(tp.alpha, s.repulsion);
  if (!quotient_by_recip(k)) manybody_split<false, false>(d, s, k, lvs, nfs, nfa);
  else if (level_guard_holds(d, s)) manybody_split<true, true>(d, s, k, lvs, nfs, nfa);
  else manybody_split<true, false>(d, s, k, lvs, nfs, nfa);
}

// Two points of one finest cell per thread (manybody_duo.cuh): every result
// is the one manybody_point gives that point.  GUARD (the host's
// level_guard): when no binned point lies outside the space this tick, no
// level term's length can leave [1, 2^52], and the level terms run without
// the range flag.
template <bool GUARD>
__device__ __forceinline__ void manybody_duo(const DeviceView& d, const SimScalars& s, uint32_t jA, uint32_t jB,
                                             bool single, float k) {
  const uint32_t iA = d.sorted_idx[jA], iB = d.sorted_idx[jB];
  const float2 pA = d.sorted_pos[jA], pB = d.sorted_pos[jB];
  const int gf = s.gf, L = s.levels;
  const int fcx = cell_index(pA.x, s.csf, gf), fcy = cell_index(pA.y, s.csf, gf);
  const PairUnits pu = s.units;
  const Duo P = {make_float2(pA.x, pB.x), make_float2(pA.y, pB.y)};
  Duo vel = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll 1
  for (int l = 0; l < L; ++l) {
    const int sh = L - 1 - l;
    const float4* lv = d.rec + d.level_off[l];
    bool out = false;
    Duo v = level_terms_duo<!GUARD>(lv, 4 << l, fcx >> sh, fcy >> sh, P, k, pu, out);
    if (!GUARD && out) {   // a length outside the sequences: each point's level with the tested terms
      const float2 a = level_terms<true, false>(lv, 4 << l, fcx >> sh, fcy >> sh, pA, k, pu);
      const float2 b = level_terms<true, false>(lv, 4 << l, fcx >> sh, fcy >> sh, pB, k, pu);
      v.x = make_float2(a.x, b.x);
      v.y = make_float2(a.y, b.y);
    }
    vel.x = add2(vel.x, v.x, pu);
    vel.y = add2(vel.y, v.y, pu);
  }
  const float2 rA = d.jitter[iA], rB = d.jitter[iB];
  const Duo R = {make_float2(rA.x, rB.x), make_float2(rA.y, rB.y)};
  Duo nf = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  const float4* fine = d.rec + d.level_off[L - 1];
  // the 3x3 near field in row order; the own cell is the middle one
#pragma unroll 1
  for (int c = 0; c < 4; ++c)
    near_cell_duo<false>(fine, d.cell_start, d.sorted_pos, gf, fcx, fcy, c % 3 - 1, c / 3 - 1, jA, jB, P, R, k, pu, nf);
  near_cell_duo<true>(fine, d.cell_start, d.sorted_pos, gf, fcx, fcy, 0, 0, jA, jB, P, R, k, pu, nf);
#pragma unroll 1
  for (int c = 5; c < 9; ++c)
    near_cell_duo<false>(fine, d.cell_start, d.sorted_pos, gf, fcx, fcy, c % 3 - 1, c / 3 - 1, jA, jB, P, R, k, pu, nf);
  finish_point(d, s, iA, pA, rA, make_float2(vel.x.x, vel.y.x), make_float2(nf.x.x, nf.y.x), pu);
  if (!single) finish_point(d, s, iB, pB, rB, make_float2(vel.x.y, vel.y.y), make_float2(nf.x.y, nf.y.y), pu);
}

// Four blocks per SM (62 registers): five spill and run 13% slower, three
// leave warps short and run 6% slower (1M-point SBM, GB300).
template <bool GUARD>
__global__ void __launch_bounds__(kBlock, 4) k_manybody_duo(DeviceView d, SimScalars s) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= d.pair_start[s.gf * s.gf]) return;
  const TickParams tp = tick_params(d);
  const float k = __fmul_rn(tp.alpha, s.repulsion);
  const uint32_t e = d.pair_list[w];
  const uint32_t jA = e & ~kSingleBit;
  const bool single = (e & kSingleBit) != 0;
  const uint32_t jB = single ? jA : jA + 1;
  if (!quotient_by_recip(k)) {   // quotients outside the reciprocal method's range: one point at a time
    manybody_point<false>(d, s, jA, k);
    if (!single) manybody_point<false>(d, s, jB, k);
  } else if (GUARD && __ldg(&d.big_count[kOutsideFlag]) == 0) {
    manybody_duo<true>(d, s, jA, jB, single, k);
  } else {
    manybody_duo<false>(d, s, jA, jB, single, k);
  }
}

__global__ void __launch_bounds__(kBlock, 6) k_manybody(DeviceView d, SimScalars s) {
  const TickParams tp = tick_params(d);
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = d.cell_start[s.gf * s.gf];
  if (j >= total) return;
  const float k = __fmul_rn(tp.alpha, s.repulsion);
  if (!quotient_by_recip(k)) manybody_point<false>(d, s, j, k);
  else if (level_guard_holds(d, s)) manybody_point<true, true>(d, s, j, k);
  else manybody_point<true>(d, s, j, k);
}

// The early points (the early hubs and their incoming link targets), a thread
// each, at their sorted positions: the terms of manybody_point, so each result
// is the one the whole pass gives that point.  The whole pass then skips them
// (SimScalars::skip_early), and the early hubs' chains start on them while it
// runs.
__global__ void __launch_bounds__(kBlock) k_manybody_early(DeviceView d, SimScalars s) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_early_pts) return;
  const TickParams tp = tick_params(d);
  const float k = __fmul_rn(tp.alpha, s.repulsion);
  const uint32_t j = d.inv[d.early_pts[t]];
  if (!quotient_by_recip(k)) manybody_point<false>(d, s, j, k, true);
  else if (level_guard_holds(d, s)) manybody_point<true, true>(d, s, j, k, true);
  else manybody_point<true>(d, s, j, k, true);
}

// ------------------------------------------------------------------- link --
// Hub rows: a list of thousands of links is one strictly sequential chain
// (each spring reads the velocity the previous one left).  One CTA per hub, in
// rounds of kHubChunk links: in round c lane 0 of warp 0 runs the chain over
// chunk c from shared memory, recording the velocity before each link, while
// warps 1..7 stage chunk c + 1 (entry, neighbour position, rest length) and
// check chunk c - 1 link by link (spring_chain_check), so neither the loads
// nor the checks sit on the chain.  Three buffers rotate.  A chunk whose check
// fails runs again with the correctly rounded springs from its recorded
// starting velocity, and so does the chunk that followed it.
constexpr int kHubChunk = kBlock - 32;
constexpr int kHubBufs = 3;
constexpr uint32_t kHubInlineChunks = 8;   // lists of up to 8 chunks (1,792 links) check on the chain thread
struct HubStage {
  float4 a[kHubBufs][kHubChunk];   // neighbour x, y, rest length d, 0.99 d
  float4 b[kHubBufs][kHubChunk];   // strength, bias, absent flag, rcp.approx(0.99 d)
  float2 v[kHubBufs][kHubChunk];   // velocity before each link, when the chunk ran on the fast chain
  int fast[kHubBufs];              // the chunk ran on the fast chain (its check is due)
};

// Stages link at + (thread - 32); returns kStagedAbsent when its target is
// absent and kStagedStrength when its strength is not 1.
constexpr int kStagedAbsent = 1, kStagedStrength = 2;
__device__ __forceinline__ int hub_fill(HubStage& st, int buf, uint32_t at, uint32_t e1, const uint4* __restrict__ ent,
                                        const float2* __restrict__ src, float span, float r0, float dist) {
  const int k = threadIdx.x - 32;
  if (at + k >= e1) return 0;
  const uint4 en = __ldg(&ent[at + k]);
  const bool absent = en.x == kAbsentTarget;
  const float2 q = absent ? make_float2(0.f, 0.f) : __ldg(&src[en.x]);
  const float dd = __fmul_rn(__fadd_rn(__fmul_rn(__uint_as_float(en.y), span), r0), dist);
  st.a[buf][k] = make_float4(q.x, q.y, dd, __fmul_rn(dd, 0.99f));
  st.b[buf][k] = make_float4(__uint_as_float(en.w), __uint_as_float(en.z), absent ? 1.f : 0.f,
                             rcp_estimate(__fmul_rn(dd, 0.99f)));
  return (absent ? kStagedAbsent : 0) | (__uint_as_float(en.w) != 1.0f ? kStagedStrength : 0);
}

// The fast chain over one staged chunk without absent targets, recording the
// velocity before each link (a full chunk with a constant trip count).
template <bool UNIT_STRENGTH>
__device__ __forceinline__ void hub_chunk_chain(const float4* A, const float4* B, float2* V, uint32_t len, float2 pp,
                                                float2& vel, float sa, PairUnits pu) {
  if (len == (uint32_t)kHubChunk) {
#pragma unroll 4
    for (int k = 0; k < kHubChunk; ++k) {
      const float4 a = A[k];
      const float4 b = B[k];
      V[k] = vel;
      spring_chain_step<UNIT_STRENGTH>(pp, vel, make_float2(a.x, a.y), a.z, a.w, b.w, sa, b.x, b.y, pu);
    }
  } else {
#pragma unroll 4
    for (uint32_t k = 0; k < len; ++k) {
      const float4 a = A[k];
      const float4 b = B[k];
      V[k] = vel;
      spring_chain_step<UNIT_STRENGTH>(pp, vel, make_float2(a.x, a.y), a.z, a.w, b.w, sa, b.x, b.y, pu);
    }
  }
}

// The fast chain over one staged chunk without absent targets, its checks on
// the chain thread: at the first link whose check fails the chain goes back
// to that link's starting velocity (recorded in V), takes it with the
// correctly rounded spring and goes on from the next link, so only the links
// after it run twice (the whole chunk ran again exactly before).  Every link
// before a failing one passed its check, so the result is the correctly
// rounded chain's; each round ends at least one link further on.
template <bool UNIT_STRENGTH>
__device__ __forceinline__ void hub_chunk_resumed(const float4* A, const float4* B, float2* V, uint32_t len,
                                                  float2 pp, float2& vel, float sa, PairUnits pu) {
  uint32_t k0 = 0;
  while (k0 < len) {
    uint32_t bad = len;   // the first link whose check fails
#pragma unroll 4
    for (uint32_t k = k0; k < len; ++k) {
      const float4 a = A[k];
      const float4 b = B[k];
      V[k] = vel;
      bool out = false;
      spring_chain_step_checked<UNIT_STRENGTH>(pp, vel, make_float2(a.x, a.y), a.z, a.w, b.w, sa, b.x, b.y, pu, out);
      bad = (out && bad == len) ? k : bad;
    }
    if (bad == len) return;
    vel = V[bad];
    const float4 a = A[bad];
    const float4 b = B[bad];
    spring_step(pp, vel, make_float2(a.x, a.y), a.z, a.w, sa, b.x, b.y, pu);
    k0 = bad + 1;
  }
}

// The correctly rounded springs over one staged chunk (absent targets skipped).
__device__ __forceinline__ void hub_chunk_exact(const float4* A, const float4* B, uint32_t len, float2 pp, float2& vel,
                                                float sa, PairUnits pu) {
  for (uint32_t k = 0; k < len; ++k) {
    const float4 a = A[k];
    const float4 b = B[k];
    if (b.z != 0.f) continue;
    spring_step(pp, vel, make_float2(a.x, a.y), a.z, a.w, sa, b.x, b.y, pu);
  }
}

// Blocks [0, nhub) take the hub rows rows[0..nhub) (longest first, so the
// longest chain starts first); the other blocks take one row per thread from
// rows[nhub..nrows): the rest of the points by list length, so the lanes of a
// warp walk lists of (nearly) the same length.
__global__ void __launch_bounds__(kBlock) k_link(DeviceView d, SimScalars s, const uint32_t* __restrict__ rowptr,
                                                 const uint4* __restrict__ ent, const uint32_t* __restrict__ woff,
                                                 const uint4* __restrict__ lane_ent, const float2* __restrict__ src,
                                                 float2* __restrict__ dst, const uint32_t* __restrict__ rows,
                                                 uint32_t nrows, uint32_t nhub, uint32_t block0) {
  // ForceLink.run (ForceLink/index.ts:221-263), force-spring.ts:38-96
  // block0: the first block's place in the whole pass (a launch of the light
  // rows alone starts at nhub)
  const uint32_t bx = blockIdx.x + block0;
  extern __shared__ float4 hub_smem[];   // a HubStage when nhub > 0, else nothing
  HubStage& hub = *reinterpret_cast<HubStage*>(hub_smem);
  const TickParams tp = tick_params(d);
  const float sa = __fmul_rn(s.link_spring, tp.alpha);
  const PairUnits pu = s.units;
  const float span = __fsub_rn(s.link_r1, s.link_r0);
  if (bx < nhub) {
    const uint32_t p = rows[bx];
    const float2 pp = src[p];
    const uint8_t f = d.flags[p];
    if (f & kAbsent) {
      if (threadIdx.x == 0) dst[p] = pp;
      return;
    }
    const uint32_t e0 = rowptr[p], e1 = rowptr[p + 1];
    const uint32_t chunks = (e1 - e0 + kHubChunk - 1) / kHubChunk;
    auto chunk_len = [&](uint32_t c) { return min((uint32_t)kHubChunk, e1 - e0 - c * kHubChunk); };
    int staged = 0;
    if (threadIdx.x >= 32) staged = hub_fill(hub, 0, e0, e1, ent, src, span, s.link_r0, s.link_distance);
    int absent = __syncthreads_or(staged & kStagedAbsent);       // some target of chunk c is absent
    int strengths = __syncthreads_or(staged & kStagedStrength);  // some strength of chunk c is not 1
    float2 vel = make_float2(0.f, 0.f);
    if (chunks <= kHubInlineChunks) {
      // a short list: two buffers, the checks on the chain thread (a round of
      // checks after the chain would cost more than it saves)
      for (uint32_t c = 0; c < chunks; ++c) {
        const int buf = c & 1;
        int next = 0;
        if (threadIdx.x >= 32) {
          if (c + 1 < chunks)
            next = hub_fill(hub, buf ^ 1, e0 + (c + 1) * kHubChunk, e1, ent, src, span, s.link_r0, s.link_distance);
        } else if (threadIdx.x == 0) {
          const uint32_t len = chunk_len(c);
          if (absent) hub_chunk_exact(hub.a[buf], hub.b[buf], len, pp, vel, sa, pu);
          else if (strengths) hub_chunk_resumed<false>(hub.a[buf], hub.b[buf], hub.v[buf], len, pp, vel, sa, pu);
          else hub_chunk_resumed<true>(hub.a[buf], hub.b[buf], hub.v[buf], len, pp, vel, sa, pu);
        }
        absent = __syncthreads_or(next & kStagedAbsent);
        strengths = __syncthreads_or(next & kStagedStrength);
      }
      if (threadIdx.x == 0) dst[p] = (f & kPinned) ? pp : integrate(pp, vel.x, vel.y, s.friction, s.space);
      return;
    }
    // round c: chain over chunk c, staging of chunk c + 1, check of chunk c - 1
    for (uint32_t c = 0; c <= chunks; ++c) {
      const int buf = c % kHubBufs, prev = (c + kHubBufs - 1) % kHubBufs;
      int next = 0;
      bool bad = false;
      if (threadIdx.x >= 32) {
        if (c + 1 < chunks)
          next = hub_fill(hub, (c + 1) % kHubBufs, e0 + (c + 1) * kHubChunk, e1, ent, src, span, s.link_r0,
                          s.link_distance);
        const uint32_t k = threadIdx.x - 32;
        if (c > 0 && hub.fast[prev] && k < chunk_len(c - 1)) {
          const float4 a = hub.a[prev][k];
          bad = !spring_chain_check(pp, hub.v[prev][k], make_float2(a.x, a.y), a.z, a.w, hub.b[prev][k].w, pu);
        }
      } else if (threadIdx.x == 0 && c < chunks) {
        const uint32_t len = chunk_len(c);
        if (absent) {   // absent targets: the correctly rounded springs, skipping them
          hub_chunk_exact(hub.a[buf], hub.b[buf], len, pp, vel, sa, pu);
          hub.fast[buf] = 0;
        } else {        // no per-link branch: the chain runs back to back
          if (strengths) hub_chunk_chain<false>(hub.a[buf], hub.b[buf], hub.v[buf], len, pp, vel, sa, pu);
          else hub_chunk_chain<true>(hub.a[buf], hub.b[buf], hub.v[buf], len, pp, vel, sa, pu);
          hub.fast[buf] = 1;
        }
      }
      absent = __syncthreads_or(next & kStagedAbsent);
      strengths = __syncthreads_or(next & kStagedStrength);
      if (__syncthreads_or(bad)) {   // chunk c - 1 left the sequences: it and chunk c again, exactly
        if (threadIdx.x == 0) {
          vel = hub.v[prev][0];
          hub_chunk_exact(hub.a[prev], hub.b[prev], chunk_len(c - 1), pp, vel, sa, pu);
          if (c < chunks) {
            hub_chunk_exact(hub.a[buf], hub.b[buf], chunk_len(c), pp, vel, sa, pu);
            hub.fast[buf] = 0;
          }
        }
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) dst[p] = (f & kPinned) ? pp : integrate(pp, vel.x, vel.y, s.friction, s.space);
    return;
  }
  const uint32_t t = nhub + (bx - nhub) * kBlock + threadIdx.x;
  if (t >= nrows) return;
  const uint32_t p = rows[t];
  const float2 pp = src[p];
  const uint8_t f = d.flags[p];
  if (f & kAbsent) { dst[p] = pp; return; }
  // This lane's list in its warp's block: entry k at 32 k (one coalesced load
  // per entry for the warp), padded with absent entries to the warp's longest.
  const uint32_t lt = t - nhub;
  const uint32_t o0 = woff[lt >> 5], cnt = (woff[(lt >> 5) + 1] - o0) >> 5;
  const uint4* col = lane_ent + o0 + (lt & 31);
  // The loads do not depend on the running velocity: issue them kLinkBatch
  // links ahead, then apply the springs strictly in list order.
  // Short lists on many threads: the correctly rounded springs (spring_step);
  // the in-range sequences save latency on a hub's long chain, not here.
  float2 vel = make_float2(0.f, 0.f);
  auto spring = [&](const uint4 en, const float2 q) {
    float dd = __fadd_rn(__fmul_rn(__uint_as_float(en.y), span), s.link_r0);
    dd = __fmul_rn(dd, s.link_distance);
    spring_step(pp, vel, q, dd, __fmul_rn(dd, 0.99f), sa, __uint_as_float(en.w), __uint_as_float(en.z), pu);
  };

  constexpr int kLinkBatch = 4;
  uint32_t at = 0;
  for (; at + kLinkBatch <= cnt; at += kLinkBatch) {
    uint4 en[kLinkBatch];
    float2 q[kLinkBatch];
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) en[u] = __ldg(&col[32 * (at + u)]);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) q[u] = en[u].x != kAbsentTarget ? __ldg(&src[en[u].x]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u)
      if (en[u].x != kAbsentTarget) spring(en[u], q[u]);
  }
  for (; at < cnt; ++at) {
    const uint4 en = __ldg(&col[32 * at]);
    if (en.x == kAbsentTarget) continue;
    spring(en, __ldg(&src[en.x]));
  }
  dst[p] = (f & kPinned) ? pp : integrate(pp, vel.x, vel.y, s.friction, s.space);
}

__global__ void __launch_bounds__(kBlock) k_warp_lengths(const uint32_t* __restrict__ order,
                                                         const uint32_t* __restrict__ rowptr, uint32_t nhub,
                                                         uint32_t n, uint32_t* __restrict__ woff) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nw = (n - nhub + 31) / 32;
  if (w > nw) return;
  uint32_t len = 0;
  if (w < nw) {   // the first row of a warp has its longest list
    const uint32_t p = order[nhub + 32 * w];
    len = rowptr[p + 1] - rowptr[p];
  }
  woff[w] = 32 * len;
}

__global__ void __launch_bounds__(kBlock) k_fill_lanes(const uint32_t* __restrict__ order,
                                                       const uint32_t* __restrict__ rowptr,
                                                       const uint4* __restrict__ ent, uint32_t nhub, uint32_t n,
                                                       const uint32_t* __restrict__ woff, uint4* __restrict__ lane_ent) {
  const uint32_t lt = blockIdx.x * blockDim.x + threadIdx.x;
  if (lt >= n - nhub) return;
  const uint32_t p = order[nhub + lt];
  const uint32_t e0 = rowptr[p], len = rowptr[p + 1] - e0;
  const uint32_t o0 = woff[lt >> 5], cnt = (woff[(lt >> 5) + 1] - o0) >> 5;
  uint4* col = lane_ent + o0 + (lt & 31);
  for (uint32_t k = 0; k < cnt; ++k) col[32 * k] = k < len ? ent[e0 + k] : make_uint4(kAbsentTarget, 0u, 0u, 0u);
}


// -------------------------------------------------------------- collision --
// The arithmetic is collision.cuh's, shared with the batched engine.
// Points are taken in `order` (the many-body pass's cell order) when given,
// so the lanes of a warp fall into a few grid cells.
__global__ void __launch_bounds__(kBlock) k_coll_grid(DeviceView d, SimScalars s, const uint32_t* __restrict__ order,
                                                      uint32_t count, const uint8_t* __restrict__ skip) {
  // build-grid.vert:28-62 for the 4 offsets (ForceCollision/index.ts:19-24);
  // points marked in `skip` are left to another launch (integer sums: the
  // grids do not depend on the order in which points are added)
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t i = 0;
  bool live = t < count;
  if (live) {
    i = order ? order[t] : t;
    live = !(d.flags[i] & kAbsent) && !(skip && skip[i]);
  }
  if (!__any_sync(0xffffffffu, live)) return;   // warp-uniform
  float2 p = make_float2(0.f, 0.f);
  float sz = 0.f;
  if (live) { p = d.pos[i]; sz = d.size[i]; }
  coll_accumulate(d.cgrid_acc, s.coll_grid, s.coll_cell, s.fx, p, sz, live);
}

template <bool ZERO>
__global__ void __launch_bounds__(kBlock) k_coll_convert(DeviceView d, SimScalars s) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = 4u * (uint32_t)(s.coll_grid * s.coll_grid);
  if (k >= total) return;
  coll_convert_cell<ZERO>(d.cgrid_acc + 4 * (size_t)k, d.cgrid + k, s.fx);
}

__global__ void __launch_bounds__(kBlock) k_coll_force(DeviceView d, SimScalars s, const uint32_t* __restrict__ order,
                                                       uint32_t count) {
  // force-collision-spatial.frag:103-168, 4 passes blended, then update
  const TickParams tp = tick_params(d);
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const uint32_t i = order ? order[t] : t;   // cell order: neighbouring lanes read the same grid cells
  const uint8_t f = d.flags[i];
  if (f & kAbsent) return;
  const float2 p = d.pos[i];
  const CollParams cp{s.coll_grid, s.coll_cell, s.coll_radius, s.coll_padding, __fmul_rn(tp.alpha, s.coll_strength)};
  const float2 v = coll_velocity(d.cgrid, cp, p, d.size[i], i, d.n);
  if (!(f & kPinned)) d.pos[i] = integrate(p, v.x, v.y, s.friction, s.space);
}

// k_coll_force into pos_coll, every point but the late ones (absent and
// pinned points copied), from grids that lack the late points.
__global__ void __launch_bounds__(kBlock) k_coll_force_early(DeviceView d, SimScalars s,
                                                             const uint32_t* __restrict__ order, uint32_t count,
                                                             const uint8_t* __restrict__ late) {
  const TickParams tp = tick_params(d);
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const uint32_t i = order ? order[t] : t;
  if (late[i]) return;
  const uint8_t f = d.flags[i];
  const float2 p = d.pos[i];
  float2 out = p;
  if (!(f & (kAbsent | kPinned))) {
    const CollParams cp{s.coll_grid, s.coll_cell, s.coll_radius, s.coll_padding,
                        __fmul_rn(tp.alpha, s.coll_strength)};
    const float2 v = coll_velocity(d.cgrid, cp, p, d.size[i], i, d.n);
    out = integrate(p, v.x, v.y, s.friction, s.space);
  }
  d.pos_coll[i] = out;
}

// One thread per (late point, grid, cell of its 3x3 window): the window's
// cells marked; the centre thread converts the late point's cell again from
// the sums that now hold every point (the same value for late points sharing
// a cell).
__global__ void __launch_bounds__(kBlock) k_coll_late(DeviceView d, SimScalars s,
                                                      const uint32_t* __restrict__ late_list, uint32_t n_late) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_late * 36u) return;
  const uint32_t i = late_list[t / 36u];
  if (d.flags[i] & kAbsent) return;
  const int g = (int)((t / 9u) % 4u), w = (int)(t % 9u);
  const int G = s.coll_grid;
  const float gm1 = (float)G - 1.0f;
  const float2 p = d.pos[i];
  const int cx = (int)coll_bin(p.x, coll_offset_x(g), s.coll_cell, gm1);
  const int cy = (int)coll_bin(p.y, coll_offset_y(g), s.coll_cell, gm1);
  const uint32_t G2 = (uint32_t)(G * G);
  if (w == 4) {
    const uint32_t k = (uint32_t)g * G2 + (uint32_t)(cy * G + cx);
    coll_convert_cell<false>(d.cgrid_acc + 4 * (size_t)k, d.cgrid + k, s.fx);
  }
  const int mx = cx + w % 3 - 1, my = cy + w / 3 - 1;
  if (mx < 0 || mx >= G || my < 0 || my >= G) return;
  const uint32_t bit = (uint32_t)g * G2 + (uint32_t)(my * G + mx);
  atomicOr(&d.coll_mark[bit >> 5], 1u << (bit & 31u));
}

// Every live point's final collision result into pos: pos_coll's, or, when
// the point is late or one of its four cells is marked, listed in coll_redo
// (a warp's entries with one atomic): those points are scattered over the
// indices (a hub's link targets gather in its cells), so k_coll_redo computes
// them with every lane busy.
__global__ void __launch_bounds__(kBlock) k_coll_fixup(DeviceView d, SimScalars s, const uint8_t* __restrict__ late) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool again = false;
  if (i < d.n && !(d.flags[i] & kAbsent)) {   // absent points keep their (NaN) position
    const float2 p = d.pos[i];
    const int G = s.coll_grid;
    const float gm1 = (float)G - 1.0f;
    const uint32_t G2 = (uint32_t)(G * G);
    again = late[i] != 0;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int cx = (int)coll_bin(p.x, coll_offset_x(g), s.coll_cell, gm1);
      const int cy = (int)coll_bin(p.y, coll_offset_y(g), s.coll_cell, gm1);
      const uint32_t bit = (uint32_t)g * G2 + (uint32_t)(cy * G + cx);
      again |= (__ldg(&d.coll_mark[bit >> 5]) >> (bit & 31u)) & 1u;
    }
    if (!again) d.pos[i] = d.pos_coll[i];
  }
  const unsigned m = __ballot_sync(0xffffffffu, again);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&d.coll_redo[0], (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (again) d.coll_redo[1 + base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = i;
}

// The listed points' collision results from the complete grids (grid-stride
// over the device-side count).
__global__ void __launch_bounds__(kBlock) k_coll_redo(DeviceView d, SimScalars s) {
  const uint32_t count = d.coll_redo[0];
  const TickParams tp = tick_params(d);
  const CollParams cp{s.coll_grid, s.coll_cell, s.coll_radius, s.coll_padding, __fmul_rn(tp.alpha, s.coll_strength)};
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
    const uint32_t i = d.coll_redo[1 + t];
    if (d.flags[i] & kPinned) continue;
    const float2 p = d.pos[i];
    const float2 v = coll_velocity(d.cgrid, cp, p, d.size[i], i, d.n);
    d.pos[i] = integrate(p, v.x, v.y, s.friction, s.space);
  }
}

// --------------------------------------------------------------- clusters --
// Clusters.run (Clusters/index.ts:426-469).  Centre of mass per cluster
// (calculate-centermass.vert:22-52: live, clustered points only) as exact
// integer sums.  The lanes of a warp sum their terms per cluster first
// (kCollRounds distinct clusters per warp, the rest add their own); with at
// most kClusterSmem clusters a block also sums in shared memory and adds each
// cluster's total once, so a few clusters do not serialise on a few atomics.
constexpr uint32_t kClusterSmem = 256;

template <bool SMEM>
__global__ void __launch_bounds__(kBlock) k_cluster_sum(DeviceView d, SimScalars s) {
  __shared__ unsigned long long tab[SMEM ? 3 * kClusterSmem : 1];
  const uint32_t K = d.n_clusters;
  if (SMEM) {
    for (uint32_t k = threadIdx.x; k < 3 * K; k += blockDim.x) tab[k] = 0;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  auto add = [&](uint32_t c, long long x, long long y, long long n) {
    unsigned long long* a = SMEM ? &tab[3 * c] : (unsigned long long*)&d.cluster_acc[3 * (size_t)c];
    atomicAdd(&a[0], (unsigned long long)x);
    atomicAdd(&a[1], (unsigned long long)y);
    atomicAdd(&a[2], (unsigned long long)n);
  };
  const uint32_t stride = SMEM ? gridDim.x * blockDim.x : d.n;
  for (uint32_t base = blockIdx.x * blockDim.x; base < d.n; base += stride) {   // uniform per block
    const uint32_t i = base + threadIdx.x;
    uint32_t c = kNoClusterId;
    bool on = i < d.n;
    if (on) {
      c = d.cluster_of[i];
      on = c != kNoClusterId && !(d.flags[i] & kAbsent);
    }
    unsigned todo = __ballot_sync(0xffffffffu, on);
    if (!todo) continue;   // warp-uniform
    const float2 p = on ? d.pos[i] : make_float2(0.f, 0.f);
    const long long fx = on ? to_fixed(p.x, s.fx) : 0, fy = on ? to_fixed(p.y, s.fx) : 0;
#pragma unroll 1
    for (int r = 0; r < kCollRounds && todo; ++r) {
      const int l = __ffs(todo) - 1;
      const uint32_t cl = __shfl_sync(0xffffffffu, c, l);
      const bool mine = ((todo >> lane) & 1u) && c == cl;
      const unsigned grp = __ballot_sync(0xffffffffu, mine);
      const long long sx = warp_sum64(mine ? fx : 0);
      const long long sy = warp_sum64(mine ? fy : 0);
      if (lane == l) add(cl, sx, sy, __popc(grp));
      todo &= ~grp;
    }
    if ((todo >> lane) & 1u) add(c, fx, fy, 1);
  }
  if (SMEM) {
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
      if (!tab[3 * k + 2]) continue;
      unsigned long long* a = (unsigned long long*)&d.cluster_acc[3 * (size_t)k];
      atomicAdd(&a[0], tab[3 * k]);
      atomicAdd(&a[1], tab[3 * k + 1]);
      atomicAdd(&a[2], tab[3 * k + 2]);
    }
  }
}

// force-cluster.frag:28-53, then the update (update-position.frag:26-59).
__global__ void __launch_bounds__(kBlock) k_cluster_force(DeviceView d, SimScalars s) {
  const TickParams tp = tick_params(d);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const uint8_t f = d.flags[i];
  if (f & kAbsent) return;   // absent points keep their (NaN) position
  const float2 p = d.pos[i];
  float vx = 0.f, vy = 0.f;
  const uint32_t c = d.cluster_of[i];
  if (c != kNoClusterId) {
    float2 t = d.cluster_custom[c];
    if (t.x < 0.f || t.y < 0.f) {   // no custom position: centre of mass
      const long long* a = d.cluster_acc + 3 * (size_t)c;
      const float cnt = (float)a[2];
      t = make_float2(__fdiv_rn(from_fixed(a[0], s.fx), cnt), __fdiv_rn(from_fixed(a[1], s.fx), cnt));
    }
    const float dx = __fsub_rn(t.x, p.x), dy = __fsub_rn(t.y, p.y);
    const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    if (dist > 0.f) {
      const float add = __fmul_rn(__fmul_rn(__fmul_rn(tp.alpha, dist), s.cluster), d.cluster_coeff[i]);
      const float inv = __frcp_rn(dist);   // normalize(v) = v * (1 / length(v))
      // velocity starts at vec4(0) and `+=` adds to it: 0 + w turns a -0 into +0
      vx = __fadd_rn(0.f, __fmul_rn(add, __fmul_rn(dx, inv)));
      vy = __fadd_rn(0.f, __fmul_rn(add, __fmul_rn(dy, inv)));
    }
  }
  if (!(f & kPinned)) d.pos[i] = integrate(p, vx, vy, s.friction, s.space);
}

__global__ void k_tick_end(DeviceView d) { *d.tick_ctr += 1; }

// ---------------------------------------------------------------- pointer --
// force-mouse.frag:23-38 then the update: push away from the pointer with
// 100 * repulsion / max(|d|, 10)^2 along (cos, sin)(atan(d.y, d.x)) = d / |d|
// (the direction of atan2(0, 0) = 0, (1, 0), when the pointer is on the point).
__global__ void __launch_bounds__(kBlock) k_mouse(DeviceView d, SimScalars s, float2 mouse, float repulsion) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const uint8_t f = d.flags[i];
  if (f & (kAbsent | kPinned)) return;
  const float2 p = d.pos[i];
  const float dx = __fsub_rn(mouse.x, p.x), dy = __fsub_rn(mouse.y, p.y);
  const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  const float dist = gmax(r, 10.0f);
  const float add = __fdiv_rn(__fmul_rn(100.0f, repulsion), __fmul_rn(dist, dist));
  float cx = 1.f, cy = 0.f;
  if (r > 0.f) { cx = __fdiv_rn(dx, r); cy = __fdiv_rn(dy, r); }
  const float vx = __fsub_rn(0.f, __fmul_rn(add, cx)), vy = __fsub_rn(0.f, __fmul_rn(add, cy));
  d.pos[i] = integrate(p, vx, vy, s.friction, s.space);
}

// drag-point.frag:22-31: the texel whose index channel equals the dragged
// index takes the pointer position (pinned and absence flags are not consulted).
__global__ void k_drag(DeviceView d, uint32_t index, float2 mouse) { d.pos[index] = mouse; }

// buildPositionTextureData (Points/position-utils.ts:9-27): texel i = (x, y, i, 0)
// for the points, zeros for the rest of the T x T texture.
__global__ void __launch_bounds__(kBlock) k_position_texture(DeviceView d, float4* __restrict__ out, uint32_t texels) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= texels) return;
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (t < d.n) {
    const float2 p = d.pos[t];
    v = make_float4(p.x, p.y, (float)t, 0.f);
  }
  out[t] = v;
}

inline uint32_t blocks_for(uint32_t n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

uint32_t scan_blocks(uint32_t cells) { return (cells + kScanChunk - 1) / kScanChunk; }

void launch_prepass(const DeviceView& d, const SimScalars& s, uint32_t mode, cudaStream_t st) {
  const uint32_t nb = blocks_for(d.n);
  if (nb == 0) return;
  switch (mode) {
    case kPreGravity: k_prepass<kPreGravity><<<nb, kBlock, 0, st>>>(d, s); break;
    case kPreGravity | kPreBin: k_prepass<kPreGravity | kPreBin><<<nb, kBlock, 0, st>>>(d, s); break;
    case kPreGravity | kPreCentroid: k_prepass<kPreGravity | kPreCentroid><<<nb, kBlock, 0, st>>>(d, s); break;
    case kPreCentroid: k_prepass<kPreCentroid><<<nb, kBlock, 0, st>>>(d, s); break;
    case kPreBin: k_prepass<kPreBin><<<nb, kBlock, 0, st>>>(d, s); break;
    default: break;
  }
}

void launch_center(const DeviceView& d, const SimScalars& s, bool bin, cudaStream_t st) {
  const uint32_t nb = blocks_for(d.n);
  if (nb == 0) return;
  if (bin) k_center<true><<<nb, kBlock, 0, st>>>(d, s);
  else k_center<false><<<nb, kBlock, 0, st>>>(d, s);
}

namespace {
// Chunk 1 looks back at chunk 0, whose status word nothing sets (all zero).
__global__ void k_wait_limit(const unsigned long long* status, uint32_t* error) {
  if (threadIdx.x < 32) (void)scan_look_back(status, 1u, 0ull, error, kErrorScan);
}
}  // namespace

void launch_wait_limit(const unsigned long long* status, uint32_t* error, cudaStream_t st) {
  k_wait_limit<<<1, 32, 0, st>>>(status, error);
}

void launch_scan(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  const uint32_t cells = (uint32_t)(s.gf * s.gf);
  const uint32_t nb = scan_blocks(cells);
  if (s.pairs) k_scan<true><<<nb, kBlock, 0, st>>>(d, cells);
  else k_scan<false><<<nb, kBlock, 0, st>>>(d, cells);
}

void launch_scatter(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  const uint32_t nb = blocks_for(d.n);
  if (!nb) return;
  const uint32_t cells = (uint32_t)(s.gf * s.gf);
  if (s.pairs) k_scatter<true><<<nb, kBlock, 0, st>>>(d, cells);
  else k_scatter<false><<<nb, kBlock, 0, st>>>(d, cells);
}

void launch_cells(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  // grid-stride over the dense cells; blocks beyond one resident wave (3 per SM)
  // start as others finish and even out the cells' unequal sizes (measured
  // best at 8 per SM).  A graph of n points has at most n / (kSmallCell + 1)
  // dense cells: small graphs launch a warp for each, not 8 idle blocks per SM.
  const uint32_t most = d.n / (kSmallCell + 1);
  const uint32_t nb = std::min(8u * sm_count(), std::max(1u, (most + kBlock / 32 - 1) / (kBlock / 32)));
  k_bigcells<<<nb, kBlock, 0, st>>>(d, s);
  const int tiles = (s.gf / s.tile) * (s.gf / s.tile);
  const size_t smem = 3 * sizeof(long long) * s.tile * s.tile;
  k_cells<<<tiles, s.tile * s.tile, smem, st>>>(d, s);
}

// With fewer than two blocks of one-thread points per SM the GPU is short of
// warps and each point's serial chain of terms sets the pass time; below that
// the split kernel spreads a point over 16 threads (2k-50k points: 1.2-2x
// faster; at 100k it is 16% slower).
// Graphs with at least one point per finest cell on average (the finest grid
// is capped at 512, so from 262,144 points) take two points of a cell per
// thread: at most (n + cells) / 2 work items.
void launch_manybody(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  if (!d.n) return;
  if (s.pairs) {
    const uint32_t items = (uint32_t)(((uint64_t)d.n + (uint64_t)s.gf * s.gf) / 2 + 1);
    if (s.level_guard) k_manybody_duo<true><<<blocks_for(items), kBlock, 0, st>>>(d, s);
    else k_manybody_duo<false><<<blocks_for(items), kBlock, 0, st>>>(d, s);
  } else if (s.mb_kernel == kManybodySplit) {
    k_manybody_split<<<(d.n + kSplitPoints - 1) / kSplitPoints, kBlock, 0, st>>>(d, s);
  } else {
    k_manybody<<<blocks_for(d.n), kBlock, 0, st>>>(d, s);
  }
}

void launch_manybody_early(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  if (d.n_early_pts) k_manybody_early<<<blocks_for(d.n_early_pts), kBlock, 0, st>>>(d, s);
}

// The leading hubs' CTAs ask for all the shared memory a CTA may have, so no
// other CTA shares their SM: the chain thread then issues without the
// many-body warps beside it (each CTA also holds 1 KB of the SM's 228 KB).
// sizeof(HubStage) where the device does not allow that much.  Set once per
// device (the attribute is per device; concurrent first calls set the same).
static size_t hub_exclusive_smem() {
  constexpr int kDevices = 64;
  static std::atomic<size_t> bytes[kDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) {
    cudaGetLastError();
    return sizeof(HubStage);
  }
  size_t b = bytes[dev].load(std::memory_order_relaxed);
  if (!b) {
    int optin = 0;
    b = sizeof(HubStage);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
        (size_t)optin > b &&
        cudaFuncSetAttribute(k_link, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) == cudaSuccess)
      b = (size_t)optin;
    cudaGetLastError();   // a refused attribute leaves no error behind
    bytes[dev].store(b, std::memory_order_relaxed);
  }
  return b;
}

void launch_link(const DeviceView& d, const SimScalars& s, int direction, bool swap_back, cudaStream_t st,
                 int part) {
  if (!d.n) return;
  const uint32_t* rp = direction == 0 ? d.rowptr_in : d.rowptr_out;
  const uint4* en = direction == 0 ? d.ent_in : d.ent_out;
  const uint32_t* order = direction == 0 ? d.heavy_in : d.heavy_out;   // all points, longest lists first
  const uint32_t nhub = direction == 0 ? d.n_heavy_in : d.n_heavy_out;
  const uint32_t* woff = direction == 0 ? d.woff_in : d.woff_out;
  const uint4* lane_ent = direction == 0 ? d.lane_ent_in : d.lane_ent_out;
  const float2* src = swap_back ? d.pos_alt : d.pos;
  float2* dst = swap_back ? d.pos : d.pos_alt;
  const uint32_t nlight = blocks_for(d.n - nhub);
  const uint32_t early = std::min(direction == 0 ? d.n_early_hubs : d.n_first_out, nhub);
  const uint32_t next = direction == 0 ? 0u : std::min(d.n_next_out, nhub - early);
  const uint32_t lead = early + next;
  if (part == kLinkHubs) {
    if (nhub) k_link<<<nhub, kBlock, sizeof(HubStage), st>>>(d, s, rp, en, woff, lane_ent, src, dst, order, d.n, nhub, 0u);
  } else if (part == kLinkFirstHubs) {
    if (early)
      k_link<<<early, kBlock, hub_exclusive_smem(), st>>>(d, s, rp, en, woff, lane_ent, src, dst, order, d.n, nhub, 0u);
  } else if (part == kLinkNextHubs) {
    if (next)
      k_link<<<next, kBlock, sizeof(HubStage), st>>>(d, s, rp, en, woff, lane_ent, src, dst, order, d.n, nhub, early);
  } else if (part == kLinkAfterFirst) {
    const uint32_t nb = nhub - lead + nlight;
    if (nb)
      k_link<<<nb, kBlock, nhub > lead ? sizeof(HubStage) : 0, st>>>(d, s, rp, en, woff, lane_ent, src, dst, order,
                                                                      d.n, nhub, lead);
  } else if (part == kLinkLight) {
    if (nlight) k_link<<<nlight, kBlock, 0, st>>>(d, s, rp, en, woff, lane_ent, src, dst, order, d.n, nhub, nhub);
  } else {
    k_link<<<nhub + nlight, kBlock, nhub ? sizeof(HubStage) : 0, st>>>(d, s, rp, en, woff, lane_ent, src, dst, order,
                                                                      d.n, nhub, 0u);
  }
}

namespace {
__global__ void __launch_bounds__(kBlock) k_mark_hubs(const uint32_t* __restrict__ order, uint32_t nhub,
                                                      uint8_t* __restrict__ mark) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nhub) mark[order[t]] = 1;
}
}  // namespace

void launch_mark_hubs(const uint32_t* order, uint32_t nhub, uint8_t* mark, cudaStream_t st) {
  if (nhub) k_mark_hubs<<<blocks_for(nhub), kBlock, 0, st>>>(order, nhub, mark);
}

namespace {
__global__ void __launch_bounds__(kBlock) k_hub_spans(const uint32_t* __restrict__ order,
                                                      const uint32_t* __restrict__ rowptr, uint32_t m,
                                                      uint2* __restrict__ spans) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) spans[t] = make_uint2(rowptr[order[t]], rowptr[order[t] + 1]);
}
}  // namespace

void launch_hub_spans(const uint32_t* order, const uint32_t* rowptr, uint32_t m, uint2* spans, cudaStream_t st) {
  if (m) k_hub_spans<<<blocks_for(m), kBlock, 0, st>>>(order, rowptr, m, spans);
}

namespace {
__global__ void __launch_bounds__(kBlock) k_cell_keys(const float2* __restrict__ pos, const uint32_t* __restrict__ pts,
                                                      uint32_t m, float csf, int gf, uint32_t* __restrict__ keys) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const float2 p = pos[pts[t]];
  keys[t] = (uint32_t)cell_index(p.y, csf, gf) * (uint32_t)gf + (uint32_t)cell_index(p.x, csf, gf);
}
}  // namespace

void launch_cell_keys(const float2* pos, const uint32_t* pts, uint32_t m, float csf, int gf, uint32_t* keys,
                      cudaStream_t st) {
  if (m) k_cell_keys<<<blocks_for(m), kBlock, 0, st>>>(pos, pts, m, csf, gf, keys);
}

void launch_warp_lengths(const uint32_t* order, const uint32_t* rowptr, uint32_t nhub, uint32_t n, uint32_t* woff,
                         cudaStream_t st) {
  const uint32_t nw = (n - nhub + 31) / 32;
  k_warp_lengths<<<blocks_for(nw + 1), kBlock, 0, st>>>(order, rowptr, nhub, n, woff);
}

void launch_fill_lanes(const uint32_t* order, const uint32_t* rowptr, const uint4* ent, uint32_t nhub, uint32_t n,
                       const uint32_t* woff, uint4* lane_ent, cudaStream_t st) {
  const uint32_t nb = blocks_for(n - nhub);
  if (nb) k_fill_lanes<<<nb, kBlock, 0, st>>>(order, rowptr, ent, nhub, n, woff, lane_ent);
}

void launch_cluster_sum(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  if (!d.n) return;
  if (d.n_clusters <= kClusterSmem)
    k_cluster_sum<true><<<std::min(blocks_for(d.n), 4u * sm_count()), kBlock, 0, st>>>(d, s);
  else
    k_cluster_sum<false><<<blocks_for(d.n), kBlock, 0, st>>>(d, s);
}

void launch_cluster_force(const DeviceView& d, const SimScalars& s, cudaStream_t st) {
  const uint32_t nb = blocks_for(d.n);
  if (nb) k_cluster_force<<<nb, kBlock, 0, st>>>(d, s);
}

void launch_collision_sums(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                           const uint8_t* skip, cudaStream_t st) {
  if (!order) count = d.n;
  const uint32_t nb = blocks_for(count);
  if (nb) k_coll_grid<<<nb, kBlock, 0, st>>>(d, s, order, count, skip);
}

void launch_collision_convert(const DeviceView& d, const SimScalars& s, cudaStream_t st, bool zero) {
  const uint32_t cells = 4u * (uint32_t)(s.coll_grid * s.coll_grid);
  if (zero) k_coll_convert<true><<<blocks_for(cells), kBlock, 0, st>>>(d, s);
  else k_coll_convert<false><<<blocks_for(cells), kBlock, 0, st>>>(d, s);
}

void launch_collision_force_early(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                                  const uint8_t* late, cudaStream_t st) {
  if (!order) count = d.n;
  const uint32_t nb = blocks_for(count);
  if (nb) k_coll_force_early<<<nb, kBlock, 0, st>>>(d, s, order, count, late);
}

void launch_collision_late(const DeviceView& d, const SimScalars& s, const uint32_t* late_list, uint32_t n_late,
                           cudaStream_t st) {
  if (n_late) k_coll_late<<<blocks_for(n_late * 36u), kBlock, 0, st>>>(d, s, late_list, n_late);
}

void launch_collision_fixup(const DeviceView& d, const SimScalars& s, const uint8_t* late, cudaStream_t st) {
  const uint32_t nb = blocks_for(d.n);
  if (!nb) return;
  k_coll_fixup<<<nb, kBlock, 0, st>>>(d, s, late);
  k_coll_redo<<<std::min(nb, 8u * sm_count()), kBlock, 0, st>>>(d, s);
}

void launch_collision_grid(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                           cudaStream_t st) {
  launch_collision_sums(d, s, order, count, nullptr, st);
  launch_collision_convert(d, s, st);
}

void launch_collision_force(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                            cudaStream_t st) {
  if (!order) count = d.n;
  const uint32_t nb = blocks_for(count);
  if (nb) k_coll_force<<<nb, kBlock, 0, st>>>(d, s, order, count);
}

void launch_tick_end(const DeviceView& d, cudaStream_t st) { k_tick_end<<<1, 1, 0, st>>>(d); }

void launch_mouse(const DeviceView& d, const SimScalars& s, float2 mouse, float repulsion, cudaStream_t st) {
  const uint32_t nb = blocks_for(d.n);
  if (nb) k_mouse<<<nb, kBlock, 0, st>>>(d, s, mouse, repulsion);
}

void launch_drag(const DeviceView& d, uint32_t index, float2 mouse, cudaStream_t st) {
  if (index < d.n) k_drag<<<1, 1, 0, st>>>(d, index, mouse);
}

void launch_position_texture(const DeviceView& d, float4* out, uint32_t texels, cudaStream_t st) {
  const uint32_t nb = blocks_for(texels);
  if (nb) k_position_texture<<<nb, kBlock, 0, st>>>(d, out, texels);
}

}  // namespace cgl
