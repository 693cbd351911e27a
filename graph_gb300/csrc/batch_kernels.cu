// batch_kernels.cu — one tick of many graphs at once.
//
// The per-graph arithmetic is the plain engine's (kernels.cu), operation for
// operation; only the addressing differs: each point or cell finds its graph
// (gid / cell_gid), its graph's descriptor and its graph's tick parameters.
// Point indices that enter the arithmetic (peel hash, tie-break, self test)
// are graph-local, so a graph advances exactly as it would alone.
#include "batch.cuh"
#include "collision.cuh"
#include "manybody_duo.cuh"
#include "device_util.cuh"
#include "warp_cells.cuh"

namespace cgl {
namespace {


__device__ __forceinline__ const BatchTick& tick_of(const BatchView& v, uint32_t g) {
  return v.ticks[(size_t)(*v.tick_ctr) * v.slots + g];
}

__device__ __forceinline__ uint32_t level_base(int l) {
  // sum over m < l of (4 << m)^2 = 16 (4^l - 1) / 3
  return (uint32_t)(16u * (((1u << (2 * l)) - 1u) / 3u));
}

// ---------------------------------------------------------------- prepass --

__device__ __forceinline__ void kb_bin(const BatchView& v, const GraphDesc& D, uint32_t P, float2 p) {
  const int cx = cell_index(p.x, D.csf, D.gf), cy = cell_index(p.y, D.csf, D.gf);
  const uint32_t key = D.cell_off + (uint32_t)(cy * D.gf + cx);
  v.key[P] = key;
  v.rank[P] = atomicAdd(&v.counts[key], 1u);
  const bool outside = !(p.x >= 0.f && p.x <= D.space && p.y >= 0.f && p.y <= D.space);
  const unsigned am = __activemask();
  if (__ballot_sync(am, outside) && (threadIdx.x & 31) == (unsigned)(__ffs(am) - 1))
    atomicOr(&v.big_count[kBatchOutside], 1u);
}

// Adds each `live` lane's exact (x, y, 1) into its graph's centroid sums; all
// 32 lanes take part.  The lanes of one graph (points of a graph are
// contiguous in the arena, so a warp holds one or two) sum first and one lane
// adds the totals.  Integer sums: the order does not matter.
__device__ __forceinline__ void centroid_accumulate(const BatchView& v, uint32_t g, bool live, long long sx,
                                                    long long sy) {
  const int lane = threadIdx.x & 31;
  unsigned todo = __ballot_sync(0xffffffffu, live);
  while (todo) {
    const int l = __ffs(todo) - 1;
    const uint32_t gl = __shfl_sync(0xffffffffu, g, l);
    const bool mine = ((todo >> lane) & 1u) && g == gl;
    const unsigned grp = __ballot_sync(0xffffffffu, mine);
    const long long tx = warp_sum64(mine ? sx : 0), ty = warp_sum64(mine ? sy : 0);
    if (lane == l) {
      long long* c = v.centroid + 3 * (size_t)gl;
      atomicAdd((unsigned long long*)&c[0], (unsigned long long)tx);
      atomicAdd((unsigned long long*)&c[1], (unsigned long long)ty);
      atomicAdd((unsigned long long*)&c[2], (unsigned long long)__popc(grp));
    }
    todo &= ~grp;
  }
}

// Gravity and binning (k_prepass); a graph with the center force sums its
// centroid here instead and bins in kb_center, after the pull.
__global__ void __launch_bounds__(kBlock) kb_prepass(BatchView v) {
  const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t g = kNoGraph;
  bool centre = false;
  long long sx = 0, sy = 0;
  if (P < v.point_hwm && (g = v.gid[P]) != kNoGraph) {
    const GraphDesc& D = v.desc[g];
    const BatchTick tp = tick_of(v, g);
    if (!tp.active) {
      v.key[P] = kNoCell;
    } else {
      const uint8_t f = v.flags[P];
      float2 p = v.pos[P];
      if (D.stages & kGGravity) {   // force-gravity.frag:24-40
        const float c = __fmul_rn(D.space, 0.5f);
        const float dx = __fsub_rn(c, p.x), dy = __fsub_rn(c, p.y);
        const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
        float vx = 0.f, vy = 0.f;
        if (dist > 0.f) {
          const float add = __fmul_rn(__fmul_rn(__fmul_rn(tp.alpha, D.gravity), dist), 0.1f);
          vx = __fadd_rn(vx, __fmul_rn(add, __fdiv_rn(dx, dist)));
          vy = __fadd_rn(vy, __fmul_rn(add, __fdiv_rn(dy, dist)));
        }
        if (!(f & (kPinned | kAbsent))) {
          p = integrate(p, vx, vy, D.friction, D.space);
          v.pos[P] = p;
        }
      }
      if (D.stages & kGCenter) {
        // calculate-centermass.vert:18-28 over the live points
        centre = !(f & kAbsent);
        if (centre) { sx = to_fixed(p.x, D.fx); sy = to_fixed(p.y, D.fx); }
      } else if ((D.stages & kGManybody) && !(f & kAbsent)) {
        kb_bin(v, D, P, p);
      } else {
        v.key[P] = kNoCell;
      }
    }
  }
  if (v.any_center) centroid_accumulate(v, g, centre, sx, sy);
}

// ForceCenter.run (ForceCenter/index.ts:149-199): force-center.frag:22-36 from
// the graph's centroid, the update, then the binning.
__global__ void __launch_bounds__(kBlock) kb_center(BatchView v) {
  const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= v.point_hwm) return;
  const uint32_t g = v.gid[P];
  if (g == kNoGraph) return;
  const GraphDesc& D = v.desc[g];
  if (!(D.stages & kGCenter)) return;
  const BatchTick tp = tick_of(v, g);
  if (!tp.active) return;
  const long long* cs = v.centroid + 3 * (size_t)g;
  const float sx = from_fixed(cs[0], D.fx), sy = from_fixed(cs[1], D.fx);
  const float cnt = (float)cs[2];
  const float cmx = __fdiv_rn(sx, cnt), cmy = __fdiv_rn(sy, cnt);
  const uint8_t f = v.flags[P];
  float2 p = v.pos[P];
  const float dx = __fsub_rn(cmx, p.x), dy = __fsub_rn(cmy, p.y);
  const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  float vx = 0.f, vy = 0.f;
  if (dist > 0.f) {
    const float add = __fmul_rn(__fmul_rn(__fmul_rn(tp.alpha, D.center), dist), 0.01f);
    vx = __fadd_rn(vx, __fmul_rn(add, __fdiv_rn(dx, dist)));
    vy = __fadd_rn(vy, __fmul_rn(add, __fdiv_rn(dy, dist)));
  }
  if (!(f & (kPinned | kAbsent))) {
    p = integrate(p, vx, vy, D.friction, D.space);
    v.pos[P] = p;
  }
  if ((D.stages & kGManybody) && !(f & kAbsent)) kb_bin(v, D, P, p);
  else v.key[P] = kNoCell;
}

// ------------------------------------------------------------------- scan --
// The cell histogram's exclusive scan over the used cell arena in one pass
// (device_util.cuh's look-back): cell starts, the histogram zeroed for the
// next tick, the dense cells listed.  A block scans kChunk cells as kScanSub
// coalesced sub-chunks of kBlock x 4 (one look-back per block: more bytes in
// flight per wait).  cell_hwm is a multiple of 64 (every range is a
// power-of-two grid of at least 8 x 8), so a thread's four cells of a
// sub-chunk are all inside or all outside.
__global__ void __launch_bounds__(kBlock) kb_scan(BatchView v) {
  __shared__ unsigned long long s_seq, s_prefix;
  if (threadIdx.x == 0) s_seq = atomicAdd(v.scan_seq, 1ull);
  __syncthreads();
  const uint32_t n = v.cell_hwm, nb = gridDim.x;
  const uint32_t vb = (uint32_t)(s_seq % nb);
  const unsigned long long parity = ((s_seq / nb) & 1ull) << 63;
  uint4 x[kScanSub];
  unsigned long long off[kScanSub], tot[kScanSub];
  unsigned long long total = 0;
#pragma unroll
  for (int k = 0; k < kScanSub; ++k) {
    const uint32_t base = vb * kChunk + k * (kBlock * 4) + threadIdx.x * 4;
    x[k] = base < n ? reinterpret_cast<const uint4*>(v.counts)[base >> 2] : make_uint4(0u, 0u, 0u, 0u);
  }
#pragma unroll
  for (int k = 0; k < kScanSub; ++k) {
    off[k] = block_exclusive_scan64((unsigned long long)x[k].x + x[k].y + x[k].z + x[k].w, &tot[k]);
    total += tot[k];
  }
  if (threadIdx.x < 32) {
    unsigned long long prefix = 0;
    if (vb == 0) {
      if (threadIdx.x == 0) st_relaxed_u64(&v.scan_status[0], parity | kScanInclusive | total);
    } else {
      if (threadIdx.x == 0) st_relaxed_u64(&v.scan_status[vb], parity | kScanTotal | total);
      prefix = scan_look_back(v.scan_status, vb, parity, v.error_word, kBatchErrorScan);
      if (threadIdx.x == 0) st_relaxed_u64(&v.scan_status[vb], parity | kScanInclusive | ((prefix + total) & kScanValue));
    }
    if (threadIdx.x == 0) s_prefix = prefix;
  }
  __syncthreads();
  unsigned long long run = s_prefix;
#pragma unroll
  for (int k = 0; k < kScanSub; ++k) {
    const uint32_t base = vb * kChunk + k * (kBlock * 4) + threadIdx.x * 4;
    if (base < n) {
      const uint32_t o0 = (uint32_t)(run + off[k]), o1 = o0 + x[k].x, o2 = o1 + x[k].y, o3 = o2 + x[k].z;
      reinterpret_cast<uint4*>(v.cell_start)[base >> 2] = make_uint4(o0, o1, o2, o3);
      reinterpret_cast<uint4*>(v.counts)[base >> 2] = make_uint4(0u, 0u, 0u, 0u);
      const uint32_t cnt[4] = {x[k].x, x[k].y, x[k].z, x[k].w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t c = base + q;
        if (cnt[q] > kBigCell) v.big_list[atomicAdd(&v.big_count[0], 1u)] = c;
        else if (cnt[q] > kWarpSmallCell) v.big_list[n + atomicAdd(&v.big_count[1], 1u)] = c;
        else if (cnt[q] > kSmallCell) v.big_list[2 * n - 1 - atomicAdd(&v.big_count[2], 1u)] = c;
      }
    }
    run += tot[k];
  }
  if (vb == nb - 1 && threadIdx.x == 0) v.cell_start[n] = (uint32_t)(s_prefix + total);
}

// ---------------------------------------------------------------- scatter --
__global__ void __launch_bounds__(kBlock) kb_scatter(BatchView v) {
  const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= v.point_hwm) return;
  if (v.gid[P] == kNoGraph) return;
  const uint32_t k = v.key[P];
  if (k == kNoCell) return;
  const uint32_t dst = v.cell_start[k] + v.rank[P];
  v.sorted_idx[dst] = P;
  v.sorted_pos[dst] = v.pos[P];
}

// ------------------------------------------------------------------ cells --
// Slot keys use graph-local indices (the peel hash and tie-break of the
// graph alone).
__device__ __forceinline__ unsigned long long local_key(uint32_t P, uint32_t p_off, uint32_t seed) {
  return peel_key(P - p_off, seed);
}

__device__ void kb_move_head(const BatchView& v, uint32_t b, int ns, uint32_t (&at)[kSlots]) {
#pragma unroll
  for (int q = 0; q < kSlots; ++q) {
    if (q < ns) {
      const uint32_t tq = b + q, pq = at[q];
      if (pq != tq) {
        const uint32_t i0 = v.sorted_idx[tq], i1 = v.sorted_idx[pq];
        const float2 p0 = v.sorted_pos[tq], p1 = v.sorted_pos[pq];
        v.sorted_idx[tq] = i1; v.sorted_pos[tq] = p1;
        v.sorted_idx[pq] = i0; v.sorted_pos[pq] = p0;
#pragma unroll
        for (int r = q + 1; r < kSlots; ++r)
          if (at[r] == tq) at[r] = pq;
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock) kb_bigcells(BatchView v) {
  __shared__ unsigned long long skey[kBlock * kSlots];
  __shared__ uint32_t spos[kBlock * kSlots];
  __shared__ unsigned long long wmin[kBlock / 32];
  __shared__ uint32_t wpos[kBlock / 32];
  __shared__ long long rx[kBlock / 32], ry[kBlock / 32];
  __shared__ unsigned long long sel_key;
  __shared__ uint32_t sel_at[kSlots];
  __shared__ int sel_n;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nbig = v.big_count[0];
  for (uint32_t wi = blockIdx.x; wi < nbig; wi += gridDim.x) {
    const uint32_t c = v.big_list[wi];
    const uint32_t g = v.cell_gid[c];
    const GraphDesc& D = v.desc[g];
    const uint32_t seed = tick_of(v, g).seed_bits;
    const uint32_t b = v.cell_start[c], e = v.cell_start[c + 1];
    long long ax = 0, ay = 0;
    unsigned long long best[kSlots];
    uint32_t at[kSlots];
#pragma unroll
    for (int q = 0; q < kSlots; ++q) { best[q] = ~0ull; at[q] = 0; }
    for (uint32_t j = b + threadIdx.x; j < e; j += blockDim.x) {
      const float2 p = v.sorted_pos[j];
      ax += to_fixed(p.x, D.fx);
      ay += to_fixed(p.y, D.fx);
      top8_insert(best, at, local_key(v.sorted_idx[j], D.p_off, seed), j);
    }
#pragma unroll
    for (int q = 0; q < kSlots; ++q) { skey[threadIdx.x * kSlots + q] = best[q]; spos[threadIdx.x * kSlots + q] = at[q]; }
    ax = warp_sum_ll(ax);
    ay = warp_sum_ll(ay);
    if (lane == 0) { rx[w] = ax; ry[w] = ay; }
    if (threadIdx.x == 0) sel_n = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long tx = 0, ty = 0;
      for (int k = 0; k < kBlock / 32; ++k) { tx += rx[k]; ty += ry[k]; }
      v.big_sx[c] = tx;
      v.big_sy[c] = ty;
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
      kb_move_head(v, b, ns, pat);
      v.big_ns[c] = (uint32_t)ns;
    }
    __syncthreads();
  }
  // warp cells (warp_cells.cuh), one warp each, the heavy ones (above
  // kWarpSmallCell points) first, so the longest start first
  __shared__ uint32_t cand[kBlock / 32][3][kCandidates];
  const uint32_t nheavy = v.big_count[1], nwarp = nheavy + v.big_count[2];
  const uint32_t n = v.cell_hwm;
  // the first cell by warp id, the next ones from the ticket
  const uint32_t nw_grid = gridDim.x * (blockDim.x >> 5);
  for (uint32_t wi = blockIdx.x * (blockDim.x >> 5) + w; wi < nwarp;) {
    const uint32_t c = wi < nheavy ? v.big_list[n + wi] : v.big_list[2 * n - 1 - (wi - nheavy)];
    const uint32_t g = v.cell_gid[c];
    const GraphDesc& D = v.desc[g];
    warp_cell(v, D.fx, tick_of(v, g).seed_bits, D.p_off, c, cand[w]);
    if (lane == 0) wi = nw_grid + atomicAdd(&v.big_count[3], 1u);
    wi = __shfl_sync(0xffffffffu, wi, 0);
  }
}

// One finest cell: its exact sums (from kb_bigcells for a dense cell, else
// from its points), its near-field slots moved to the head of its segment
// [b, e) (build-nearfield-slots.vert), its record (calculate-level.vert).
__device__ __forceinline__ void kb_finest_cell(const BatchView& v, const GraphDesc& D, uint32_t seed, uint32_t c,
                                               uint32_t lc, uint32_t b, uint32_t e, long long& ax, long long& ay) {
  ax = 0;
  ay = 0;
  int ns = 0;
  if (e - b > kSmallCell) {
    ax = v.big_sx[c];
    ay = v.big_sy[c];
    ns = (int)v.big_ns[c];
  } else if (e > b) {
    unsigned long long best[kSlots];
    uint32_t at[kSlots];
#pragma unroll
    for (int q = 0; q < kSlots; ++q) { best[q] = ~0ull; at[q] = 0; }
    for (uint32_t j = b; j < e; ++j) {
      const float2 p = v.sorted_pos[j];
      ax += to_fixed(p.x, D.fx);
      ay += to_fixed(p.y, D.fx);
      top8_insert(best, at, local_key(v.sorted_idx[j], D.p_off, seed), j);
    }
#pragma unroll
    for (int q = 0; q < kSlots; ++q) ns += best[q] != ~0ull;
    kb_move_head(v, b, ns, at);
  }
  float4 r = make_float4(0.f, 0.f, 0.f, (float)ns);
  if (e > b) {
    const float cf = (float)(e - b);
    r.x = __fdiv_rn(from_fixed(ax, D.fx), cf);
    r.y = __fdiv_rn(from_fixed(ay, D.fx), cf);
    r.z = cf;
  }
  v.rec[D.rec_off + level_base(D.levels - 1) + lc] = r;
}

__device__ __forceinline__ float4 level_record(long long sx, long long sy, long long n, const FixedScale& fx) {
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if (n > 0) {
    const float cf = (float)n;
    r.x = __fdiv_rn(from_fixed(sx, fx), cf);
    r.y = __fdiv_rn(from_fixed(sy, fx), cf);
    r.z = cf;
  }
  return r;
}

// The many-body pass's work items of one parent cell: its points are the
// sorted positions [a0, a2) (the upper two children) then [b0, b2) (the lower
// two), taken two at a time in that order, the last alone when their number
// is odd.  Items are appended with one atomic per warp.  Called by all 32
// lanes of the warp (lanes without a parent cell pass empty ranges).
__device__ __forceinline__ void sib_items(const BatchView& v, uint32_t a0, uint32_t a2, uint32_t b0, uint32_t b2) {
  const uint32_t n0 = a2 - a0, n = n0 + (b2 - b0);
  const uint32_t items = (n + 1) >> 1;
  const int lane = threadIdx.x & 31;
  uint32_t incl = items;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  uint32_t base = 0;
  if (lane == 31 && incl) base = atomicAdd(&v.big_count[kBatchSibs], incl);
  base = __shfl_sync(0xffffffffu, base, 31) + incl - items;
  for (uint32_t t = 0; t < items; ++t) {
    const uint32_t i0 = 2 * t, i1 = i0 + 1;
    const uint32_t jA = i0 < n0 ? a0 + i0 : b0 + (i0 - n0);
    const uint32_t jB = i1 >= n ? kNoPoint : i1 < n0 ? a0 + i1 : b0 + (i1 - n0);
    v.sib_list[base + t] = make_uint2(jA, jB);
  }
}

// One CTA per (graph, tile) of the work list.  A tile is T x T finest cells
// (T = GraphDesc::tile <= 32); each thread takes a 2 x 2 quad of them, whose
// sums make one cell of the next level in registers; the levels above, inside
// the tile, by shared-memory reduction; coarser levels by integer atomics
// finished in kb_coarse.  A quad's four cell starts are six loads issued
// together, so a sparse graph's mostly empty cells cost little beyond them.
__global__ void __launch_bounds__(kBlock) kb_cells(BatchView v) {
  __shared__ long long smx[kBlock], smy[kBlock], smn[kBlock];
  const uint2 wk = v.tiles[blockIdx.x];
  const uint32_t g = wk.x;
  const GraphDesc& D = v.desc[g];
  const BatchTick tp = tick_of(v, g);
  if (!tp.active || !(D.stages & kGManybody)) return;
  const int T = D.tile, Q = T >> 1, gf = D.gf, L = D.levels;
  const int tiles_row = gf / T;
  const int tile_x = (int)wk.y % tiles_row, tile_y = (int)wk.y / tiles_row;
  const bool live = (int)threadIdx.x < Q * Q;
  const int qx = (int)threadIdx.x % Q, qy = (int)threadIdx.x / Q;
  long long sx = 0, sy = 0, sn = 0;
  uint32_t a0 = 0, a2 = 0, b0 = 0, b2 = 0;   // the quad's points: [a0, a2) and [b0, b2)
  if (live) {
    const int cx = tile_x * T + 2 * qx, cy = tile_y * T + 2 * qy;
    const uint32_t l0 = (uint32_t)(cy * gf + cx), l1 = l0 + (uint32_t)gf;
    const uint32_t c0 = D.cell_off + l0, c1 = D.cell_off + l1;
    a0 = v.cell_start[c0];
    const uint32_t a1 = v.cell_start[c0 + 1];
    a2 = v.cell_start[c0 + 2];
    b0 = v.cell_start[c1];
    const uint32_t b1 = v.cell_start[c1 + 1];
    b2 = v.cell_start[c1 + 2];
    long long x, y;
    kb_finest_cell(v, D, tp.seed_bits, c0, l0, a0, a1, x, y);
    sx += x; sy += y;
    kb_finest_cell(v, D, tp.seed_bits, c0 + 1, l0 + 1, a1, a2, x, y);
    sx += x; sy += y;
    kb_finest_cell(v, D, tp.seed_bits, c1, l1, b0, b1, x, y);
    sx += x; sy += y;
    kb_finest_cell(v, D, tp.seed_bits, c1 + 1, l1 + 1, b1, b2, x, y);
    sx += x; sy += y;
    sn = (long long)(a2 - a0) + (long long)(b2 - b0);
    const int G = gf >> 1;   // level L - 2
    v.rec[D.rec_off + level_base(L - 2) + (tile_y * Q + qy) * G + tile_x * Q + qx] = level_record(sx, sy, sn, D.fx);
  }
  sib_items(v, a0, a2, b0, b2);   // every lane of the warp (empty ranges outside the tile)
  smx[threadIdx.x] = sx; smy[threadIdx.x] = sy; smn[threadIdx.x] = sn;
  __syncthreads();
  int gsz = Q;
  int lv = L - 2;
  while (gsz > 1 && lv > 0) {
    gsz >>= 1;
    --lv;
    long long vx = 0, vy = 0, vn = 0;
    const bool active = live && qx < gsz && qy < gsz;
    if (active) {
      const int i00 = (2 * qy) * Q + 2 * qx;
      vx = smx[i00] + smx[i00 + 1] + smx[i00 + Q] + smx[i00 + Q + 1];
      vy = smy[i00] + smy[i00 + 1] + smy[i00 + Q] + smy[i00 + Q + 1];
      vn = smn[i00] + smn[i00 + 1] + smn[i00 + Q] + smn[i00 + Q + 1];
    }
    __syncthreads();
    if (active) {
      smx[qy * Q + qx] = vx; smy[qy * Q + qx] = vy; smn[qy * Q + qx] = vn;
      const int G = 4 << lv;
      v.rec[D.rec_off + level_base(lv) + (tile_y * gsz + qy) * G + tile_x * gsz + qx] = level_record(vx, vy, vn, D.fx);
    }
    __syncthreads();
  }
  if (lv == 0 || threadIdx.x != 0) return;
  const long long tx_ = smx[0], ty_ = smy[0], tn_ = smn[0];
  for (int l = lv - 1; l >= 0; --l) {
    const int sh = lv - l;
    const int G = 4 << l;
    long long* a = v.acc + 3 * (size_t)(D.acc_off + level_base(l) + (tile_y >> sh) * G + (tile_x >> sh));
    atomicAdd((unsigned long long*)&a[0], (unsigned long long)tx_);
    atomicAdd((unsigned long long*)&a[1], (unsigned long long)ty_);
    atomicAdd((unsigned long long*)&a[2], (unsigned long long)tn_);
  }
}

// Levels coarser than the tile: one CTA per graph converts and re-zeroes.
__global__ void __launch_bounds__(kBlock) kb_coarse(BatchView v) {
  const uint32_t g = blockIdx.x;
  const GraphDesc& D = v.desc[g];
  if (D.n == 0 || D.acc_cells == 0) return;
  if (!tick_of(v, g).active || !(D.stages & kGManybody)) return;
  for (uint32_t k = threadIdx.x; k < D.acc_cells; k += blockDim.x) {
    long long* a = v.acc + 3 * (size_t)(D.acc_off + k);
    const long long vx = a[0], vy = a[1], vn = a[2];
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (vn > 0) {
      const float cf = (float)vn;
      r.x = __fdiv_rn(from_fixed(vx, D.fx), cf);
      r.y = __fdiv_rn(from_fixed(vy, D.fx), cf);
      r.z = cf;
    }
    v.rec[D.rec_off + k] = r;   // coarse levels come first in both layouts
    a[0] = 0; a[1] = 0; a[2] = 0;
  }
}

// --------------------------------------------------------------- manybody --
// The near field (force-nearfield.frag:199-263) of the point at sorted
// position j, added to its level velocity, and the update.
template <bool FAST>
__device__ __forceinline__ void kb_finish_point(const BatchView& v, const GraphDesc& D, uint32_t j, uint32_t P, float2 p,
                                                int fcx, int fcy, float2 vel, float k) {
  const PairUnits pu = v.units;
  const float4* fine = v.rec + D.rec_off + level_base(D.levels - 1);
  const float2 rj = v.jitter[P];
  float2 nf = near_terms<FAST>(fine, v.cell_start + D.cell_off, v.sorted_pos, D.gf, fcx, fcy, j, p, rj, k, pu);
  nf = add2(nf, mul2(nf, rj, pu), pu);
  const float max_step = __fmul_rn(2.0f, D.csf);
  const float2 nsq = mul2(nf, nf, pu);
  const float speed = __fsqrt_rn(__fadd_rn(nsq.x, nsq.y));
  if (speed > max_step) nf = mul2(nf, splat(__fdiv_rn(max_step, speed)), pu);
  vel = add2(vel, nf, pu);
  if (!(v.flags[P] & kPinned)) v.pos[P] = integrate(p, vel.x, vel.y, D.friction, D.space);
}

// One point (force-level.frag:70-95 for every level, then the near field).
// FAST: the repulsion quotients come from the reciprocals (quotient_by_recip(k)).
// GUARDED: the level terms without the range flag (the job's level_guard and
// no binned point of the batch outside its space this tick).
template <bool FAST, bool GUARDED = false>
__device__ __forceinline__ void kb_manybody_point(const BatchView& v, const GraphDesc& D, uint32_t j, uint32_t P,
                                                  float2 p, float k) {
  const int gf = D.gf, L = D.levels;
  const int fcx = cell_index(p.x, D.csf, gf), fcy = cell_index(p.y, D.csf, gf);
  const PairUnits pu = v.units;
  const float4* rec = v.rec + D.rec_off;
  float2 vel = make_float2(0.f, 0.f);
#pragma unroll 1
  for (int l = 0; l < L; ++l) {
    const int sh = L - 1 - l;
    vel = add2(vel, level_terms<FAST, FAST, GUARDED>(rec + level_base(l), 4 << l, fcx >> sh, fcy >> sh, p, k, pu), pu);
  }
  kb_finish_point<FAST>(v, D, j, P, p, fcx, fcy, vel, k);
}

// Two points of one parent cell (sorted positions jA, jB; the same finest
// cell or sibling cells) on f32x2 lanes (manybody_duo.cuh): the levels above
// the finest are the same cells for both, the finest level is one walk over
// the shared 6x6 block that each point takes outside its own 3x3
// (level_terms_duo_sibs); each lane is the one-point chain, in its order, so
// each result is bit for bit kb_manybody_point's.  A level with a length
// outside the in-range sequences is summed again per point with the tested
// terms; the near fields are per point.  `single`: jA alone.
template <bool GUARD>
__device__ __forceinline__ void kb_manybody_sibs(const BatchView& v, const GraphDesc& D, uint32_t jA, uint32_t jB,
                                                 bool single, float k) {
  const uint32_t PA = v.sorted_idx[jA], PB = v.sorted_idx[jB];
  const float2 pA = v.sorted_pos[jA], pB = v.sorted_pos[jB];
  const int gf = D.gf, L = D.levels;
  const int ax = cell_index(pA.x, D.csf, gf), ay = cell_index(pA.y, D.csf, gf);
  const int bx = cell_index(pB.x, D.csf, gf), by = cell_index(pB.y, D.csf, gf);
  const PairUnits pu = v.units;
  const float4* rec = v.rec + D.rec_off;
  const Duo P = {make_float2(pA.x, pB.x), make_float2(pA.y, pB.y)};
  Duo vel = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll 1
  for (int l = 0; l < L; ++l) {
    const int sh = L - 1 - l;
    const float4* lv = rec + level_base(l);
    const int G = 4 << l;
    bool out = false;
    Duo w = sh ? level_terms_duo<!GUARD>(lv, G, ax >> sh, ay >> sh, P, k, pu, out)
               : level_terms_duo_sibs<!GUARD>(lv, G, ax, ay, bx, by, P, k, pu, out);
    if (!GUARD && out) {   // a length outside the sequences: each point's level with the tested terms
      const float2 a = level_terms<true, false>(lv, G, ax >> sh, ay >> sh, pA, k, pu);
      const float2 b = level_terms<true, false>(lv, G, bx >> sh, by >> sh, pB, k, pu);
      w.x = make_float2(a.x, b.x);
      w.y = make_float2(a.y, b.y);
    }
    vel.x = add2(vel.x, w.x, pu);
    vel.y = add2(vel.y, w.y, pu);
  }
  kb_finish_point<true>(v, D, jA, PA, pA, ax, ay, make_float2(vel.x.x, vel.y.x), k);
  if (!single) kb_finish_point<true>(v, D, jB, PB, pB, bx, by, make_float2(vel.x.y, vel.y.y), k);
}

// One work item per thread: up to two points of one parent cell (sib_list,
// written by kb_cells; big_count[kBatchSibs] items this tick).  Four blocks
// per SM, as the plain engine's two-point pass.
__global__ void __launch_bounds__(kBlock, 4) kb_manybody(BatchView v) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= __ldg(&v.big_count[kBatchSibs])) return;
  const uint2 it = v.sib_list[w];
  const bool single = it.y == kNoPoint;
  const uint32_t jA = it.x, jB = single ? it.x : it.y;
  const uint32_t PA = v.sorted_idx[jA];
  const uint32_t g = v.gid[PA];
  const GraphDesc& D = v.desc[g];
  const BatchTick tp = tick_of(v, g);
  const float k = __fmul_rn(tp.alpha, D.repulsion);
  if (!quotient_by_recip(k)) {   // quotients outside the reciprocal method's range: one point at a time
    kb_manybody_point<false>(v, D, jA, PA, v.sorted_pos[jA], k);
    if (!single) kb_manybody_point<false>(v, D, jB, v.sorted_idx[jB], v.sorted_pos[jB], k);
  } else if (D.level_guard && __ldg(&v.big_count[kBatchOutside]) == 0) {
    kb_manybody_sibs<true>(v, D, jA, jB, single, k);
  } else {
    kb_manybody_sibs<false>(v, D, jA, jB, single, k);
  }
}

// ------------------------------------------------------------------- link --
// ForceLink.run (ForceLink/index.ts:221-263), force-spring.ts:38-96, as
// k_link: one list per thread, springs strictly in list order.  Graphs that
// do not run this pass (no links, masked, or inactive) copy their positions
// through, so the ping-pong buffers stay consistent.
struct LinkScalars {
  float sa, span, r0, dist;
};

__device__ __forceinline__ LinkScalars link_scalars(const GraphDesc& D, const BatchTick& tp) {
  return LinkScalars{__fmul_rn(D.link_spring, tp.alpha), __fsub_rn(D.link_r1, D.link_r0), D.link_r0, D.link_distance};
}

__device__ __forceinline__ void batch_spring(const LinkScalars& ls, const uint4 en, const float2 pp, const float2 q,
                                             float2& vel, const PairUnits& pu) {
  float dd = __fadd_rn(__fmul_rn(__uint_as_float(en.y), ls.span), ls.r0);
  dd = __fmul_rn(dd, ls.dist);
  spring_step(pp, vel, q, dd, __fmul_rn(dd, 0.99f), ls.sa, __uint_as_float(en.w), __uint_as_float(en.z), pu);
}

// The long lists (more than kHeavyDegree links): rows[t] is an arena point.
__global__ void __launch_bounds__(kBlock) kb_link_heavy(BatchView v, int direction, const float2* __restrict__ src,
                                                        float2* __restrict__ dst, const uint32_t* __restrict__ rows,
                                                        uint32_t nrows) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const uint32_t P = rows[t];
  const uint32_t g = v.gid[P];
  if (g == kNoGraph) return;
  const GraphDesc& D = v.desc[g];
  const BatchTick tp = tick_of(v, g);
  const float2 pp = src[P];
  const uint32_t stage = direction == 0 ? kGLinkIn : kGLinkOut;
  const uint8_t f = v.flags[P];
  if (!tp.active || !(D.stages & stage) || (f & kAbsent)) { dst[P] = pp; return; }
  const uint32_t rp = (direction == 0 ? D.rp_in : D.rp_out) + (P - D.p_off);
  const uint4* ent = v.ent + (direction == 0 ? D.e_in : D.e_out);
  const uint32_t e0 = v.rowptr[rp], e1 = v.rowptr[rp + 1];
  const float2* gsrc = src + D.p_off;
  const LinkScalars ls = link_scalars(D, tp);
  const PairUnits pu = v.units;
  float2 vel = make_float2(0.f, 0.f);
  constexpr int kLinkBatch = 4;
  uint32_t at = e0;
  for (; at + kLinkBatch <= e1; at += kLinkBatch) {
    uint4 en[kLinkBatch];
    float2 q[kLinkBatch];
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) en[u] = __ldg(&ent[at + u]);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) q[u] = en[u].x != kAbsentTarget ? __ldg(&gsrc[en[u].x]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u)
      if (en[u].x != kAbsentTarget) batch_spring(ls, en[u], pp, q[u], vel, pu);
  }
  for (; at < e1; ++at) {
    const uint4 en = __ldg(&ent[at]);
    if (en.x == kAbsentTarget) continue;
    batch_spring(ls, en, pp, __ldg(&gsrc[en.x]), vel, pu);
  }
  dst[P] = (f & kPinned) ? pp : integrate(pp, vel.x, vel.y, D.friction, D.space);
}

// The light rows by warps (GraphDesc::lr, lw, ln, nw): a block takes
// kLinkWarpsPerBlock warps of one graph from the work list; a warp's lanes walk
// lists of nearly the same length, and entry k of all 32 lists is one
// coalesced 512-byte load.
// Five blocks per SM (48 registers, a few bytes of spills): 272 -> 259 us a
// pass against four (56 registers) on 512 jobs.
__global__ void __launch_bounds__(kBlock, 5) kb_link_warps(BatchView v, int direction, const float2* __restrict__ src,
                                                        float2* __restrict__ dst) {
  const uint2 wk = v.lwork[direction][blockIdx.x];
  const uint32_t g = wk.x;
  const GraphDesc& D = v.desc[g];
  const uint32_t w = wk.y + (threadIdx.x >> 5);
  if (w >= D.nw[direction]) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t i = __ldg(&v.lrow[D.lr[direction] + 32 * w + lane]);
  if (i == kNoPoint) return;
  const uint32_t P = D.p_off + i;
  const BatchTick tp = tick_of(v, g);
  const float2 pp = src[P];
  const uint32_t stage = direction == 0 ? kGLinkIn : kGLinkOut;
  const uint8_t f = v.flags[P];
  if (!tp.active || !(D.stages & stage) || (f & kAbsent)) { dst[P] = pp; return; }
  const uint32_t* wo = v.lwoff + D.lw[direction] + w;
  const uint32_t o0 = __ldg(&wo[0]), cnt = (__ldg(&wo[1]) - o0) >> 5;
  const uint4* col = v.lanes + D.ln[direction] + o0 + lane;
  const float2* gsrc = src + D.p_off;
  const LinkScalars ls = link_scalars(D, tp);
  const PairUnits pu = v.units;
  float2 vel = make_float2(0.f, 0.f);
  constexpr int kLinkBatch = 4;
  uint32_t at = 0;
  for (; at + kLinkBatch <= cnt; at += kLinkBatch) {
    uint4 en[kLinkBatch];
    float2 q[kLinkBatch];
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) en[u] = __ldg(&col[32 * (at + u)]);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) q[u] = en[u].x != kAbsentTarget ? __ldg(&gsrc[en[u].x]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u)
      if (en[u].x != kAbsentTarget) batch_spring(ls, en[u], pp, q[u], vel, pu);
  }
  for (; at < cnt; ++at) {
    const uint4 en = __ldg(&col[32 * at]);
    if (en.x == kAbsentTarget) continue;
    batch_spring(ls, en, pp, __ldg(&gsrc[en.x]), vel, pu);
  }
  dst[P] = (f & kPinned) ? pp : integrate(pp, vel.x, vel.y, D.friction, D.space);
}

__global__ void __launch_bounds__(kBlock) kb_warp_lengths(const uint32_t* __restrict__ order,
                                                          const uint32_t* __restrict__ len, uint32_t nh, uint32_t n,
                                                          uint32_t* __restrict__ woff) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nw = (n - nh + 31) / 32;
  if (w > nw) return;
  woff[w] = w < nw ? 32 * len[order[nh + 32 * w]] : 0u;   // a warp's first row has its longest list
}

__global__ void __launch_bounds__(kBlock) kb_warp_rows(const uint32_t* __restrict__ order, uint32_t nh, uint32_t n,
                                                       uint32_t* __restrict__ lrow) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nw = (n - nh + 31) / 32;
  if (t >= 32 * nw) return;
  lrow[t] = t < n - nh ? order[nh + t] : kNoPoint;
}

// -------------------------------------------------------------- collision --
// ForceCollision.run per graph (collision.cuh's arithmetic, the plain
// engine's): grid sums of the four offset grids, their conversion, the force.
__global__ void __launch_bounds__(kBlock) kb_coll_grid(BatchView v) {
  const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
  bool live = false;
  const GraphDesc* D = nullptr;
  float2 p = make_float2(0.f, 0.f);
  float sz = 0.f;
  if (P < v.point_hwm) {
    const uint32_t g = v.gid[P];
    if (g != kNoGraph) {
      D = &v.desc[g];
      live = (D->stages & kGCollision) && tick_of(v, g).active && !(v.flags[P] & kAbsent);
      if (live) { p = v.pos[P]; sz = v.size[P]; }
    }
  }
  if (!__any_sync(0xffffffffu, live)) return;   // warp-uniform
  const FixedScale none{1.f, 1.f, 1.f};
  coll_accumulate(live ? v.cgrid_acc + 4 * (size_t)D->coll_off : v.cgrid_acc, live ? D->coll_grid : 1,
                  live ? D->coll_cell : 1.f, live ? D->fx : none, p, sz, live);
}

__global__ void __launch_bounds__(kBlock) kb_coll_convert(BatchView v) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= v.coll_hwm) return;
  const uint32_t g = v.coll_gid[c];
  if (g == kNoGraph) return;
  coll_convert_cell(v.cgrid_acc + 4 * (size_t)c, v.cgrid + c, v.desc[g].fx);
}

__global__ void __launch_bounds__(kBlock) kb_coll_force(BatchView v) {
  const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
  if (P >= v.point_hwm) return;
  const uint32_t g = v.gid[P];
  if (g == kNoGraph) return;
  const GraphDesc& D = v.desc[g];
  if (!(D.stages & kGCollision)) return;
  const BatchTick tp = tick_of(v, g);
  if (!tp.active) return;
  const uint8_t f = v.flags[P];
  if (f & kAbsent) return;
  const float2 p = v.pos[P];
  const CollParams cp{D.coll_grid, D.coll_cell, D.coll_radius, D.coll_padding, __fmul_rn(tp.alpha, D.coll_strength)};
  const float2 w = coll_velocity(v.cgrid + D.coll_off, cp, p, v.size[P], P - D.p_off, D.n);
  if (!(f & kPinned)) v.pos[P] = integrate(p, w.x, w.y, D.friction, D.space);
}

__global__ void kb_tick_end(BatchView v) { *v.tick_ctr += 1; }

inline uint32_t blocks(uint32_t n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

void batch_launch_tick(const BatchView& v, cudaStream_t st, cudaStream_t side, cudaEvent_t* fork, cudaEvent_t* join) {
  cudaMemsetAsync(v.big_count, 0, 8 * sizeof(uint32_t), st);
  if (v.any_center) cudaMemsetAsync(v.centroid, 0, 3 * sizeof(long long) * (size_t)v.slots, st);
  if (v.point_hwm) kb_prepass<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  if (v.any_center && v.point_hwm) kb_center<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  if (v.cell_hwm) kb_scan<<<batch_scan_blocks(v.cell_hwm), kBlock, 0, st>>>(v);
  if (v.point_hwm) kb_scatter<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  kb_bigcells<<<8 * sm_count(), kBlock, 0, st>>>(v);   // as k_bigcells: 8 blocks per SM
  if (v.n_tiles) kb_cells<<<v.n_tiles, kBlock, 0, st>>>(v);
  if (v.slots) kb_coarse<<<v.slots, kBlock, 0, st>>>(v);
  if (v.point_hwm) kb_manybody<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);   // items <= points
  for (int dir = 0; dir < 2; ++dir) {
    const float2* src = dir == 0 ? v.pos : v.pos_alt;
    float2* dst = dir == 0 ? v.pos_alt : v.pos;
    const uint32_t* heavy = dir == 0 ? v.heavy_in : v.heavy_out;
    const uint32_t nh = dir == 0 ? v.n_heavy_in : v.n_heavy_out;
    if (nh) {
      cudaEventRecord(fork[dir], st);
      cudaStreamWaitEvent(side, fork[dir], 0);
      kb_link_heavy<<<blocks(nh), kBlock, 0, side>>>(v, dir, src, dst, heavy, nh);
      cudaEventRecord(join[dir], side);
    }
    if (v.n_lwork[dir]) kb_link_warps<<<v.n_lwork[dir], kBlock, 0, st>>>(v, dir, src, dst);
    if (nh) cudaStreamWaitEvent(st, join[dir], 0);
  }
  if (v.any_collision && v.point_hwm) {   // after the links, as in runSimulationStep (src/index.ts:2068-2078)
    kb_coll_grid<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
    if (v.coll_hwm) kb_coll_convert<<<blocks(v.coll_hwm), kBlock, 0, st>>>(v);
    kb_coll_force<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  }
  kb_tick_end<<<1, 1, 0, st>>>(v);
}

uint32_t batch_scan_blocks(uint32_t cells) { return (cells + kChunk - 1) / kChunk; }

void batch_warp_lengths(const uint32_t* order, const uint32_t* len, uint32_t nh, uint32_t n, uint32_t* woff,
                        cudaStream_t st) {
  const uint32_t nw = (n - nh + 31) / 32;
  kb_warp_lengths<<<blocks(nw + 1), kBlock, 0, st>>>(order, len, nh, n, woff);
}

void batch_warp_rows(const uint32_t* order, uint32_t nh, uint32_t n, uint32_t* lrow, cudaStream_t st) {
  const uint32_t nw = (n - nh + 31) / 32;
  if (nw) kb_warp_rows<<<blocks(32 * nw), kBlock, 0, st>>>(order, nh, n, lrow);
}

uint32_t batch_kernels_per_tick(const BatchView& v) {
  uint32_t k = 1 + 1 + 1 + 1 + 1;       // prepass, scatter, big cells, coarse, manybody
  k += (v.n_lwork[0] > 0) + (v.n_lwork[1] > 0);
  if (v.cell_hwm) k += 1;
  if (v.n_tiles) k += 1;
  k += (v.n_heavy_in > 0) + (v.n_heavy_out > 0);
  if (v.any_center) k += 1;
  if (v.any_collision) k += 2 + (v.coll_hwm > 0);
  return k + 1;                          // tick end
}

}  // namespace cgl
