// batch_kernels.cu — one tick of many graphs at once.
//
// The per-graph arithmetic is the plain engine's (kernels.cu), operation for
// operation; only the addressing differs: each point or cell finds its graph
// (gid / cell_gid), its graph's descriptor and its graph's tick parameters.
// Point indices that enter the arithmetic (peel hash, tie-break, self test)
// are graph-local, so a graph advances exactly as it would alone.
#include "batch.cuh"
#include "collision.cuh"
#include "device_util.cuh"
#include "warp_cells.cuh"

namespace cgl {
namespace {

constexpr int kChunk = 1024;   // scan: cells per block (kBlock threads x 4)

__device__ __forceinline__ const BatchTick& tick_of(const BatchView& v, uint32_t g) {
  return v.ticks[(size_t)(*v.tick_ctr) * v.slots + g];
}

__device__ __forceinline__ uint32_t level_base(int l) {
  // sum over m < l of (4 << m)^2 = 16 (4^l - 1) / 3
  return (uint32_t)(16u * (((1u << (2 * l)) - 1u) / 3u));
}

// ---------------------------------------------------------------- prepass --
constexpr uint32_t kBatchOutside = 4;   // big_count word: a binned point outside its space

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
// Three-level exclusive scan of the cell histogram over the used cell arena.
__global__ void __launch_bounds__(kBlock) kb_scan_reduce(const uint32_t* in, uint32_t n, uint32_t* out) {
  const uint32_t base = blockIdx.x * kChunk;
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t c = base + k * kBlock + threadIdx.x;
    if (c < n) sum += in[c];
  }
  uint32_t total;
  block_exclusive_scan(sum, &total);
  if (threadIdx.x == 0) out[blockIdx.x] = total;
}

// Exclusive scan of `n` values in chunks of kChunk, plus the chunk offsets
// `off` (nullptr: none); the grand total goes to total_out when non-null.
__global__ void __launch_bounds__(kBlock) kb_scan_down(uint32_t* vals, uint32_t n, const uint32_t* off,
                                                       uint32_t* out, uint32_t* total_out) {
  const uint32_t base = blockIdx.x * kChunk + threadIdx.x * 4;
  uint32_t x[4];
  uint32_t run = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    x[k] = base + k < n ? vals[base + k] : 0;
    run += x[k];
  }
  uint32_t total;
  uint32_t o = block_exclusive_scan(run, &total) + (off ? off[blockIdx.x] : 0);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < n) out[base + k] = o;
    o += x[k];
  }
  if (total_out && threadIdx.x == 0) *total_out = total;
}

// Last level: cell starts, histogram zeroed, dense cells listed.
__global__ void __launch_bounds__(kBlock) kb_scan_cells(BatchView v, const uint32_t* off) {
  const uint32_t n = v.cell_hwm;
  const uint32_t base = blockIdx.x * kChunk + threadIdx.x * 4;
  uint32_t x[4];
  uint32_t run = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    x[k] = base + k < n ? v.counts[base + k] : 0;
    run += x[k];
  }
  uint32_t total;
  uint32_t o = block_exclusive_scan(run, &total) + off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t c = base + k;
    if (c < n) {
      v.cell_start[c] = o;
      v.counts[c] = 0;
      if (x[k] > kBigCell) v.big_list[atomicAdd(&v.big_count[0], 1u)] = c;
      else if (x[k] > kWarpSmallCell) v.big_list[n + atomicAdd(&v.big_count[1], 1u)] = c;
      else if (x[k] > kSmallCell) v.big_list[2 * n - 1 - atomicAdd(&v.big_count[2], 1u)] = c;
    }
    o += x[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == kBlock - 1) v.cell_start[n] = o;
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

// One CTA per (graph, tile) of the work list; thread per finest cell of the
// tile; levels inside the tile by shared-memory reduction, coarser levels by
// integer atomics finished in kb_coarse.
__global__ void __launch_bounds__(kBlock) kb_cells(BatchView v) {
  __shared__ long long smx[kBlock], smy[kBlock], smn[kBlock];
  const uint2 wk = v.tiles[blockIdx.x];
  const uint32_t g = wk.x;
  const GraphDesc& D = v.desc[g];
  const BatchTick tp = tick_of(v, g);
  if (!tp.active || !(D.stages & kGManybody)) return;
  const int T = D.tile;
  const int tiles_row = D.gf / T;
  const int tile_x = (int)wk.y % tiles_row, tile_y = (int)wk.y / tiles_row;
  const bool live = (int)threadIdx.x < T * T;
  const int tx = (int)threadIdx.x % T, ty = (int)threadIdx.x / T;
  const int cx = tile_x * T + tx, cy = tile_y * T + ty;
  const uint32_t lc = (uint32_t)(cy * D.gf + cx);
  const uint32_t c = D.cell_off + lc;
  long long ax = 0, ay = 0, cnt = 0;
  if (live) {
    const uint32_t b = v.cell_start[c], e = v.cell_start[c + 1];
    cnt = e - b;
    int ns = 0;
    if (e - b > kSmallCell) {
      ax = v.big_sx[c];
      ay = v.big_sy[c];
      ns = (int)v.big_ns[c];
    } else {
      unsigned long long best[kSlots];
      uint32_t at[kSlots];
#pragma unroll
      for (int q = 0; q < kSlots; ++q) { best[q] = ~0ull; at[q] = 0; }
      for (uint32_t j = b; j < e; ++j) {
        const float2 p = v.sorted_pos[j];
        ax += to_fixed(p.x, D.fx);
        ay += to_fixed(p.y, D.fx);
        top8_insert(best, at, local_key(v.sorted_idx[j], D.p_off, tp.seed_bits), j);
      }
#pragma unroll
      for (int q = 0; q < kSlots; ++q) ns += best[q] != ~0ull;
      kb_move_head(v, b, ns, at);
    }
    float4 r = make_float4(0.f, 0.f, 0.f, (float)ns);
    if (cnt > 0) {
      const float cf = (float)cnt;
      r.x = __fdiv_rn(from_fixed(ax, D.fx), cf);
      r.y = __fdiv_rn(from_fixed(ay, D.fx), cf);
      r.z = cf;
    }
    v.rec[D.rec_off + level_base(D.levels - 1) + lc] = r;
  }
  smx[threadIdx.x] = ax; smy[threadIdx.x] = ay; smn[threadIdx.x] = cnt;
  __syncthreads();
  int gsz = T;
  int lv = D.levels - 1;
  while (gsz > 1 && lv > 0) {
    gsz >>= 1;
    --lv;
    long long vx = 0, vy = 0, vn = 0;
    const bool active = live && tx < gsz && ty < gsz;
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
      const int gx = tile_x * gsz + tx, gy = tile_y * gsz + ty;
      float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
      if (vn > 0) {
        const float cf = (float)vn;
        r.x = __fdiv_rn(from_fixed(vx, D.fx), cf);
        r.y = __fdiv_rn(from_fixed(vy, D.fx), cf);
        r.z = cf;
      }
      v.rec[D.rec_off + level_base(lv) + gy * G + gx] = r;
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
  for (int l = 0; l < L; ++l) {   // force-level.frag:70-95
    const int sh = L - 1 - l;
    vel = add2(vel, level_terms<FAST, FAST, GUARDED>(rec + level_base(l), 4 << l, fcx >> sh, fcy >> sh, p, k, pu), pu);
  }
  // near field (force-nearfield.frag:199-263)
  const float2 rj = v.jitter[P];
  float2 nf = near_terms<FAST>(rec + level_base(L - 1), v.cell_start + D.cell_off, v.sorted_pos, gf, fcx, fcy, j, p, rj,
                               k, pu);
  nf = add2(nf, mul2(nf, rj, pu), pu);
  const float max_step = __fmul_rn(2.0f, D.csf);
  const float2 nsq = mul2(nf, nf, pu);
  const float speed = __fsqrt_rn(__fadd_rn(nsq.x, nsq.y));
  if (speed > max_step) nf = mul2(nf, splat(__fdiv_rn(max_step, speed)), pu);
  vel = add2(vel, nf, pu);
  if (!(v.flags[P] & kPinned)) v.pos[P] = integrate(p, vel.x, vel.y, D.friction, D.space);
}

__global__ void __launch_bounds__(kBlock) kb_manybody(BatchView v) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = v.cell_start[v.cell_hwm];
  if (j >= total) return;
  const uint32_t P = v.sorted_idx[j];
  const uint32_t g = v.gid[P];
  const GraphDesc& D = v.desc[g];
  const BatchTick tp = tick_of(v, g);
  const float2 p = v.sorted_pos[j];
  const float k = __fmul_rn(tp.alpha, D.repulsion);
  if (!quotient_by_recip(k)) kb_manybody_point<false>(v, D, j, P, p, k);
  else if (D.level_guard && __ldg(&v.big_count[kBatchOutside]) == 0) kb_manybody_point<true, true>(v, D, j, P, p, k);
  else kb_manybody_point<true>(v, D, j, P, p, k);
}

// ------------------------------------------------------------------- link --
// Graphs that do not run this pass (no links, masked, or inactive) copy their
// positions through, so the ping-pong buffers stay consistent.
__global__ void __launch_bounds__(kBlock) kb_link(BatchView v, int direction, const float2* __restrict__ src,
                                                  float2* __restrict__ dst, const uint32_t* __restrict__ rows,
                                                  uint32_t nrows) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const uint32_t P = rows ? rows[t] : t;
  const uint32_t g = v.gid[P];
  if (g == kNoGraph) return;
  const GraphDesc& D = v.desc[g];
  const BatchTick tp = tick_of(v, g);
  const uint32_t i = P - D.p_off;
  const uint32_t rp = (direction == 0 ? D.rp_in : D.rp_out) + i;
  const uint32_t e0 = v.rowptr[rp], e1 = v.rowptr[rp + 1];
  if (!rows && e1 - e0 > kHeavyDegree) return;
  const float2 pp = src[P];
  const uint32_t stage = direction == 0 ? kGLinkIn : kGLinkOut;
  const uint8_t f = v.flags[P];
  if (!tp.active || !(D.stages & stage) || (f & kAbsent)) { dst[P] = pp; return; }
  const float sa = __fmul_rn(D.link_spring, tp.alpha);
  const PairUnits pu = v.units;
  const float span = __fsub_rn(D.link_r1, D.link_r0);
  float2 vel = make_float2(0.f, 0.f);
  auto spring = [&](const uint4 en, const float2 q) {
    float dd = __fadd_rn(__fmul_rn(__uint_as_float(en.y), span), D.link_r0);
    dd = __fmul_rn(dd, D.link_distance);
    spring_step(pp, vel, q, dd, __fmul_rn(dd, 0.99f), sa, __uint_as_float(en.w), __uint_as_float(en.z), pu);
  };

  constexpr int kLinkBatch = 4;
  uint32_t at = e0;
  for (; at + kLinkBatch <= e1; at += kLinkBatch) {
    uint4 en[kLinkBatch];
    float2 q[kLinkBatch];
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) en[u] = __ldg(&v.ent[at + u]);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u) q[u] = en[u].x != kAbsentTarget ? __ldg(&src[en[u].x]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kLinkBatch; ++u)
      if (en[u].x != kAbsentTarget) spring(en[u], q[u]);
  }
  for (; at < e1; ++at) {
    const uint4 en = __ldg(&v.ent[at]);
    if (en.x == kAbsentTarget) continue;
    spring(en, __ldg(&src[en.x]));
  }
  dst[P] = (f & kPinned) ? pp : integrate(pp, vel.x, vel.y, D.friction, D.space);
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
  if (v.cell_hwm) {
    const uint32_t n1 = (v.cell_hwm + kChunk - 1) / kChunk;   // partials of 1024 cells
    const uint32_t n2 = (n1 + kChunk - 1) / kChunk;           // partials of 1024^2 cells (<= 1024)
    kb_scan_reduce<<<n1, kBlock, 0, st>>>(v.counts, v.cell_hwm, v.scan1);
    kb_scan_reduce<<<n2, kBlock, 0, st>>>(v.scan1, n1, v.scan2);
    kb_scan_down<<<1, kBlock, 0, st>>>(v.scan2, n2, nullptr, v.scan2, nullptr);
    kb_scan_down<<<n2, kBlock, 0, st>>>(v.scan1, n1, v.scan2, v.scan1, nullptr);
    kb_scan_cells<<<n1, kBlock, 0, st>>>(v, v.scan1);
  }
  if (v.point_hwm) kb_scatter<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  kb_bigcells<<<8 * sm_count(), kBlock, 0, st>>>(v);   // as k_bigcells: 8 blocks per SM
  if (v.n_tiles) kb_cells<<<v.n_tiles, kBlock, 0, st>>>(v);
  if (v.slots) kb_coarse<<<v.slots, kBlock, 0, st>>>(v);
  if (v.point_hwm) kb_manybody<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  for (int dir = 0; dir < 2; ++dir) {
    const float2* src = dir == 0 ? v.pos : v.pos_alt;
    float2* dst = dir == 0 ? v.pos_alt : v.pos;
    const uint32_t* heavy = dir == 0 ? v.heavy_in : v.heavy_out;
    const uint32_t nh = dir == 0 ? v.n_heavy_in : v.n_heavy_out;
    if (nh) {
      cudaEventRecord(fork[dir], st);
      cudaStreamWaitEvent(side, fork[dir], 0);
      kb_link<<<blocks(nh), kBlock, 0, side>>>(v, dir, src, dst, heavy, nh);
      cudaEventRecord(join[dir], side);
    }
    if (v.point_hwm) kb_link<<<blocks(v.point_hwm), kBlock, 0, st>>>(v, dir, src, dst, nullptr, v.point_hwm);
    if (nh) cudaStreamWaitEvent(st, join[dir], 0);
  }
  if (v.any_collision && v.point_hwm) {   // after the links, as in runSimulationStep (src/index.ts:2068-2078)
    kb_coll_grid<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
    if (v.coll_hwm) kb_coll_convert<<<blocks(v.coll_hwm), kBlock, 0, st>>>(v);
    kb_coll_force<<<blocks(v.point_hwm), kBlock, 0, st>>>(v);
  }
  kb_tick_end<<<1, 1, 0, st>>>(v);
}

uint32_t batch_kernels_per_tick(const BatchView& v) {
  uint32_t k = 1 + 1 + 1 + 1 + 1 + 2;   // prepass, scatter, big cells, coarse, manybody, link x2
  if (v.cell_hwm) k += 5;
  if (v.n_tiles) k += 1;
  k += (v.n_heavy_in > 0) + (v.n_heavy_out > 0);
  if (v.any_center) k += 1;
  if (v.any_collision) k += 2 + (v.coll_hwm > 0);
  return k + 1;                          // tick end
}

}  // namespace cgl
