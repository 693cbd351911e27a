// collision.cuh — the collision force's device arithmetic, shared by the
// plain engine (kernels.cu) and the batched one (batch_kernels.cu):
// ForceCollision.run (ForceCollision/index.ts:264-345), build-grid.vert:28-62
// for the grid sums and force-collision-spatial.frag:103-168 for the force.
#pragma once
#include "common.cuh"

namespace cgl {

// The four grid offsets (ForceCollision/index.ts:19-24): (0,0), (.5,0), (0,.5), (.5,.5).
__device__ __forceinline__ float coll_offset_x(int g) { return (g & 1) ? 0.5f : 0.f; }
__device__ __forceinline__ float coll_offset_y(int g) { return (g & 2) ? 0.5f : 0.f; }

// clamp(floor((p + o * cs) / cs), 0, G - 1) (build-grid.vert, force-collision-spatial.frag)
__device__ __forceinline__ float coll_bin(float p, float o, float cs, float gm1) {
  const float off = __fadd_rn(p, __fmul_rn(o, cs));
  float c = gclamp(floorf(__fdiv_rn(off, cs)), 0.f, gm1);
  if (!(c == c)) c = 0.f;
  return c;
}

// Warp-wide sum of a 64-bit value (all 32 lanes take part).
__device__ __forceinline__ long long warp_sum64(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Adds the point's exact (x, y, size, 1) terms into its cell of each of the
// four G x G grids at acc (4 longs per cell, grid g at 4 G^2 g).  All 32 lanes
// call it (`live` marks the lanes with a point): the lanes of one cell sum
// their terms first and one lane adds the cell's total (at most kCollRounds
// cells per warp and grid, the rest add their own terms).  Integer sums are
// order-free, so the grids are the same whichever lanes meet.
constexpr int kCollRounds = 6;
__device__ __forceinline__ void coll_accumulate(long long* __restrict__ acc, int G, float cs, const FixedScale& fxs,
                                                float2 p, float sz, bool live) {
  const int lane = threadIdx.x & 31;
  const float gm1 = (float)G - 1.0f;
  const long long fx = live ? to_fixed(p.x, fxs) : 0, fy = live ? to_fixed(p.y, fxs) : 0;
  const long long fs = live ? to_fixed(sz, fxs) : 0;
  const uint32_t G2 = (uint32_t)(G * G);
  const unsigned active = __ballot_sync(0xffffffffu, live);
#pragma unroll 1
  for (int g = 0; g < 4; ++g) {
    const int cx = (int)coll_bin(p.x, coll_offset_x(g), cs, gm1);
    const int cy = (int)coll_bin(p.y, coll_offset_y(g), cs, gm1);
    const uint32_t key = (uint32_t)(cy * G + cx);
    long long* a = acc + 4 * ((size_t)g * G2 + key);
    unsigned todo = active;
#pragma unroll 1
    for (int r = 0; r < kCollRounds && todo; ++r) {
      const int l = __ffs(todo) - 1;
      const long long* al = (const long long*)__shfl_sync(0xffffffffu, (unsigned long long)a, l);
      const bool mine = ((todo >> lane) & 1u) && a == al;
      const unsigned grp = __ballot_sync(0xffffffffu, mine);
      const long long sx = warp_sum64(mine ? fx : 0);
      const long long sy = warp_sum64(mine ? fy : 0);
      const long long ss = warp_sum64(mine ? fs : 0);
      if (lane == l) {
        atomicAdd((unsigned long long*)&a[0], (unsigned long long)sx);
        atomicAdd((unsigned long long*)&a[1], (unsigned long long)sy);
        atomicAdd((unsigned long long*)&a[2], (unsigned long long)ss);
        atomicAdd((unsigned long long*)&a[3], (unsigned long long)__popc(grp));
      }
      todo &= ~grp;
    }
    if ((todo >> lane) & 1u) {
      atomicAdd((unsigned long long*)&a[0], (unsigned long long)fx);
      atomicAdd((unsigned long long*)&a[1], (unsigned long long)fy);
      atomicAdd((unsigned long long*)&a[2], (unsigned long long)fs);
      atomicAdd((unsigned long long*)&a[3], 1ull);
    }
  }
}

// One grid cell's sums rounded once to f32 (sx, sy, ssize, count), and the
// integer sums zeroed for the next tick.
template <bool ZERO = true>
__device__ __forceinline__ void coll_convert_cell(long long* a, float4* out, const FixedScale& fx) {
  *out = make_float4(from_fixed(a[0], fx), from_fixed(a[1], fx), from_fixed(a[2], fx), (float)a[3]);
  if (ZERO) { a[0] = 0; a[1] = 0; a[2] = 0; a[3] = 0; }
}

struct CollParams {
  int grid;         // G (collision grid size)
  float cell;       // cell size
  float radius;     // simulationCollisionRadius, 0 when undefined (radius from the sizes)
  float padding;
  float alpha_strength;   // alpha * simulationCollision, rounded to f32
};

// The collision velocity of point `index` (of n) at p with size csz: the four
// offset grids' 3x3 neighbourhoods, each pass damped and capped, summed in
// pass order (force-collision-spatial.frag:103-168).
__device__ __forceinline__ float2 coll_velocity(const float4* __restrict__ grids, const CollParams& cp, float2 p,
                                                float csz, uint32_t index, uint32_t n) {
  const float cs = cp.cell;
  const int G = cp.grid;
  const float Gf = (float)G;
  const float gm1 = Gf - 1.0f;
  const uint32_t G2 = (uint32_t)(G * G);
  const float cur = (float)index;
  const float cr = cp.radius, pad = cp.padding;
  const float R = __fadd_rn(cr > 0.f ? cr : __fmul_rn(csz, 0.5f), pad);
  float vx = 0.f, vy = 0.f;
  if (cur < 0.f || cur >= (float)n) return make_float2(vx, vy);
  for (int g = 0; g < 4; ++g) {
    const float mx = coll_bin(p.x, coll_offset_x(g), cs, gm1);
    const float my = coll_bin(p.y, coll_offset_y(g), cs, gm1);
    const float4* grid = grids + (size_t)g * G2;
    float total = 0.f, gx = 0.f, gy = 0.f;
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy) {
        const float ncx = __fadd_rn(mx, (float)dx), ncy = __fadd_rn(my, (float)dy);
        if (ncx < 0.f || ncx >= Gf || ncy < 0.f || ncy >= Gf) continue;
        const float4 cd = __ldg(&grid[(int)ncy * G + (int)ncx]);
        const float cnt = cd.w;
        if (cnt < 0.5f) continue;
        float ec = cnt, spx = cd.x, spy = cd.y, ss = cd.z;
        if (dx == 0 && dy == 0) {
          ec = __fsub_rn(cnt, 1.0f);
          spx = __fsub_rn(spx, p.x); spy = __fsub_rn(spy, p.y); ss = __fsub_rn(ss, csz);
        }
        if (ec < 0.5f) continue;
        total = __fadd_rn(total, ec);
        const float avx = __fdiv_rn(spx, ec), avy = __fdiv_rn(spy, ec);
        const float avs = __fdiv_rn(ss, ec);
        const float oR = __fadd_rn(cr > 0.f ? cr : __fmul_rn(avs, 0.5f), pad);
        const float comb = __fadd_rn(R, oR);
        const float ddx = __fsub_rn(p.x, avx), ddy = __fsub_rn(p.y, avy);
        const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(ddy, ddy)));
        if (dist < comb && dist > 0.001f) {
          const float ov = __fdiv_rn(__fsub_rn(comb, dist), comb);
          const float soft = __fmul_rn(__fmul_rn(__fsqrt_rn(ov), comb), 0.5f);
          const float dirx = __fdiv_rn(ddx, dist), diry = __fdiv_rn(ddy, dist);
          float fo = __fmul_rn(__fmul_rn(__fmul_rn(cp.alpha_strength, soft), 0.25f), ec);
          fo = gmin(fo, __fmul_rn(comb, 0.5f));
          gx = __fadd_rn(gx, __fmul_rn(fo, dirx));
          gy = __fadd_rn(gy, __fmul_rn(fo, diry));
        } else if (dist <= 0.001f && ec > 0.f) {
          const float ang = __fmul_rn(cur, 0.618033988749895f);
          const float fo = gmin(__fmul_rn(__fmul_rn(cp.alpha_strength, comb), 0.1f), __fmul_rn(comb, 0.3f));
          float sn, cn;
          portable_sincos(ang, &sn, &cn);
          const float fe = __fmul_rn(fo, ec);
          gx = __fadd_rn(gx, __fmul_rn(fe, cn));
          gy = __fadd_rn(gy, __fmul_rn(fe, sn));
        }
      }
    if (total > 2.0f) {
      const float dmp = __fdiv_rn(2.0f, total);
      gx = __fmul_rn(gx, dmp); gy = __fmul_rn(gy, dmp);
    }
    const float maxc = __fmul_rn(R, 0.1f);
    const float corr = __fsqrt_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)));
    if (corr > maxc) {
      const float sc = __fdiv_rn(maxc, corr);
      gx = __fmul_rn(gx, sc); gy = __fmul_rn(gy, sc);
    }
    vx = __fadd_rn(vx, gx);
    vy = __fadd_rn(vy, gy);
  }
  return make_float2(vx, vy);
}

}  // namespace cgl
