// ingest.h — host-side ingest shared by the plain and the batched engine:
// what Graph.render does before the first tick (GraphData.update,
// Points.updatePositions, ForceManyBody.create, ForceLink.create).
// Both engines call these functions, so a graph ingested into a batch gets the
// same device data, random draws included, as the same graph on its own.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/cgl.h"
#include "common.cuh"
#include "random_stream.h"

namespace cgl {
namespace ingest {

// SplitMix64 draw k (0-based) of seed s (the counter stream, below).
inline uint64_t splitmix_draw(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline double splitmix_unit(uint64_t seed, uint64_t k) { return (double)(splitmix_draw(seed, k) >> 11) * 0x1.0p-53; }

// The random draws of one graph, in the reference's order and count
// (Store.getRandomFloat, Store/index.ts:200-202).  By default they are the
// reference's own stream (random_stream.h: random@4.1.0 over seedrandom@3.0.5,
// seeded with String(randomSeed)).  cgl_config.random_stream =
// CGL_RANDOM_COUNTER selects SplitMix64 instead (draw k of seed s =
// splitmix(s + (k + 1) * golden gamma), u = top 53 bits / 2^53): not the
// reference's values, but draw k needs no earlier draw, so the device builds
// large graphs' jitter and link draws itself.
struct Rng {
  bool counter = false;
  RandomStream ref;        // the reference's stream
  uint64_t seed = 0;       // the counter stream's seed
  uint64_t ctr = 0;        // draws so far

  double unit() {
    const double u = counter ? splitmix_unit(seed, ctr) : ref.next();
    ++ctr;
    return u;
  }
  // Random.float(min, max) = next() * (max - min) + min
  double uniform(double mn, double mx) { return unit() * (mx - mn) + mn; }

  // out[k] = f32(float(0, 1)), n draws (ForceLink/index.ts:76)
  void fill_unit_f32(float* out, uint64_t n) {
    if (counter) {
      for (uint64_t k = 0; k < n; ++k) out[k] = (float)splitmix_unit(seed, ctr + k);
    } else {
      ref.fill_unit_f32(out, n);
    }
    ctr += n;
  }
  // ForceManyBody.create jitter (ForceManyBody/index.ts:133-138): two draws per
  // texel of `texels`, f32(float(-1, 1) * 0.00001); the first `keep` texels kept.
  void fill_jitter(float* out_xy, uint64_t keep, uint64_t texels) {
    if (counter) {
      for (uint64_t t = 0; t < texels; ++t) {
        const double ux = splitmix_unit(seed, ctr + 2 * t), uy = splitmix_unit(seed, ctr + 2 * t + 1);
        if (t < keep) {
          out_xy[2 * t] = (float)((ux * 2.0 + -1.0) * 0.00001);
          out_xy[2 * t + 1] = (float)((uy * 2.0 + -1.0) * 0.00001);
        }
      }
    } else {
      ref.fill_jitter(out_xy, keep, texels);
    }
    ctr += 2 * texels;
  }
};

// Store.addRandomSeed(randomSeed) (Store/index.ts:196-198, src/index.ts:452):
// the seed text is random_seed_text when given, else random_seed in decimal
// (JavaScript's String(n) for an integer below 2^53).  Without a seed the
// reference draws from Math.random; the engine seeds from the host's entropy.
inline void seed_rng(const cgl_config& c, Rng& r) {
  r = Rng{};
  r.counter = c.random_stream == CGL_RANDOM_COUNTER;
  if (c.has_random_seed) {
    r.seed = c.random_seed;
    if (c.random_seed_text) r.ref.seed_utf8(c.random_seed_text);
    else r.ref.seed_utf8(std::to_string(c.random_seed).c_str());
  } else {
    std::random_device rd;
    r.seed = ((uint64_t)rd() << 32) ^ rd();
    r.ref.seed_utf8(std::to_string(r.seed).c_str());
  }
}

// Store.adjustSpaceSize (Store/index.ts:209-233)
inline double adjusted_space(const cgl_config& c) {
  double s = c.space_size;
  if (!(s > 0) || !std::isfinite(s)) s = 4096;
  if (s < 2) s = 2;
  const double m = c.max_texture_dimension;
  if (m > 0 && std::isfinite(m) && m >= 2 && s >= m) s = std::max(m / 2, 2.0);
  return s;
}

// GraphData.isPointIndex (GraphData/index.ts:286-289)
inline bool is_point_index(double v, uint64_t n) {
  return std::isfinite(v) && v == std::floor(v) && v >= 0 && v < (double)n;
}

// Exact cell sums: coordinates saturate at B = smallest power of two >= 2*S,
// scaled by 2^F with F = 62 - ceil(log2 N) - log2 B (N * B * 2^F <= 2^62).
inline FixedScale fixed_for(uint64_t n, double space, int* bits) {
  const float S = (float)space;
  int lb = 0;
  while (std::ldexp(1.0, lb) < 2.0 * (double)S) ++lb;
  int ln = 0;
  while ((1ull << ln) < (n < 1 ? 1 : n)) ++ln;
  int F = 62 - ln - lb;
  if (F > 60) F = 60;
  if (bits) *bits = F;
  FixedScale fx;
  fx.bound = (float)std::ldexp(1.0, lb);
  fx.scale = std::ldexp(1.0f, F);
  fx.inv = std::ldexp(1.0f, -F);
  return fx;
}

// ForceManyBody.createLevels (ForceManyBody/index.ts:646-667)
struct Grid {
  int gf = 0, levels = 0;
};
inline Grid grid_for(uint64_t n) {
  Grid g;
  const double target = 2 * std::sqrt((double)n);
  const double f = std::min((double)kMaxGrid, std::max(8.0, std::pow(2.0, std::ceil(std::log2(target)))));
  g.gf = (int)f;
  g.levels = (int)std::log2(f) - 1;
  return g;
}
// cells of all levels of a pyramid with `levels` levels, and the offset of level l
inline uint32_t level_base(int l) { uint32_t o = 0; for (int m = 0; m < l; ++m) o += (uint32_t)((4 << m) * (4 << m)); return o; }

// Math.min / Math.max of two doubles: NaN if either is NaN, -0 below +0.
inline double js_min(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return NAN;
  if (a == b) return std::signbit(a) ? a : b;
  return a < b ? a : b;
}
inline double js_max(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return NAN;
  if (a == b) return std::signbit(a) ? b : a;
  return a > b ? a : b;
}

// Points.updatePositions' rescale decision (Points/index.ts:396-402):
// rescalePositions, or true when it is undefined and the simulation is off;
// setPointPositions(…, dontRescale) skips it once.
inline bool should_rescale(const cgl_config& c, bool dont_rescale) {
  bool r = c.rescale_positions == 1;
  if (c.rescale_positions < 0 && !c.enable_simulation) r = true;
  return r && !dont_rescale;
}

// Points.rescaleInitialNodePositions (Points/index.ts:3134-3218) on the staged
// positions, in place: the extent of the live points (absent = NaN in either
// coordinate, left as they are), then x' = (x - minX) * scale + offsetX in FP64
// as in JavaScript, stored as f32 like the reference's Float32Array.  `space` is
// the configured spaceSize (not the adjusted one).
inline void rescale_positions(float* xy, uint64_t n, double space) {
  if (space == 0 || std::isnan(space)) return;
  double minX = INFINITY, maxX = -INFINITY, minY = INFINITY, maxY = -INFINITY;
  for (uint64_t i = 0; i < n; ++i) {
    const float x = xy[2 * i], y = xy[2 * i + 1];
    if (std::isnan(x) || std::isnan(y)) continue;
    minX = js_min(minX, x);
    maxX = js_max(maxX, x);
    minY = js_min(minY, y);
    maxY = js_max(maxY, y);
  }
  if (!std::isfinite(minX)) return;   // no live point (or an infinite extent): no scale
  const double w = maxX - minX, h = maxY - minY;
  const double range = js_max(w, h);
  if (range == 0) {   // one point or all coincident: centre them, keeping offsets
    const double center = space / 2;
    for (uint64_t i = 0; i < n; ++i) {
      if (std::isnan(xy[2 * i]) || std::isnan(xy[2 * i + 1])) continue;
      xy[2 * i] = (float)((double)xy[2 * i] - minX + center);
      xy[2 * i + 1] = (float)((double)xy[2 * i + 1] - minY + center);
    }
    return;
  }
  if (range > space) return;
  const double density = space * space * 0.001;
  const double effective = (double)n > density ? space * js_max(1.2, std::sqrt((double)n) / space) : space * 0.1;
  const double scale = effective / range;
  const double center_off = (space - effective) / 2;
  const double offX = ((range - w) / 2) * scale + center_off;
  const double offY = ((range - h) / 2) * scale + center_off;
  for (uint64_t i = 0; i < n; ++i) {
    if (std::isnan(xy[2 * i]) || std::isnan(xy[2 * i + 1])) continue;
    xy[2 * i] = (float)(((double)xy[2 * i] - minX) * scale + offX);
    xy[2 * i + 1] = (float)(((double)xy[2 * i + 1] - minY) * scale + offY);
  }
}

// Points.updatePositions (Points/index.ts:390-592, position-utils.ts:9-27):
// a NaN in either coordinate makes the point absent (both coordinates NaN).
inline uint64_t canonical_positions(const float* xy, uint64_t n, std::vector<float2>& pos, std::vector<uint8_t>& absent) {
  pos.resize(n);
  absent.assign(n, 0);
  uint64_t live = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const float x = xy[2 * i], y = xy[2 * i + 1];
    const bool ab = std::isnan(x) || std::isnan(y);
    absent[i] = ab;
    live += !ab;
    pos[i] = ab ? make_float2(NAN, NAN) : make_float2(x, y);
  }
  return live;
}

// ForceManyBody.create jitter (ForceManyBody/index.ts:133-138): two draws per
// texel of the pointsTextureSize^2 texture, texel order, only the first n kept.
inline void jitter(Rng& rng, uint64_t n, std::vector<float2>& out) {
  out.resize(n);
  const uint64_t T = (uint64_t)std::ceil(std::sqrt((double)n));
  rng.fill_jitter((float*)out.data(), n, T * T);
}

struct Csr {
  std::vector<uint32_t> rowptr;   // n + 1
  std::vector<uint4> ent;         // (neighbour, random distance draw bits, bias bits, strength bits)
  std::vector<uint32_t> heavy;    // points whose list is longer than kHeavyDegree
  std::vector<uint32_t> order;    // all points by list length, longest first (ties by index)
  uint32_t max_degree = 0;
};

// ForceLink.create for one direction (ForceLink/index.ts:40-83): lists in
// link-index order (GraphData/index.ts:534-547); bias and strength in FP64
// rounded to f32; one random draw per entry in list order.  Links to absent
// points keep their draw and carry the kAbsentTarget sentinel.
inline void build_direction(const float* links, uint64_t E, uint64_t N, bool incoming, const std::vector<uint32_t>& deg,
                            const float* strength, const std::vector<uint8_t>& absent, Rng& rng, Csr& c) {
  c.rowptr.assign(N + 1, 0);
  std::vector<uint8_t> valid(E, 0);
  for (uint64_t i = 0; i < E; ++i) {
    const double s = links[2 * i], t = links[2 * i + 1];
    if (!is_point_index(s, N) || !is_point_index(t, N)) continue;
    valid[i] = 1;
    c.rowptr[(uint32_t)(incoming ? s : t) + 1]++;
  }
  c.max_degree = 0;
  c.heavy.clear();
  for (uint64_t p = 0; p < N; ++p) {
    c.max_degree = std::max(c.max_degree, c.rowptr[p + 1]);
    if (c.rowptr[p + 1] > kHeavyDegree) c.heavy.push_back((uint32_t)p);
  }
  {   // counting sort of the points by list length, descending
    std::vector<uint32_t> bucket((size_t)c.max_degree + 2, 0);
    for (uint64_t p = 0; p < N; ++p) bucket[c.max_degree - c.rowptr[p + 1] + 1]++;
    for (size_t k = 1; k < bucket.size(); ++k) bucket[k] += bucket[k - 1];
    c.order.assign(N, 0);
    for (uint64_t p = 0; p < N; ++p) c.order[bucket[c.max_degree - c.rowptr[p + 1]]++] = (uint32_t)p;
  }
  for (uint64_t p = 0; p < N; ++p) c.rowptr[p + 1] += c.rowptr[p];
  const uint32_t M = c.rowptr[N];
  c.ent.assign(M, make_uint4(0, 0, 0, 0));
  std::vector<uint32_t> lidx(M);
  std::vector<uint32_t> cur(c.rowptr.begin(), c.rowptr.end() - 1);
  for (uint64_t i = 0; i < E; ++i) {
    if (!valid[i]) continue;
    const uint32_t s = (uint32_t)links[2 * i], t = (uint32_t)links[2 * i + 1];
    const uint32_t p = incoming ? s : t, q = incoming ? t : s;
    const uint32_t at = cur[p]++;
    c.ent[at].x = q;
    lidx[at] = (uint32_t)i;
  }
  for (uint64_t p = 0; p < N; ++p) {
    for (uint32_t at = c.rowptr[p]; at < c.rowptr[p + 1]; ++at) {
      const uint32_t q = c.ent[at].x;
      const double degree = deg[q], connected = deg[p];
      const double sum = degree + connected;
      const double bias = sum != 0 ? degree / sum : 0.5;
      const double mind = std::min(degree, connected);
      double st;
      const double si = strength ? (double)strength[lidx[at]] : 0.0;
      if (!strength || !std::isfinite(si) || si < 0) st = 1.0 / std::max(mind, 1.0);
      else st = si;
      st = std::sqrt(st);
      const float fb = (float)bias, fs = (float)st, fr = (float)rng.uniform(0, 1);
      std::memcpy(&c.ent[at].y, &fr, 4);
      std::memcpy(&c.ent[at].z, &fb, 4);
      std::memcpy(&c.ent[at].w, &fs, 4);
      if (absent[q]) c.ent[at].x = kAbsentTarget;
    }
  }
}

// ForceLink.create(INCOMING) then (OUTGOING) (src/index.ts:1663-1666).
// `strength` is used only when its length matched linksNumber
// (GraphData/index.ts:408-418); pass nullptr otherwise.
inline void build_links(const float* links, uint64_t E, uint64_t N, const float* strength,
                        const std::vector<uint8_t>& absent, Rng& rng, Csr& in, Csr& out) {
  std::vector<uint32_t> deg(N, 0);
  for (uint64_t i = 0; i < E; ++i) {
    const double s = links[2 * i], t = links[2 * i + 1];
    if (is_point_index(s, N) && is_point_index(t, N)) { deg[(size_t)s]++; deg[(size_t)t]++; }
  }
  build_direction(links, E, N, true, deg, strength, absent, rng, in);
  build_direction(links, E, N, false, deg, strength, absent, rng, out);
}

// Clusters.create (Clusters/index.ts:54-100) on GraphData.updateClusters
// (GraphData/index.ts:420-441): per-point clusters apply only when there is
// one value per point, cluster positions whenever set, per-point strength only
// when there is one value per point.  A cluster index is a non-negative
// integer below 2^24; NaN (undefined), negative, non-integer and infinite
// values leave the point unclustered.  clusterCount = max index + 1 (at least
// 1); a cluster position is (x, y), -1 where undefined (NaN) or not given.
struct Clusters {
  bool point_clusters = false;     // GraphData.pointClusters defined
  bool positions = false;          // GraphData.clusterPositions defined
  uint32_t count = 0;              // clusterCount
  std::vector<uint32_t> of;        // [N] cluster of each point, kNoClusterId if none
  std::vector<float> coeff;        // [N] clusterForceCoefficient
  std::vector<float2> custom;      // [count] cluster position, negative = centre of mass
};
inline void build_clusters(uint64_t N, bool have_idx, const std::vector<float>& idx, bool have_pos,
                           const std::vector<float>& cpos, bool have_str, const std::vector<float>& str, Clusters& c) {
  c.point_clusters = have_idx && N > 0 && idx.size() == N;
  c.positions = have_pos && N > 0;
  c.of.assign(N, kNoClusterId);
  c.coeff.assign(N, 1.0f);
  uint32_t maxc = 0;
  if (c.point_clusters)
    for (uint64_t i = 0; i < N; ++i) {
      const float v = idx[i];
      if (!(v >= 0.f) || !(v < 16777216.f) || v != std::floor(v)) continue;
      c.of[i] = (uint32_t)v;
      maxc = std::max(maxc, (uint32_t)v);
    }
  c.count = maxc + 1;
  if (have_str && str.size() == N) std::copy(str.begin(), str.end(), c.coeff.begin());
  c.custom.assign(c.count, make_float2(-1.f, -1.f));
  if (c.positions)
    for (uint32_t k = 0; k < c.count; ++k) {
      if (2 * (size_t)k < cpos.size() && !std::isnan(cpos[2 * (size_t)k])) c.custom[k].x = cpos[2 * (size_t)k];
      if (2 * (size_t)k + 1 < cpos.size() && !std::isnan(cpos[2 * (size_t)k + 1])) c.custom[k].y = cpos[2 * (size_t)k + 1];
    }
}

}  // namespace ingest
}  // namespace cgl
