// oracle.cpp — CPU restatement of cosmos.gl's per-tick force simulation.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
// engine in graph_gb300/: only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load it, and only as the checker or the timed CPU
// baseline.  Nothing in the product links, loads or calls it.
//
// Parity status: UNPINNED by the reference.  cosmos.gl (@cosmos.gl/graph
// v3.4.1) ships no tests, fixtures or golden vectors for this path, and the
// reference (TypeScript + GLSL ES 3.00 over WebGL2) cannot execute on this
// machine.  This file restates the reference's shaders and TypeScript logic
// operation by operation; the knowns it is pinned to are the documented
// invariants (exactly-once pyramid tiling, sparse-cell exactness, the
// lowbias32 definition) and hand-derived known answers in tests/golden/.
//
// Restatement rules (applied uniformly, and identically by the engine):
//  * every FP32 operation of a shader is one IEEE-754 correctly rounded
//    operation, in the shader's order; no FMA contraction (build flag
//    -ffp-contract=off).  GLSL leaves division/sqrt precision to the driver;
//    this fixes it to correct rounding.
//  * GLSL builtins: max(x,y) = x<y ? y : x; min(x,y) = y<x ? y : x;
//    clamp = min(max()); length(v) = sqrt(v.x*v.x + v.y*v.y);
//    normalize(v) = v * (1/length(v)), the reciprocal correctly rounded
//    (GPUs evaluate normalize as v * inversesqrt(dot(v, v)); GLSL fixes
//    neither form).
//  * vec2(cos(atan(y,x)), sin(atan(y,x))) (force-gravity.frag:36-38,
//    force-center.frag:31-33) is the unit vector (x/r, y/r), r = length,
//    its exact mathematical value.
//  * sin/cos of an arbitrary angle (force-collision-spatial.frag:147) use
//    cgl-portable sincos: Cody-Waite reduction by pi/2 in FP64 and Taylor
//    series, rounded to FP32 (see portable_sincos below).
//  * additive blending of a point-list draw (cell sums: calculate-level.vert,
//    build-grid.vert, calculate-centermass.vert) = the EXACT sum of the f32
//    inputs, rounded once to f32.  The exact sum is an integer in units of
//    2^-F (F from the point count and space size, coordinates saturated at
//    +-B), so it is order-free.  The reference's own blending is a sequence of
//    f32 adds in draw order; that variant is kept as sum_mode 1 to put the
//    difference on record.  Blending of full-screen passes into the velocity
//    target is restated as f32 adds in pass order.
//  * random numbers: the reference's generator, random@4.1.0 over
//    seedrandom@3.0.5 (package-lock.json:8264-8274, 8687-8690; neither is
//    vendored in the reference), restated from their published algorithms in
//    Arc4Seed below: Random.clone(seed) seeds seedrandom with String(seed);
//    seedrandom mixes the string's UTF-16 code units into an RC4 key, drops
//    256 bytes and builds each double from 7+ bytes; Random.float(min, max) =
//    next() * (max - min) + min.  Pinned by seedrandom's README known answers
//    (tests/test_oracle.py).  Draw ORDER and COUNT follow the call sites of
//    Store.getRandomFloat (Store/index.ts:200-202): ForceManyBody/index.ts:133-138,
//    :521; ForceLink/index.ts:76.  The one step no available source pins is
//    random's own glue (that it seeds with `seed + ''` and scales next() as
//    above); it is the package's documented behaviour.  random_stream =
//    CGL_RANDOM_COUNTER selects SplitMix64 instead (Steele, Lea, Flood 2014;
//    draw k of seed s = mix(s + (k+1)*0x9E3779B97F4A7C15), u = (mix >> 11) *
//    2^-53), the engine's opt-in stream for device-side draws.
//  * near-field peel ties (build-nearfield-slots.vert:146-162): slot k of a
//    cell holds the lowest-index point among those with the k-th smallest
//    DISTINCT f32 hash (the depth test keeps the first-drawn of equal depths;
//    eligibility `hash > previous.hash` drops the rest).
#include "../include/cgl.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- helpers --
inline float gmax(float x, float y) { return x < y ? y : x; }
inline float gmin(float x, float y) { return y < x ? y : x; }
inline float gclamp(float x, float a, float b) { return gmin(gmax(x, a), b); }

// ivec2(floor(p / cellSize)) clamped to [0, G-1]  (calculate-level.vert:47-48,
// build-nearfield-slots.vert:143-144, force-level.frag:66, force-nearfield.frag:209).
inline int cell_index(float p, float cs, int G) {
  float f = floorf(p / cs);
  int c;
  if (!(f >= -1.0f)) c = -1;                 // also NaN
  else if (f > (float)G) c = G;
  else c = (int)f;
  return c < 0 ? 0 : (c > G - 1 ? G - 1 : c);
}

// SplitMix64 draw k (0-based) for seed s.
inline uint64_t splitmix_draw(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline double splitmix_unit(uint64_t seed, uint64_t k) {
  return (double)(splitmix_draw(seed, k) >> 11) * 0x1.0p-53;
}

// seedrandom@3.0.5's default generator, restated from its published source
// description in the arithmetic it uses (JavaScript doubles):
//   mixkey(seed, key): for j over the seed string's UTF-16 code units,
//     key[j & 255] = 255 & ((smear ^= key[j & 255] * 19) + code[j]);
//   ARC4(key): RC4 key schedule over key (empty key = [0]), then g(256) drops
//     256 output bytes; g(count) = the next `count` output bytes as a base-256
//     number;
//   prng(): n = g(6), d = 2^48, x = 0; while (n < 2^52) { n = (n + x) * 256;
//     d *= 256; x = g(1) }; while (n >= 2^53) { n /= 2; d /= 2; x >>>= 1 };
//     return (n + x) / d.
struct Arc4Seed {
  int S[256];
  int i = 0, j = 0;
  void seed(const std::vector<uint16_t>& code) {
    std::vector<int> key;
    double smear = 0;   // `undefined` before the first ^=, which reads as 0
    for (size_t k = 0; k < code.size(); ++k) {
      const size_t at = k & 255;
      const int prev = at < key.size() ? key[at] : 0;   // undefined * 19 -> NaN -> 0 under ^
      smear = (double)((int32_t)smear ^ (int32_t)(prev * 19));
      const int v = 255 & (int)(smear + code[k]);
      if (at < key.size()) key[at] = v; else key.push_back(v);
    }
    if (key.empty()) key.push_back(0);
    for (int k = 0; k < 256; ++k) S[k] = k;
    int jj = 0;
    for (int k = 0; k < 256; ++k) {
      const int t = S[k];
      jj = 255 & (jj + key[k % key.size()] + t);
      S[k] = S[jj];
      S[jj] = t;
    }
    i = j = 0;
    g(256);
  }
  double g(int count) {
    double r = 0;
    while (count--) {
      i = 255 & (i + 1);
      const int t = S[i];
      j = 255 & (j + t);
      S[i] = S[j];
      S[j] = t;
      r = r * 256 + S[255 & (S[i] + t)];
    }
    return r;
  }
  double prng() {
    double n = g(6), d = 281474976710656.0, x = 0;   // 2^48
    while (n < 4503599627370496.0) {                  // 2^52
      n = (n + x) * 256;
      d *= 256;
      x = g(1);
    }
    while (n >= 9007199254740992.0) {                 // 2^53
      n /= 2;
      d /= 2;
      x = (double)((uint32_t)x >> 1);
    }
    return (n + x) / d;
  }
};

// A UTF-8 string as UTF-16 code units (JavaScript's string of the same text).
std::vector<uint16_t> utf16_units(const char* s) {
  std::vector<uint16_t> u;
  const unsigned char* p = (const unsigned char*)s;
  while (p && *p) {
    uint32_t c = *p++;
    int more = c >= 0xF0 ? 3 : c >= 0xE0 ? 2 : c >= 0xC0 ? 1 : 0;
    if (more) c &= (0x3F >> more);
    bool ok = c < 0x80 || more > 0;
    for (int k = 0; k < more && ok; ++k) {
      if ((*p & 0xC0) != 0x80) ok = false;
      else c = (c << 6) | (*p++ & 0x3F);
    }
    if (!ok || c > 0x10FFFF || (c >= 0xD800 && c < 0xE000)) { u.push_back(0xFFFD); continue; }
    if (c >= 0x10000) {
      u.push_back((uint16_t)(0xD800 + ((c - 0x10000) >> 10)));
      u.push_back((uint16_t)(0xDC00 + ((c - 0x10000) & 0x3FF)));
    } else {
      u.push_back((uint16_t)c);
    }
  }
  return u;
}

// lowbias32 (build-nearfield-slots.vert:130-135).
inline uint32_t lowbias32(uint32_t h) {
  h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
  return h;
}
// hashValue (build-nearfield-slots.vert:139-140).
inline float peel_hash(uint32_t index, uint32_t seed_bits) {
  uint32_t h = lowbias32(index ^ seed_bits);
  float v = ((float)(h >> 8u) + 0.5f) / 16777216.0f;
  return 0.001f + v * 0.998f;
}
inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// Portable sincos: Cody-Waite reduction of a by pi/2 in FP64 with a 30+30+53
// bit split of pi/2 (k*P1, k*P2 exact for |k| < 2^23), then Taylor series of
// sin/cos on [-pi/4, pi/4] to degree 15/16, rounded to f32.
void portable_sincos(float af, float* s_out, float* c_out) {
  const double P1 = 0x1.921fb54000000p+0, P2 = 0x1.10b4611800000p-30, P3 = 0x1.313198a2e0370p-61;
  const double TWO_OVER_PI = 0.6366197723675814;
  double a = (double)af;
  double k = std::nearbyint(a * TWO_OVER_PI);
  double r = ((a - k * P1) - k * P2) - k * P3;
  double r2 = r * r;
  // sin r = r(1 - r2/3! + r2^2/5! - ...), cos r = 1 - r2/2! + ...
  double sp = -1.0 / 1307674368000.0;               // -1/15!
  sp = sp * r2 + 1.0 / 6227020800.0;                 //  1/13!
  sp = sp * r2 - 1.0 / 39916800.0;                   // -1/11!
  sp = sp * r2 + 1.0 / 362880.0;                     //  1/9!
  sp = sp * r2 - 1.0 / 5040.0;                       // -1/7!
  sp = sp * r2 + 1.0 / 120.0;                        //  1/5!
  sp = sp * r2 - 1.0 / 6.0;                          // -1/3!
  double sn = r + r * (r2 * sp);
  double cp = 1.0 / 20922789888000.0;                //  1/16!
  cp = cp * r2 - 1.0 / 87178291200.0;                // -1/14!
  cp = cp * r2 + 1.0 / 479001600.0;                  //  1/12!
  cp = cp * r2 - 1.0 / 3628800.0;                    // -1/10!
  cp = cp * r2 + 1.0 / 40320.0;                      //  1/8!
  cp = cp * r2 - 1.0 / 720.0;                        // -1/6!
  cp = cp * r2 + 1.0 / 24.0;                         //  1/4!
  cp = cp * r2 - 0.5;                                // -1/2!
  double cs = 1.0 + r2 * cp;
  long long q = (long long)k & 3;
  double s, c;
  switch (q) {
    case 0: s = sn; c = cs; break;
    case 1: s = cs; c = -sn; break;
    case 2: s = -sn; c = -cs; break;
    default: s = -cs; c = sn; break;
  }
  *s_out = (float)s;
  *c_out = (float)c;
}

int ceil_log2_u64(uint64_t v) { int e = 0; while ((1ull << e) < v) ++e; return e; }

// Exact cell sums in units of 2^-F (see header).
struct Fixed {
  int F = 0;
  float bound = 0.f;   // saturation bound B (power of two)
  float scale = 1.f;   // 2^F
  float inv = 1.f;     // 2^-F
  void setup(uint64_t n_points, float space) {
    // B = smallest power of two >= 2*S; F = 62 - ceil(log2 N) - log2 B so that
    // N * B * 2^F <= 2^62.
    int lb = 0;
    while (std::ldexp(1.0, lb) < 2.0 * (double)space) ++lb;
    int ln = ceil_log2_u64(n_points < 1 ? 1 : n_points);
    F = 62 - ln - lb;
    if (F > 60) F = 60;
    bound = (float)std::ldexp(1.0, lb);
    scale = std::ldexp(1.0f, F);
    inv = std::ldexp(1.0f, -F);
  }
  int64_t to(float x) const {
    float xs = gclamp(x, -bound, bound);
    return (int64_t)std::llrint(xs * scale);
  }
  float from(int64_t v) const { return (float)v * inv; }
};

struct CellRec { float cx, cy, count; int nslot; };

constexpr int kSlots = 8;                  // NEAR_FIELD_SLOTS (ForceManyBody/index.ts:35)
constexpr int kMaxGrid = 512;              // MAX_GRID_SIZE (ForceManyBody/index.ts:19)
constexpr double kAlphaMin = 0.001;        // ALPHA_MIN (Store/index.ts:8)
constexpr float kOffsets[4][2] = {{0.f, 0.f}, {0.5f, 0.f}, {0.f, 0.5f}, {0.5f, 0.5f}};  // ForceCollision/index.ts:19-24

struct Csr {
  std::vector<uint32_t> rowptr;   // N+1
  std::vector<uint32_t> col;      // connected point
  std::vector<float> rnd;         // randomDistance draw (ForceLink/index.ts:76)
  std::vector<float> bias;        // ForceLink/index.ts:61-65
  std::vector<float> strength;    // ForceLink/index.ts:66-73
  uint32_t max_degree = 0;
};

}  // namespace

struct orc_engine {
  cgl_config cfg{};
  bool destroyed = false;
  std::string err;
  int sum_mode = 0;        // 0 exact (engine definition), 1 sequential f32 blending

  // staged input (copied at set_*, applied at render)
  bool have_pos_input = false, have_link_input = false, have_strength = false, have_sizes = false;
  bool has_strength = false;   // applied: linkStrength length matched linksNumber (GraphData/index.ts:408-418)
  std::vector<float> in_pos, in_links, in_strength, in_sizes;
  bool pinned_set = false;
  std::vector<double> pinned_input;
  bool pos_dirty = false, links_dirty = false, sizes_dirty = false;
  bool skip_rescale = false;       // Points.shouldSkipRescale

  // applied data
  uint64_t N = 0, E = 0;           // pointsNumber, linksNumber
  std::vector<float> data_pos;     // applied input positions (for absence)
  std::vector<float> data_links;
  std::vector<float> data_strength;
  std::vector<float> data_sizes;
  bool has_data_sizes = false;
  uint32_t T = 0, W = 0;           // pointsTextureSize, linksTextureSize
  std::vector<float> pos;          // 2N current positions
  std::vector<uint8_t> absent, pinned;
  std::vector<float> jitter;       // 2N
  Csr csr_in, csr_out;
  bool mb_ready = false;           // ForceManyBody.create ran for this point set
  int Gf = 0, L = 0;
  Fixed fx;

  // collision
  bool collision_ready = false;
  int cgrid = 0;
  float ccell = 0.f;

  // clusters (Clusters/index.ts): staged input, applied data
  bool have_clusters = false, have_cluster_pos = false, have_cluster_strength = false;
  std::vector<float> in_clusters, in_cluster_pos, in_cluster_strength;
  bool clusters_dirty = false;
  bool point_clusters = false;     // GraphData.pointClusters defined (length == N)
  bool cluster_positions = false;  // GraphData.clusterPositions defined
  uint32_t K = 0;                  // clusterCount
  std::vector<uint32_t> cluster_of;   // N, kNoCluster when unclustered
  std::vector<float> cluster_coeff;   // N, clusterForceCoefficient (default 1)
  std::vector<float> cluster_custom;  // 2K, -1 where undefined

  // interaction: Store.mousePosition, Graph.isRightClickMouse, the dragged point
  double mouse_x = 0, mouse_y = 0;
  bool right_button = false;
  int64_t drag_index = -1;

  // simulation state (Store)
  double adjusted_space = 4096;
  double alpha = 1.0;
  double progress = 0.0;
  bool running = false;
  uint64_t rng_seed = 0, rng_ctr = 0;   // counter stream seed; draws so far (both streams)
  bool counter_stream = false;
  Arc4Seed arc;                          // the reference's stream
  std::string seed_text;
  uint64_t tick = 0;

  // retained from the last many-body pass (test hooks)
  std::vector<std::vector<CellRec>> levels;
  std::vector<int32_t> slots;      // Gf^2 * 8

  // Store.getRandomFloat(min, max) = random.float(min, max)
  double rnd(double mn, double mx) {
    const double u = counter_stream ? splitmix_unit(rng_seed, rng_ctr) : arc.prng();
    ++rng_ctr;
    return u * (mx - mn) + mn;
  }
};

namespace {

void adjust_space_size(orc_engine* e) {
  // Store.adjustSpaceSize (Store/index.ts:209-233)
  double s = e->cfg.space_size;
  if (!(s > 0) || !std::isfinite(s)) s = 4096;
  if (s < 2) s = 2;
  double m = e->cfg.max_texture_dimension;
  if (m > 0 && std::isfinite(m) && m >= 2) {
    if (s >= m) s = std::max(m / 2, 2.0);
  }
  e->adjusted_space = s;
}

bool is_point_index(double v, uint64_t n) {
  // GraphData.isPointIndex (GraphData/index.ts:286-289)
  return std::isfinite(v) && v == std::floor(v) && v >= 0 && v < (double)n;
}

void build_csr(orc_engine* e, bool incoming, Csr& c, const std::vector<uint32_t>& deg) {
  // ForceLink.create (ForceLink/index.ts:40-83).  INCOMING walks
  // sourceIndexToTargetIndices, OUTGOING targetIndexToSourceIndices (:49);
  // both lists are in link-index order (GraphData/index.ts:534-547).
  const uint64_t N = e->N;
  c.rowptr.assign(N + 1, 0);
  std::vector<uint32_t> owner, other, lidx;
  for (uint64_t i = 0; i < e->E; ++i) {
    double s = e->data_links[2 * i], t = e->data_links[2 * i + 1];
    if (!is_point_index(s, N) || !is_point_index(t, N)) continue;
    uint32_t si = (uint32_t)s, ti = (uint32_t)t;
    uint32_t p = incoming ? si : ti, q = incoming ? ti : si;
    c.rowptr[p + 1]++;
    owner.push_back(p); other.push_back(q); lidx.push_back((uint32_t)i);
  }
  c.max_degree = 0;
  for (uint64_t p = 0; p < N; ++p) {
    c.max_degree = std::max(c.max_degree, c.rowptr[p + 1]);
    c.rowptr[p + 1] += c.rowptr[p];
  }
  size_t M = owner.size();
  c.col.assign(M, 0); c.rnd.assign(M, 0); c.bias.assign(M, 0); c.strength.assign(M, 0);
  std::vector<uint32_t> cur(c.rowptr.begin(), c.rowptr.end() - 1);
  std::vector<uint32_t> slot_link(M);
  for (size_t k = 0; k < M; ++k) {
    uint32_t at = cur[owner[k]]++;
    c.col[at] = other[k];
    slot_link[at] = lidx[k];
  }
  for (uint64_t p = 0; p < N; ++p) {
    for (uint32_t at = c.rowptr[p]; at < c.rowptr[p + 1]; ++at) {
      uint32_t q = c.col[at];
      double degree = deg[q], connected = deg[p];
      double sum = degree + connected;
      double bias = sum != 0 ? degree / sum : 0.5;
      double mind = std::min(degree, connected);
      double strength;
      bool use_input = e->has_strength;
      double si = use_input ? (double)e->data_strength[slot_link[at]] : 0.0;
      if (!use_input || !std::isfinite(si) || si < 0) strength = 1.0 / std::max(mind, 1.0);
      else strength = si;
      strength = std::sqrt(strength);
      c.bias[at] = (float)bias;
      c.strength[at] = (float)strength;
      c.rnd[at] = (float)e->rnd(0, 1);
    }
  }
}

// Math.min / Math.max (NaN if either is NaN; -0 < +0).
double js_min(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return NAN;
  if (a == b) return std::signbit(a) ? a : b;
  return a < b ? a : b;
}
double js_max(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return NAN;
  if (a == b) return std::signbit(a) ? b : a;
  return a > b ? a : b;
}

// Points.rescaleInitialNodePositions (Points/index.ts:3134-3218): FP64 as in
// JavaScript, written back into the Float32Array (rounded to f32).
void rescale_initial_positions(std::vector<float>& points, double spaceSize) {
  if (spaceSize == 0 || std::isnan(spaceSize)) return;   // `!spaceSize`
  const size_t pointsNumber = points.size() / 2;
  auto absent = [&](size_t i) { return std::isnan(points[2 * i]) || std::isnan(points[2 * i + 1]); };
  double minX = INFINITY, maxX = -INFINITY, minY = INFINITY, maxY = -INFINITY;
  for (size_t i = 0; i < pointsNumber; ++i) {
    if (absent(i)) continue;
    const double x = points[2 * i], y = points[2 * i + 1];
    minX = js_min(minX, x);
    maxX = js_max(maxX, x);
    minY = js_min(minY, y);
    maxY = js_max(maxY, y);
  }
  if (!std::isfinite(minX)) return;
  const double w = maxX - minX;
  const double h = maxY - minY;
  const double range = js_max(w, h);
  if (range == 0) {
    const double center = spaceSize / 2;
    for (size_t i = 0; i < pointsNumber; ++i) {
      if (absent(i)) continue;
      points[2 * i] = (float)((double)points[2 * i] - minX + center);
      points[2 * i + 1] = (float)((double)points[2 * i + 1] - minY + center);
    }
    return;
  }
  if (range > spaceSize) return;
  const double densityThreshold = spaceSize * spaceSize * 0.001;
  const double effectiveSpaceSize = (double)pointsNumber > densityThreshold
                                        ? spaceSize * js_max(1.2, std::sqrt((double)pointsNumber) / spaceSize)
                                        : spaceSize * 0.1;
  const double scaleFactor = effectiveSpaceSize / range;
  const double centerOffset = (spaceSize - effectiveSpaceSize) / 2;
  const double offsetX = ((range - w) / 2) * scaleFactor + centerOffset;
  const double offsetY = ((range - h) / 2) * scaleFactor + centerOffset;
  for (size_t i = 0; i < pointsNumber; ++i) {
    if (absent(i)) continue;
    points[2 * i] = (float)(((double)points[2 * i] - minX) * scaleFactor + offsetX);
    points[2 * i + 1] = (float)(((double)points[2 * i + 1] - minY) * scaleFactor + offsetY);
  }
}

void apply_pinned(orc_engine* e) {
  // Points.updatePinnedStatus (Points/index.ts:1264-1277)
  e->pinned.assign(e->N, 0);
  if (!e->pinned_set) return;
  for (double v : e->pinned_input) {
    if (v >= 0 && v < (double)e->N && v == std::floor(v)) e->pinned[(size_t)v] = 1;
  }
}

float resolved_size(orc_engine* e, uint64_t i) {
  // GraphData.getResolvedPointSize (GraphData/index.ts:189-194); EXIT_DEFAULT_SIZE = 0
  if (e->has_data_sizes && i < e->data_sizes.size()) {
    float r = e->data_sizes[i];
    if (!std::isnan(r)) return r;
  }
  if (e->absent[i]) return 0.f;
  return (float)e->cfg.point_default_size;
}

void collision_create(orc_engine* e) {
  // ForceCollision.create (ForceCollision/index.ts:61-95)
  double maxSize = e->cfg.point_default_size;
  if (e->has_data_sizes)
    for (uint64_t i = 0; i < e->N; ++i) maxSize = std::max(maxSize, (double)resolved_size(e, i));
  double cr = std::isnan(e->cfg.simulation_collision_radius) ? 0 : e->cfg.simulation_collision_radius;
  double pad = e->cfg.simulation_collision_padding;
  double effR = (cr > 0 ? cr : maxSize * 0.5) + pad;
  double cell = std::max(effR * 2, 8.0);
  int grid = (int)std::min(512.0, std::max(1.0, std::floor(e->adjusted_space / cell)));
  e->cgrid = grid;
  e->ccell = (float)(e->adjusted_space / grid);
  e->collision_ready = true;
}

// ------------------------------------------------------------------ tick --
void update_point(const orc_engine* e, size_t i, const float* prev, float vx, float vy, float* out) {
  // update-position.frag:26-59
  float px = prev[2 * i], py = prev[2 * i + 1];
  if (e->pinned[i] || e->absent[i]) { out[2 * i] = px; out[2 * i + 1] = py; return; }
  const float fr = (float)e->cfg.simulation_friction;
  const float S = (float)e->adjusted_space;
  vx = vx * fr; vy = vy * fr;
  px = px + vx; py = py + vy;
  out[2 * i] = gclamp(px, 0.f, S);
  out[2 * i + 1] = gclamp(py, 0.f, S);
}

void run_gravity(orc_engine* e, float a) {
  // force-gravity.frag:24-40 then update
  std::vector<float> prev = e->pos;
  const float g = (float)e->cfg.simulation_gravity;
  const float S = (float)e->adjusted_space;
  const float c = S * 0.5f;
  const int64_t N = (int64_t)e->N;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    float dx = c - prev[2 * i], dy = c - prev[2 * i + 1];
    float dist = sqrtf(dx * dx + dy * dy);
    float vx = 0.f, vy = 0.f;
    if (dist > 0.f) {
      float add = a * g * dist * 0.1f;
      vx = vx + add * (dx / dist);
      vy = vy + add * (dy / dist);
    }
    update_point(e, i, prev.data(), vx, vy, e->pos.data());
  }
}

void run_center(orc_engine* e, float a) {
  // ForceCenter.run (ForceCenter/index.ts:149-199): centroid over live points
  // (calculate-centermass.vert:18-28), force-center.frag:22-36, update.
  std::vector<float> prev = e->pos;
  const int64_t N = (int64_t)e->N;
  float sx, sy, cnt;
  if (e->sum_mode == 0) {
    int64_t ax = 0, ay = 0, n = 0;
#pragma omp parallel for reduction(+ : ax, ay, n) schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      if (e->absent[i]) continue;
      ax += e->fx.to(prev[2 * i]); ay += e->fx.to(prev[2 * i + 1]); n += 1;
    }
    sx = e->fx.from(ax); sy = e->fx.from(ay); cnt = (float)n;
  } else {
    sx = 0.f; sy = 0.f; cnt = 0.f;
    for (int64_t i = 0; i < N; ++i) {
      if (e->absent[i]) continue;
      sx = sx + prev[2 * i]; sy = sy + prev[2 * i + 1]; cnt = cnt + 1.0f;
    }
  }
  const float cf = (float)e->cfg.simulation_center;
  float cmx = sx / cnt, cmy = sy / cnt;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    float dx = cmx - prev[2 * i], dy = cmy - prev[2 * i + 1];
    float dist = sqrtf(dx * dx + dy * dy);
    float vx = 0.f, vy = 0.f;
    if (dist > 0.f) {
      float add = a * cf * dist * 0.01f;
      vx = vx + add * (dx / dist);
      vy = vy + add * (dy / dist);
    }
    update_point(e, i, prev.data(), vx, vy, e->pos.data());
  }
}

template <typename R>
inline R rsqrt_op(R x) { return std::sqrt(x); }

template <typename R>
inline void cell_velocity(R cx, R cy, R count, R px, R py, R k, R& vx, R& vy) {
  // force-level.frag:43-56; (cx, cy) = centermass.rg / centermass.b
  if (count <= R(0)) { vx = vx + R(0); vy = vy + R(0); return; }
  R dx = px - cx, dy = py - cy;
  R l = dx * dx + dy * dy;
  if (l <= R(0)) { vx = vx + R(0); vy = vy + R(0); return; }
  R len = rsqrt_op(l);                       // length(distVector)
  R s = l < R(1) ? rsqrt_op(len) : len;      // sqrt(l) after l = sqrt(1 * l) when l < 1
  R add = k * count / s;
  R inv = R(1) / len;                        // normalize(v) = v * (1 / length(v))
  vx = vx + add * (dx * inv);
  vy = vy + add * (dy * inv);
}

template <typename R>
inline void pair_velocity(R px, R py, R ox, R oy, R rx, R ry, R k, R& sx, R& sy) {
  // force-nearfield.frag:64-78
  R dx = px - ox, dy = py - oy;
  R l = dx * dx + dy * dy;
  if (l <= R(0)) {
    dx = rx; dy = ry;
    l = dx * dx + dy * dy;
    if (l <= R(0)) { sx = sx + R(0); sy = sy + R(0); return; }
  }
  R len = rsqrt_op(l);
  R s = l < R(1) ? rsqrt_op(len) : len;
  R add = k / s;
  R inv = R(1) / len;
  sx = sx + add * (dx * inv);
  sy = sy + add * (dy * inv);
}

// Cell centroids at precision R (double: exact sums divided in FP64).
struct Pyramid {
  std::vector<std::vector<CellRec>> f32;
  std::vector<std::vector<double>> f64;   // cx, cy, count per cell
};

// drawLevels (ForceManyBody/index.ts:464-502, calculate-level.vert:28-53) and
// drawNearFieldSlots (:511-559, build-nearfield-slots.vert:46-103).
void build_pyramid_and_slots(orc_engine* e, const std::vector<float>& prev, uint32_t seed_bits, bool want_f64,
                             std::vector<std::vector<double>>* f64_out) {
  const int64_t N = (int64_t)e->N;
  const int Gf = e->Gf, L = e->L;
  const float csf = (float)(e->adjusted_space / Gf);
  std::vector<int32_t> fcell(N, -1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    if (e->absent[i]) continue;
    int cx = cell_index(prev[2 * i], csf, Gf), cy = cell_index(prev[2 * i + 1], csf, Gf);
    fcell[i] = cy * Gf + cx;
  }
  e->levels.assign(L, {});
  if (f64_out) f64_out->assign(L, {});
  if (e->sum_mode == 0) {
    const size_t C = (size_t)Gf * Gf;
    std::vector<int64_t> sx(C, 0), sy(C, 0), cn(C, 0);
    for (int64_t i = 0; i < N; ++i) {
      int c = fcell[i];
      if (c < 0) continue;
      sx[c] += e->fx.to(prev[2 * i]); sy[c] += e->fx.to(prev[2 * i + 1]); cn[c] += 1;
    }
    for (int l = L - 1; l >= 0; --l) {
      int G = 4 << l;
      auto& lv = e->levels[l];
      lv.assign((size_t)G * G, CellRec{0, 0, 0, 0});
      if (want_f64) (*f64_out)[l].assign((size_t)G * G * 3, 0.0);
      for (int c = 0; c < G * G; ++c) {
        if (cn[c] > 0) {
          float cnt = (float)cn[c];
          lv[c].cx = e->fx.from(sx[c]) / cnt;
          lv[c].cy = e->fx.from(sy[c]) / cnt;
          lv[c].count = cnt;
          if (want_f64) {
            double inv = std::ldexp(1.0, -e->fx.F);
            (*f64_out)[l][3 * c] = (double)sx[c] * inv / (double)cn[c];
            (*f64_out)[l][3 * c + 1] = (double)sy[c] * inv / (double)cn[c];
            (*f64_out)[l][3 * c + 2] = (double)cn[c];
          }
        }
      }
      if (l > 0) {  // children -> parents (exact integers)
        int Gp = G / 2;
        std::vector<int64_t> qx((size_t)Gp * Gp, 0), qy((size_t)Gp * Gp, 0), qn((size_t)Gp * Gp, 0);
        for (int y = 0; y < G; ++y)
          for (int x = 0; x < G; ++x) {
            int c = y * G + x, p = (y / 2) * Gp + x / 2;
            qx[p] += sx[c]; qy[p] += sy[c]; qn[p] += cn[c];
          }
        sx.swap(qx); sy.swap(qy); cn.swap(qn);
      }
    }
  } else {
    for (int l = 0; l < L; ++l) {
      int G = 4 << l;
      float cs = (float)(e->adjusted_space / G);
      std::vector<float> sx((size_t)G * G, 0.f), sy((size_t)G * G, 0.f), cn((size_t)G * G, 0.f);
      for (int64_t i = 0; i < N; ++i) {
        if (e->absent[i]) continue;
        int cx = cell_index(prev[2 * i], cs, G), cy = cell_index(prev[2 * i + 1], cs, G);
        int c = cy * G + cx;
        sx[c] = sx[c] + prev[2 * i]; sy[c] = sy[c] + prev[2 * i + 1]; cn[c] = cn[c] + 1.0f;
      }
      auto& lv = e->levels[l];
      lv.assign((size_t)G * G, CellRec{0, 0, 0, 0});
      if (want_f64) (*f64_out)[l].assign((size_t)G * G * 3, 0.0);
      for (int c = 0; c < G * G; ++c)
        if (cn[c] > 0) {
          lv[c].cx = sx[c] / cn[c]; lv[c].cy = sy[c] / cn[c]; lv[c].count = cn[c];
          if (want_f64) {
            (*f64_out)[l][3 * c] = lv[c].cx; (*f64_out)[l][3 * c + 1] = lv[c].cy; (*f64_out)[l][3 * c + 2] = cn[c];
          }
        }
    }
  }
  // near-field slots: 8 smallest distinct hashes per finest cell
  const size_t C = (size_t)Gf * Gf;
  std::vector<uint32_t> start(C + 1, 0);
  for (int64_t i = 0; i < N; ++i) if (fcell[i] >= 0) start[fcell[i] + 1]++;
  for (size_t c = 0; c < C; ++c) start[c + 1] += start[c];
  std::vector<uint64_t> keys(start[C], 0);   // (hash bits << 32) | index
  {
    std::vector<uint32_t> cur(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < N; ++i) {
      int c = fcell[i];
      if (c < 0) continue;
      float h = peel_hash((uint32_t)i, seed_bits);
      keys[cur[c]++] = ((uint64_t)fbits(h) << 32) | (uint32_t)i;
    }
  }
  e->slots.assign(C * kSlots, -1);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t c = 0; c < (int64_t)C; ++c) {
    uint64_t* b = keys.data() + start[c];
    uint64_t* en = keys.data() + start[c + 1];
    std::sort(b, en);
    int k = 0;
    uint32_t last = 0xFFFFFFFFu;
    for (uint64_t* it = b; it != en && k < kSlots; ++it) {
      uint32_t hb = (uint32_t)(*it >> 32);
      if (k > 0 && hb == last) continue;
      e->slots[c * kSlots + k] = (int32_t)(uint32_t)(*it & 0xFFFFFFFFu);
      last = hb;
      ++k;
    }
    e->levels[L - 1][c].nslot = k;
  }
}

// drawForces (ForceManyBody/index.ts:565-638): level passes then the near
// field, for one point, at precision R.  Cell data from the f32 pyramid
// (R = float) or the f64 centroids (R = double).
template <typename R>
void manybody_point(const orc_engine* e, const std::vector<float>& prev, int64_t i, R k,
                    const std::vector<std::vector<double>>* f64, R& vx_out, R& vy_out) {
  const int Gf = e->Gf, L = e->L;
  const float csf = (float)(e->adjusted_space / Gf);
  const R px = prev[2 * i], py = prev[2 * i + 1];
  const int fcx = cell_index(prev[2 * i], csf, Gf), fcy = cell_index(prev[2 * i + 1], csf, Gf);
  auto cell = [&](int l, int c, R& cx, R& cy, R& cnt) {
    if (f64) { cx = (R)(*f64)[l][3 * c]; cy = (R)(*f64)[l][3 * c + 1]; cnt = (R)(*f64)[l][3 * c + 2]; }
    else { const CellRec& r = e->levels[l][c]; cx = r.cx; cy = r.cy; cnt = r.count; }
  };
  R vx = 0, vy = 0;  // the velocity target, cleared (index.ts:575-578)
  for (int l = 0; l < L; ++l) {
    const int G = 4 << l;
    const int sh = L - 1 - l;
    const int pcx = fcx >> sh, pcy = fcy >> sh;
    R lx = 0, ly = 0;
    if (l == 0) {  // force-level.frag:70-79
      for (int j = 0; j < G; ++j)
        for (int ii = 0; ii < G; ++ii) {
          if (std::max(std::abs(ii - pcx), std::abs(j - pcy)) <= 1) continue;
          R cx, cy, cnt; cell(l, j * G + ii, cx, cy, cnt);
          cell_velocity<R>(cx, cy, cnt, px, py, k, lx, ly);
        }
    } else {       // force-level.frag:80-95
      const int bx = (pcx / 2) * 2 - 2, by = (pcy / 2) * 2 - 2;
      for (int j = 0; j < 6; ++j)
        for (int ii = 0; ii < 6; ++ii) {
          int cx = bx + ii, cy = by + j;
          if (cx < 0 || cy < 0 || cx >= G || cy >= G) continue;
          if (std::max(std::abs(cx - pcx), std::abs(cy - pcy)) <= 1) continue;
          R ccx, ccy, cnt; cell(l, cy * G + cx, ccx, ccy, cnt);
          cell_velocity<R>(ccx, ccy, cnt, px, py, k, lx, ly);
        }
    }
    vx = vx + lx; vy = vy + ly;  // additive blend of the level pass
  }
  // force-nearfield.frag:199-263
  const R rx = e->jitter[2 * i], ry = e->jitter[2 * i + 1];
  const float self = (float)i;
  R nx = 0, ny = 0;
  const auto& fine = e->levels[L - 1];
  for (int j = -1; j <= 1; ++j)
    for (int ii = -1; ii <= 1; ++ii) {
      int cx = fcx + ii, cy = fcy + j;
      if (cx < 0 || cy < 0 || cx >= Gf || cy >= Gf) continue;
      int c = cy * Gf + cx;
      R others = (R)fine[c].count - ((ii == 0 && j == 0) ? R(1) : R(0));
      if (others <= R(0)) continue;
      R sx = 0, sy = 0, sampled = 0;
      for (int s = 0; s < kSlots; ++s) {
        int32_t idx = e->slots[(size_t)c * kSlots + s];
        if (idx < 0 || (float)idx == self) { sx = sx + R(0); sy = sy + R(0); continue; }
        sampled = sampled + R(1);
        pair_velocity<R>(px, py, prev[2 * (size_t)idx], prev[2 * (size_t)idx + 1], rx, ry, k, sx, sy);
      }
      if (sampled > R(0)) {
        R w = others / sampled;
        nx = nx + w * sx; ny = ny + w * sy;
      }
    }
  nx = nx + nx * rx; ny = ny + ny * ry;
  const R maxStep = R(2) * (R)csf;
  const R speed = rsqrt_op(nx * nx + ny * ny);
  if (speed > maxStep) { R s = maxStep / speed; nx = nx * s; ny = ny * s; }
  vx_out = vx + nx; vy_out = vy + ny;
}

void run_manybody(orc_engine* e, float a, float* vel_out = nullptr) {
  // ForceManyBody.run (ForceManyBody/index.ts:399-417), then the update.
  if (!e->mb_ready || e->N == 0) return;
  std::vector<float> prev = e->pos;
  const int64_t N = (int64_t)e->N;
  const float seed = (float)e->rnd(0, 1);   // ForceManyBody/index.ts:521
  build_pyramid_and_slots(e, prev, fbits(seed), false, nullptr);
  const float k = a * (float)e->cfg.simulation_repulsion;
  std::vector<float> out(prev);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < N; ++i) {
    if (e->absent[i]) continue;
    float vx, vy;
    manybody_point<float>(e, prev, i, k, nullptr, vx, vy);
    if (vel_out) { vel_out[2 * i] = vx; vel_out[2 * i + 1] = vy; }
    update_point(e, (size_t)i, prev.data(), vx, vy, out.data());
  }
  e->pos.swap(out);
}

void run_links(orc_engine* e, const Csr& c, float a) {
  // ForceLink.run (ForceLink/index.ts:221-263), force-spring.ts:38-96, update
  std::vector<float> prev = e->pos;
  const int64_t N = (int64_t)e->N;
  const float spring = (float)e->cfg.simulation_link_spring;
  const float dist = (float)e->cfg.simulation_link_distance;
  const float r0 = (float)e->cfg.simulation_link_dist_random_variation_range[0];
  const float r1 = (float)e->cfg.simulation_link_dist_random_variation_range[1];
  const float sa = spring * a;
  const float span = r1 - r0;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t p = 0; p < N; ++p) {
    float vx = 0.f, vy = 0.f;
    const float px = prev[2 * p], py = prev[2 * p + 1];
    for (uint32_t at = c.rowptr[p]; at < c.rowptr[p + 1]; ++at) {
      uint32_t q = c.col[at];
      float d = c.rnd[at] * span + r0;
      d = d * dist;
      if (e->absent[q]) continue;
      float x = prev[2 * (size_t)q] - (px + vx);
      float y = prev[2 * (size_t)q + 1] - (py + vy);
      float l = sqrtf(x * x + y * y);
      l = gmax(l, d * 0.99f);
      l = (l - d) / l;
      l = l * sa;
      l = l * c.strength[at];
      l = l * c.bias[at];
      x = x * l; y = y * l;
      vx = vx + x; vy = vy + y;
    }
    update_point(e, (size_t)p, prev.data(), vx, vy, e->pos.data());
  }
}

void run_collision(orc_engine* e, float a) {
  // ForceCollision.run (ForceCollision/index.ts:264-345), build-grid.vert:28-62,
  // force-collision-spatial.frag:103-168, update
  if (!e->collision_ready) collision_create(e);
  std::vector<float> prev = e->pos;
  const int64_t N = (int64_t)e->N;
  const int G = e->cgrid;
  const float cs = e->ccell;
  const float Gm1 = (float)G - 1.0f;
  std::vector<float> size(N);
  for (int64_t i = 0; i < N; ++i) size[i] = resolved_size(e, (uint64_t)i);
  struct GridCell { float sx, sy, ss, n; };
  std::vector<std::vector<GridCell>> grids(4, std::vector<GridCell>((size_t)G * G, GridCell{0, 0, 0, 0}));
  auto bin = [&](float p, float o) {
    float off = p + o * cs;
    float c = gclamp(floorf(off / cs), 0.f, Gm1);
    if (!(c == c)) c = 0.f;
    return c;
  };
  for (int g = 0; g < 4; ++g) {
    const float ox = kOffsets[g][0], oy = kOffsets[g][1];
    if (e->sum_mode == 0) {
      std::vector<int64_t> ax((size_t)G * G, 0), ay((size_t)G * G, 0), as((size_t)G * G, 0), an((size_t)G * G, 0);
      for (int64_t i = 0; i < N; ++i) {
        if (e->absent[i]) continue;
        int c = (int)bin(prev[2 * i + 1], oy) * G + (int)bin(prev[2 * i], ox);
        ax[c] += e->fx.to(prev[2 * i]); ay[c] += e->fx.to(prev[2 * i + 1]);
        as[c] += e->fx.to(size[i]); an[c] += 1;
      }
      for (size_t c = 0; c < (size_t)G * G; ++c)
        grids[g][c] = GridCell{e->fx.from(ax[c]), e->fx.from(ay[c]), e->fx.from(as[c]), (float)an[c]};
    } else {
      for (int64_t i = 0; i < N; ++i) {
        if (e->absent[i]) continue;
        int c = (int)bin(prev[2 * i + 1], oy) * G + (int)bin(prev[2 * i], ox);
        GridCell& gc = grids[g][c];
        gc.sx = gc.sx + prev[2 * i]; gc.sy = gc.sy + prev[2 * i + 1]; gc.ss = gc.ss + size[i]; gc.n = gc.n + 1.0f;
      }
    }
  }
  const float cr = std::isnan(e->cfg.simulation_collision_radius) ? 0.f : (float)e->cfg.simulation_collision_radius;
  const float pad = (float)e->cfg.simulation_collision_padding;
  const float str = (float)e->cfg.simulation_collision;
  const float Nf = (float)N;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < N; ++i) {
    const float px = prev[2 * i], py = prev[2 * i + 1];
    float vx = 0.f, vy = 0.f;
    const float cur = (float)i;
    if (!(cur < 0.f || cur >= Nf)) {
      const float csz = size[i];
      const float R = (cr > 0.f ? cr : csz * 0.5f) + pad;
      for (int g = 0; g < 4; ++g) {
        const float ox = kOffsets[g][0], oy = kOffsets[g][1];
        float offx = px + ox * cs, offy = py + oy * cs;
        float mx = gclamp(floorf(offx / cs), 0.f, Gm1);
        float my = gclamp(floorf(offy / cs), 0.f, Gm1);
        if (!(mx == mx)) mx = 0.f;
        if (!(my == my)) my = 0.f;
        float total = 0.f, gx = 0.f, gy = 0.f;
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy) {
            float ncx = mx + (float)dx, ncy = my + (float)dy;
            if (ncx < 0.f || ncx >= (float)G || ncy < 0.f || ncy >= (float)G) continue;
            const GridCell& cd = grids[g][(size_t)((int)ncy * G + (int)ncx)];
            float cnt = cd.n;
            if (cnt < 0.5f) continue;
            float ec = cnt, spx = cd.sx, spy = cd.sy, ss = cd.ss;
            if (dx == 0 && dy == 0) { ec = cnt - 1.0f; spx = spx - px; spy = spy - py; ss = ss - csz; }
            if (ec < 0.5f) continue;
            total = total + ec;
            float avx = spx / ec, avy = spy / ec;
            float avs = ss / ec;
            float oR = (cr > 0.f ? cr : avs * 0.5f) + pad;
            float comb = R + oR;
            float ddx = px - avx, ddy = py - avy;
            float d = sqrtf(ddx * ddx + ddy * ddy);
            if (d < comb && d > 0.001f) {
              float ov = (comb - d) / comb;
              float soft = sqrtf(ov) * comb * 0.5f;
              float dirx = ddx / d, diry = ddy / d;
              float f = a * str * soft * 0.25f * ec;
              f = gmin(f, comb * 0.5f);
              gx = gx + f * dirx; gy = gy + f * diry;
            } else if (d <= 0.001f && ec > 0.f) {
              float ang = cur * 0.618033988749895f;
              float f = gmin(a * str * comb * 0.1f, comb * 0.3f);
              float sn, cn;
              portable_sincos(ang, &sn, &cn);
              float fe = f * ec;
              gx = gx + fe * cn; gy = gy + fe * sn;
            }
          }
        if (total > 2.0f) { float dmp = 2.0f / total; gx = gx * dmp; gy = gy * dmp; }
        float maxC = R * 0.1f;
        float corr = sqrtf(gx * gx + gy * gy);
        if (corr > maxC) { float s = maxC / corr; gx = gx * s; gy = gy * s; }
        vx = vx + gx; vy = vy + gy;
      }
    }
    update_point(e, (size_t)i, prev.data(), vx, vy, e->pos.data());
  }
}

constexpr uint32_t kNoCluster = 0xFFFFFFFFu;

// Clusters.create (Clusters/index.ts:54-100) on the applied data
// (GraphData.updateClusters, GraphData/index.ts:420-441).
void clusters_create(orc_engine* e) {
  const uint64_t N = e->N;
  e->point_clusters = e->have_clusters && e->in_clusters.size() == N && N > 0;
  e->cluster_positions = e->have_cluster_pos && N > 0;
  const bool strength = e->have_cluster_strength && e->in_cluster_strength.size() == N;
  e->cluster_of.assign(N, kNoCluster);
  e->cluster_coeff.assign(N, 1.0f);
  // clusterCount = max index + 1 over defined non-negative indices (:66-69)
  uint32_t maxc = 0;
  if (e->point_clusters) {
    for (uint64_t i = 0; i < N; ++i) {
      const float v = e->in_clusters[i];
      // a non-negative integer; NaN (undefined), negatives, non-integers and
      // infinities leave the point unclustered
      if (!(v >= 0.f) || !std::isfinite(v) || v != std::floor(v) || v >= 4294967295.f) continue;
      e->cluster_of[i] = (uint32_t)v;
      maxc = std::max(maxc, (uint32_t)v);
    }
  }
  e->K = maxc + 1;
  if (strength)
    for (uint64_t i = 0; i < N; ++i) e->cluster_coeff[i] = e->in_cluster_strength[i];
  // clusterPositions texel c = (cp[2c] ?? -1, cp[2c+1] ?? -1) (:77-82)
  e->cluster_custom.assign(2 * (size_t)e->K, -1.0f);
  if (e->cluster_positions)
    for (size_t j = 0; j < 2 * (size_t)e->K && j < e->in_cluster_pos.size(); ++j)
      if (!std::isnan(e->in_cluster_pos[j])) e->cluster_custom[j] = e->in_cluster_pos[j];
}

// calculate-centermass.vert:22-52: per cluster, the sums of the live clustered
// points' positions and their count (additive blending: exact integer sums
// rounded once to f32, or f32 in index order in sum mode 1).
void cluster_sums(const orc_engine* e, const std::vector<float>& p, std::vector<float>& sx, std::vector<float>& sy,
                  std::vector<float>& sn) {
  const size_t K = e->K;
  sx.assign(K, 0.f); sy.assign(K, 0.f); sn.assign(K, 0.f);
  if (!e->point_clusters) return;
  if (e->sum_mode == 0) {
    std::vector<int64_t> ax(K, 0), ay(K, 0), an(K, 0);
    for (uint64_t i = 0; i < e->N; ++i) {
      const uint32_t c = e->cluster_of[i];
      if (e->absent[i] || c == kNoCluster) continue;
      ax[c] += e->fx.to(p[2 * i]); ay[c] += e->fx.to(p[2 * i + 1]); an[c] += 1;
    }
    for (size_t c = 0; c < K; ++c) { sx[c] = e->fx.from(ax[c]); sy[c] = e->fx.from(ay[c]); sn[c] = (float)an[c]; }
  } else {
    for (uint64_t i = 0; i < e->N; ++i) {
      const uint32_t c = e->cluster_of[i];
      if (e->absent[i] || c == kNoCluster) continue;
      sx[c] = sx[c] + p[2 * i]; sy[c] = sy[c] + p[2 * i + 1]; sn[c] = sn[c] + 1.0f;
    }
  }
}

void run_clusters(orc_engine* e, float a) {
  // Clusters.run (Clusters/index.ts:426-469): centre of mass, force-cluster.frag:28-53, update
  std::vector<float> prev = e->pos;
  const int64_t N = (int64_t)e->N;
  std::vector<float> sx, sy, sn;
  cluster_sums(e, prev, sx, sy, sn);
  const float cc = (float)e->cfg.simulation_cluster;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    float vx = 0.f, vy = 0.f;
    const uint32_t c = e->cluster_of[i];
    if (c != kNoCluster) {
      float tx = e->cluster_custom[2 * (size_t)c], ty = e->cluster_custom[2 * (size_t)c + 1];
      if (tx < 0.f || ty < 0.f) { tx = sx[c] / sn[c]; ty = sy[c] / sn[c]; }
      const float dx = tx - prev[2 * i], dy = ty - prev[2 * i + 1];
      const float dist = sqrtf(dx * dx + dy * dy);
      if (dist > 0.f) {
        const float add = a * dist * cc * e->cluster_coeff[i];
        const float inv = 1.0f / dist;   // normalize(v) = v * (1 / length(v))
        vx = 0.f + add * (dx * inv);
        vy = 0.f + add * (dy * inv);
      }
    }
    update_point(e, (size_t)i, prev.data(), vx, vy, e->pos.data());
  }
}

bool mouse_active(const orc_engine* e) { return e->right_button && e->cfg.enable_right_click_repulsion; }

void run_mouse(orc_engine* e) {
  // ForceMouse.run, force-mouse.frag:23-38, then the update.  cos/sin of
  // atan(d.y, d.x) = d / |d|; atan(0, 0) = 0 gives (1, 0).
  std::vector<float> prev = e->pos;
  const float mx = (float)e->mouse_x, my = (float)e->mouse_y;
  const float rep = (float)e->cfg.simulation_repulsion_from_mouse;
  const int64_t N = (int64_t)e->N;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    const float dx = mx - prev[2 * i], dy = my - prev[2 * i + 1];
    const float r = sqrtf(dx * dx + dy * dy);
    const float dist = gmax(r, 10.0f);
    const float add = 100.0f * rep / (dist * dist);
    float cx = 1.f, cy = 0.f;
    if (r > 0.f) { cx = dx / r; cy = dy / r; }
    update_point(e, (size_t)i, prev.data(), 0.f - add * cx, 0.f - add * cy, e->pos.data());
  }
}

void run_drag(orc_engine* e) {
  // Points.drag, drag-point.frag:22-31
  if (e->drag_index >= 0 && (uint64_t)e->drag_index < e->N) {
    e->pos[2 * (size_t)e->drag_index] = (float)e->mouse_x;
    e->pos[2 * (size_t)e->drag_index + 1] = (float)e->mouse_y;
  }
}

void run_tick(orc_engine* e) {
  // Graph.runSimulationStep (src/index.ts:2006-2099)
  if (mouse_active(e)) run_mouse(e);   // :2011-2016
  const uint32_t m = e->cfg.stage_mask;
  const float a = (float)e->alpha;
  if (e->cfg.simulation_gravity != 0 && (m & CGL_STAGE_GRAVITY)) run_gravity(e, a);
  if (e->cfg.simulation_center != 0 && (m & CGL_STAGE_CENTER)) run_center(e, a);
  if (m & CGL_STAGE_MANYBODY) run_manybody(e, a);
  if (e->W > 0) {
    if (m & CGL_STAGE_LINK_IN) run_links(e, e->csr_in, a);
    if (m & CGL_STAGE_LINK_OUT) run_links(e, e->csr_out, a);
  }
  if ((e->point_clusters || e->cluster_positions) && (m & CGL_STAGE_CLUSTERS)) run_clusters(e, a);
  if (e->cfg.simulation_collision != 0 && (m & CGL_STAGE_COLLISION)) run_collision(e, a);
  // Store.addAlpha (Store/index.ts:328-332), progress (src/index.ts:2088)
  e->alpha += (0 - e->alpha) * (1 - std::pow(kAlphaMin, 1 / e->cfg.simulation_decay));
  if (mouse_active(e)) e->alpha = std::max(e->alpha, 0.1);   // :2083-2085
  e->progress = std::sqrt(std::min(1.0, kAlphaMin / e->alpha));
  e->tick++;
}

// One animation frame (src/index.ts:2161-2175, renderFrame :2237-2317).
void run_frame(orc_engine* e, uint32_t* ticks) {
  if (e->alpha < kAlphaMin && e->running) { e->running = false; e->progress = 1; }
  if (e->cfg.enable_simulation && e->T) {
    if (e->running) { run_tick(e); ++*ticks; }
    else if (mouse_active(e)) run_mouse(e);
  }
  if (e->cfg.enable_drag) run_drag(e);
}

}  // namespace

// ================================================================ C API ====
extern "C" {

orc_engine* orc_create(const cgl_config* cfg) {
  orc_engine* e = new orc_engine();
  e->cfg = *cfg;
  // Store.addRandomSeed (Store/index.ts:196-198, src/index.ts:452)
  if (cfg->has_random_seed) e->rng_seed = cfg->random_seed;
  else { std::random_device rd; e->rng_seed = ((uint64_t)rd() << 32) ^ rd(); }
  e->counter_stream = cfg->random_stream == CGL_RANDOM_COUNTER;
  if (cfg->has_random_seed && cfg->random_seed_text) e->seed_text = cfg->random_seed_text;
  else e->seed_text = std::to_string(e->rng_seed);   // String(n) of an integer seed
  e->cfg.random_seed_text = (cfg->has_random_seed && cfg->random_seed_text) ? e->seed_text.c_str() : nullptr;
  e->arc.seed(utf16_units(e->seed_text.c_str()));
  adjust_space_size(e);
  return e;
}

void orc_destroy(orc_engine* e) { delete e; }

void orc_set_sum_mode(orc_engine* e, int mode) { e->sum_mode = mode; }

int orc_set_config(orc_engine* e, const cgl_config* cfg) {
  cgl_config prev = e->cfg;
  e->cfg = *cfg;
  e->cfg.has_random_seed = prev.has_random_seed;   // init-only (src/index.ts:1720-1724)
  e->cfg.random_seed = prev.random_seed;
  e->cfg.random_seed_text = prev.random_seed_text;
  e->cfg.random_stream = prev.random_stream;
  if (prev.space_size != e->cfg.space_size) {
    adjust_space_size(e);
    e->collision_ready = false;
    if (e->N) e->fx.setup(e->N, (float)e->adjusted_space);
    e->alpha = e->running ? e->alpha : 0;             // update(running ? alpha : 0), :1844-1851
  }
  return 0;
}

int orc_set_point_positions_ex(orc_engine* e, const float* xy, uint64_t n, int dont_rescale) {
  int st = 0;
  if (n % 2) { n -= 1; st = CGL_WARNING; }
  e->in_pos.assign(xy, xy + n);
  e->have_pos_input = true;
  e->skip_rescale = dont_rescale != 0;   // src/index.ts:553
  e->pos_dirty = true; e->links_dirty = true; e->sizes_dirty = true;
  e->clusters_dirty = true;   // src/index.ts:570
  return st;
}

int orc_set_point_positions(orc_engine* e, const float* xy, uint64_t n) {
  return orc_set_point_positions_ex(e, xy, n, 0);
}

int orc_set_point_clusters(orc_engine* e, const float* v, uint64_t n) {
  if (!v || n == 0) { e->in_clusters.clear(); e->have_clusters = false; }
  else { e->in_clusters.assign(v, v + n); e->have_clusters = true; }
  e->clusters_dirty = true;
  return 0;
}

int orc_set_cluster_positions(orc_engine* e, const float* v, uint64_t n) {
  if (!v) { e->in_cluster_pos.clear(); e->have_cluster_pos = false; }
  else { e->in_cluster_pos.assign(v, v + n); e->have_cluster_pos = true; }
  e->clusters_dirty = true;
  return 0;
}

int orc_set_point_cluster_strength(orc_engine* e, const float* v, uint64_t n) {
  if (!v || n == 0) { e->in_cluster_strength.clear(); e->have_cluster_strength = false; }
  else { e->in_cluster_strength.assign(v, v + n); e->have_cluster_strength = true; }
  e->clusters_dirty = true;
  return 0;
}

int orc_get_cluster_positions(orc_engine* e, double* out, uint64_t cap, uint64_t* n_out) {
  // Clusters.getCentroidPositions (Clusters/index.ts:389-423), from the current positions
  const uint64_t n = e->point_clusters ? 2 * (uint64_t)e->K : 0;
  if (n_out) *n_out = n;
  if (!out || n == 0) return 0;
  if (cap < n) return CGL_INVALID_ARG;
  std::vector<float> sx, sy, sn;
  cluster_sums(e, e->pos, sx, sy, sn);
  for (uint32_t c = 0; c < e->K; ++c) {
    out[2 * c] = (double)sx[c] / (double)sn[c];
    out[2 * c + 1] = (double)sy[c] / (double)sn[c];
  }
  return 0;
}

int orc_set_links(orc_engine* e, const float* st, uint64_t n) {
  int s = 0;
  if (n % 2) { n -= 1; s = CGL_WARNING; }
  e->in_links.assign(st, st + n);
  e->have_link_input = true;
  e->links_dirty = true;
  return s;
}

int orc_set_link_strength(orc_engine* e, const float* v, uint64_t n) {
  if (!v || n == 0) { e->in_strength.clear(); e->have_strength = false; }
  else { e->in_strength.assign(v, v + n); e->have_strength = true; }
  e->links_dirty = true;
  return 0;
}

int orc_set_point_sizes(orc_engine* e, const float* v, uint64_t n) {
  if (!v) { e->in_sizes.clear(); e->have_sizes = false; }
  else { e->in_sizes.assign(v, v + n); e->have_sizes = true; }
  e->sizes_dirty = true;
  return 0;
}

int orc_set_pinned_points(orc_engine* e, const double* idx, uint64_t n) {
  e->pinned_set = idx && n > 0;
  e->pinned_input.assign(idx ? idx : nullptr, idx ? idx + n : nullptr);
  if (e->N) apply_pinned(e);
  return 0;
}

int orc_render(orc_engine* e, double alpha) {
  // GraphData.update (GraphData/index.ts:443-462)
  uint64_t N = e->have_pos_input ? e->in_pos.size() / 2 : 0;
  uint64_t E = e->have_link_input ? e->in_links.size() / 2 : 0;
  if (N == 0 && E == 0) return 0;  // render() with no data (src/index.ts:941-955)
  const bool pos_changed = e->pos_dirty;
  const bool links_changed = e->links_dirty || pos_changed;
  if (pos_changed) {
    e->N = N;
    e->data_pos = e->in_pos;
    // Points.updatePositions (Points/index.ts:396-413): rescale the input
    // (in place in the reference, on the applied copy here)
    bool rescale = e->cfg.rescale_positions == 1;
    if (e->cfg.rescale_positions < 0 && !e->cfg.enable_simulation) rescale = true;
    if (e->skip_rescale) rescale = false;
    e->skip_rescale = false;
    if (rescale) rescale_initial_positions(e->data_pos, e->cfg.space_size);
  }
  e->E = E;
  e->data_links = e->in_links;
  e->has_strength = e->have_strength && e->in_strength.size() == E;
  if (e->has_strength) e->data_strength = e->in_strength;
  e->has_data_sizes = e->have_sizes;
  e->data_sizes = e->in_sizes;
  // Graph.update (src/index.ts:1987-1994)
  e->T = (uint32_t)std::ceil(std::sqrt((double)e->N));
  e->W = (uint32_t)std::ceil(std::sqrt((double)e->E * 2));
  if (pos_changed) {
    // Points.updatePositions (Points/index.ts:390-592): position, exit, pinned
    e->pos.assign(2 * e->N, 0.f);
    e->absent.assign(e->N, 0);
    for (uint64_t i = 0; i < e->N; ++i) {
      float x = e->data_pos[2 * i], y = e->data_pos[2 * i + 1];
      bool ab = std::isnan(x) || std::isnan(y);
      e->absent[i] = ab;
      e->pos[2 * i] = ab ? NAN : x;
      e->pos[2 * i + 1] = ab ? NAN : y;
    }
    apply_pinned(e);
    e->fx.setup(e->N, (float)e->adjusted_space);
    // ForceManyBody.create (ForceManyBody/index.ts:124-185): pyramid + jitter
    if (e->T) {
      double target = 2 * std::sqrt((double)e->N);
      double g = std::min((double)kMaxGrid, std::max(8.0, std::pow(2.0, std::ceil(std::log2(target)))));
      e->Gf = (int)g;
      e->L = (int)std::log2(g) - 1;
      e->jitter.assign(2 * e->N, 0.f);
      const uint64_t texels = (uint64_t)e->T * e->T;
      for (uint64_t t = 0; t < texels; ++t) {
        float jx = (float)(e->rnd(-1, 1) * 0.00001);
        float jy = (float)(e->rnd(-1, 1) * 0.00001);
        if (t < e->N) { e->jitter[2 * t] = jx; e->jitter[2 * t + 1] = jy; }
      }
      e->mb_ready = true;
    }
    e->collision_ready = false;
  }
  if (e->sizes_dirty) e->collision_ready = false;
  if (links_changed) {
    // ForceLink.create(INCOMING) then (OUTGOING) (src/index.ts:1663-1666)
    e->csr_in = Csr{}; e->csr_out = Csr{};
    if (e->T && e->W) {
      std::vector<uint32_t> deg(e->N, 0);
      for (uint64_t i = 0; i < e->E; ++i) {
        double s = e->data_links[2 * i], t = e->data_links[2 * i + 1];
        if (is_point_index(s, e->N) && is_point_index(t, e->N)) { deg[(size_t)s]++; deg[(size_t)t]++; }
      }
      build_csr(e, true, e->csr_in, deg);
      build_csr(e, false, e->csr_out, deg);
    } else {
      e->csr_in.rowptr.assign(e->N + 1, 0);
      e->csr_out.rowptr.assign(e->N + 1, 0);
    }
  }
  if (e->clusters_dirty) clusters_create(e);   // Graph.create (src/index.ts:1668)
  e->pos_dirty = e->links_dirty = e->sizes_dirty = e->clusters_dirty = false;
  if (!std::isnan(alpha)) e->alpha = alpha;
  return 0;
}

int orc_start(orc_engine* e, double alpha) {
  if (!e->cfg.enable_simulation || e->N == 0) return 0;
  e->running = true; e->progress = 0; e->alpha = alpha;
  return 0;
}
int orc_stop(orc_engine* e) { e->running = false; e->progress = 0; e->alpha = 0; return 0; }
int orc_pause(orc_engine* e) { if (e->running) e->running = false; return 0; }
int orc_unpause(orc_engine* e) { if (e->cfg.enable_simulation) e->running = true; return 0; }

int orc_step(orc_engine* e, uint32_t ticks) {
  if (!e->cfg.enable_simulation || e->T == 0) return 0;
  for (uint32_t t = 0; t < ticks; ++t) run_tick(e);
  return 0;
}

int orc_set_pointer(orc_engine* e, double x, double y, int32_t right) {
  e->mouse_x = x; e->mouse_y = y; e->right_button = right != 0;
  return 0;
}

int orc_set_drag(orc_engine* e, int64_t index) {
  if (!e->cfg.enable_drag) return 0;
  if (index >= (int64_t)e->N) return CGL_INVALID_ARG;
  e->drag_index = index < 0 ? -1 : index;
  return 0;
}

int orc_frame(orc_engine* e, uint32_t frames, uint32_t* done) {
  uint32_t n = 0;
  if (e->T)
    for (uint32_t k = 0; k < frames; ++k) run_frame(e, &n);
  if (done) *done = n;
  return 0;
}

int orc_run(orc_engine* e, uint32_t max_ticks, uint32_t* done) {
  // frames until the simulation ends (src/index.ts:2161-2175)
  uint32_t n = 0;
  if (e->cfg.enable_simulation && e->T)
    while (n < max_ticks && e->running) run_frame(e, &n);
  if (done) *done = n;
  return 0;
}

int orc_get_point_positions(orc_engine* e, float* out, uint64_t cap) {
  if (cap < 2 * e->N) return CGL_INVALID_ARG;
  for (uint64_t i = 0; i < e->N; ++i) {
    out[2 * i] = e->absent[i] ? NAN : e->pos[2 * i];
    out[2 * i + 1] = e->absent[i] ? NAN : e->pos[2 * i + 1];
  }
  return 0;
}

int orc_get_state(orc_engine* e, cgl_state* s) {
  s->alpha = e->alpha; s->progress = e->progress; s->is_simulation_running = e->running;
  s->destroyed = 0; s->tick = e->tick; s->points_number = e->N; s->links_number = e->E;
  s->rng_draws = e->rng_ctr;
  return 0;
}

int orc_get_layout(orc_engine* e, cgl_layout* o) {
  std::memset(o, 0, sizeof(*o));
  o->points_number = e->N;
  uint64_t live = 0;
  for (uint64_t i = 0; i < e->N; ++i) live += !e->absent[i];
  o->live_points = live;
  o->links_number = e->E;
  o->link_entries_in = e->csr_in.col.size();
  o->points_texture_size = e->T;
  o->finest_grid = e->Gf; o->levels = e->L;
  o->max_degree_in = e->csr_in.max_degree; o->max_degree_out = e->csr_out.max_degree;
  o->fixed_point_bits = e->fx.F; o->fixed_point_bound = e->fx.bound;
  o->collision_grid = e->cgrid; o->collision_cell_size = e->ccell;
  return 0;
}

int orc_debug_get_cells(orc_engine* e, uint32_t level, float* out, uint64_t cap) {
  if (level >= e->levels.size()) return CGL_INVALID_ARG;
  const auto& lv = e->levels[level];
  if (cap < lv.size() * 4) return CGL_INVALID_ARG;
  for (size_t c = 0; c < lv.size(); ++c) {
    out[4 * c] = lv[c].cx; out[4 * c + 1] = lv[c].cy; out[4 * c + 2] = lv[c].count;
    out[4 * c + 3] = (float)lv[c].nslot;
  }
  return 0;
}

int orc_debug_get_slots(orc_engine* e, int32_t* out, uint64_t cap) {
  if (cap < e->slots.size()) return CGL_INVALID_ARG;
  std::copy(e->slots.begin(), e->slots.end(), out);
  return 0;
}

// CSR views for ingest parity (direction 0 = incoming, 1 = outgoing).
int orc_debug_get_csr(orc_engine* e, int dir, uint32_t* rowptr, uint32_t* col, float* rnd, float* bias,
                      float* strength) {
  const Csr& c = dir == 0 ? e->csr_in : e->csr_out;
  std::copy(c.rowptr.begin(), c.rowptr.end(), rowptr);
  std::copy(c.col.begin(), c.col.end(), col);
  std::copy(c.rnd.begin(), c.rnd.end(), rnd);
  std::copy(c.bias.begin(), c.bias.end(), bias);
  std::copy(c.strength.begin(), c.strength.end(), strength);
  return 0;
}

int orc_debug_get_jitter(orc_engine* e, float* out, uint64_t cap) {
  if (cap < e->jitter.size()) return CGL_INVALID_ARG;
  std::copy(e->jitter.begin(), e->jitter.end(), out);
  return 0;
}

// Primitive functions, exposed for known-answer tests.
uint32_t orc_lowbias32(uint32_t h) { return lowbias32(h); }
float orc_peel_hash(uint32_t index, uint32_t seed_bits) { return peel_hash(index, seed_bits); }
uint64_t orc_splitmix_draw(uint64_t seed, uint64_t k) { return splitmix_draw(seed, k); }
// The first n values of seedrandom(seed_text) (random's next()).
void orc_seedrandom(const char* seed_text, uint64_t n, double* out) {
  Arc4Seed a;
  a.seed(utf16_units(seed_text));
  for (uint64_t k = 0; k < n; ++k) out[k] = a.prng();
}
void orc_sincos(float a, float* s, float* c) { portable_sincos(a, s, c); }
int orc_cell_index(float p, float cs, int G) { return cell_index(p, cs, G); }

// Many-body velocity (before friction) of every point for the current
// positions, using the engine's next per-tick seed without consuming it:
//   precision 0 — the FP32 restatement (what a tick applies);
//   precision 1 — the same grid-pyramid approximation and the same cells and
//                 slots, every force operation in FP64 (centroids from the
//                 exact cell sums);
//   precision 2 — exact all-pairs FP64 repulsion with the same clamped
//                 falloff (no jitter), O(N^2): for N up to ~20k.
// Puts the FP32 rounding error and the approximation error on record.
int orc_manybody_velocity(orc_engine* e, int precision, double* out) {
  if (!e->mb_ready) return CGL_INVALID_ARG;
  const int64_t N = (int64_t)e->N;
  const float k32 = (float)e->alpha * (float)e->cfg.simulation_repulsion;
  for (int64_t i = 0; i < 2 * N; ++i) out[i] = 0;
  if (precision == 2) {
    const double k = k32;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < N; ++i) {
      double vx = 0, vy = 0;
      if (!e->absent[i]) {
        double px = e->pos[2 * i], py = e->pos[2 * i + 1];
        for (int64_t j = 0; j < N; ++j) {
          if (j == i || e->absent[j]) continue;
          double dx = px - e->pos[2 * j], dy = py - e->pos[2 * j + 1];
          double l = dx * dx + dy * dy;
          if (l <= 0) continue;
          double len = std::sqrt(l);
          if (l < 1) l = std::sqrt(l);
          double add = k / std::sqrt(l);
          vx += add * (dx / len); vy += add * (dy / len);
        }
      }
      out[2 * i] = vx; out[2 * i + 1] = vy;
    }
    return 0;
  }
  const uint64_t saved_ctr = e->rng_ctr;
  const Arc4Seed saved_arc = e->arc;
  const float seed = (float)e->rnd(0, 1);
  e->rng_ctr = saved_ctr;
  e->arc = saved_arc;
  std::vector<std::vector<double>> f64;
  std::vector<float> prev = e->pos;
  build_pyramid_and_slots(e, prev, fbits(seed), precision == 1, &f64);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < N; ++i) {
    if (e->absent[i]) continue;
    if (precision == 0) {
      float vx, vy;
      manybody_point<float>(e, prev, i, k32, nullptr, vx, vy);
      out[2 * i] = vx; out[2 * i + 1] = vy;
    } else {
      double vx, vy;
      manybody_point<double>(e, prev, i, (double)k32, &f64, vx, vy);
      out[2 * i] = vx; out[2 * i + 1] = vy;
    }
  }
  return 0;
}

}  // extern "C"
