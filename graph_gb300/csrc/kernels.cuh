// kernels.cuh — launch interface of the per-tick kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace cgl {

// Per-tick scalars computed on the host (alpha in FP64 -> f32 uniform, the
// near-field peel seed draw), read on the device at tick_params[*tick_ctr].
struct TickParams {
  float alpha;
  uint32_t seed_bits;
};

// Device state of one engine: structure-of-arrays in HBM.
struct DeviceView {
  uint32_t n;                 // points (original index space)
  float2* pos;                // current positions [n]
  float2* pos_alt;            // ping-pong target of the link passes [n]
  const uint8_t* flags;       // kPinned | kAbsent | kEarly [n]
  const float2* jitter;       // per-point random vector (ForceManyBody/index.ts:133-138) [n]
  uint32_t* key;              // finest cell of each point, kNoCell if absent [n] (of position j when
                              // bin_state[1]: see idx_s)
  uint32_t* rank;             // rank within its cell from the histogram atomics [n] (likewise)
  uint32_t* sorted_idx;       // points grouped by finest cell; head of each cell = slots in hash order [n]
  float2* sorted_pos;         // positions in the same order (snapshot for the many-body pass) [n]
  uint32_t* counts;           // finest-cell histogram [G^2] (zeroed by the scan)
  uint32_t* cell_start;       // exclusive scan [G^2 + 1]
  unsigned long long* block_sums;  // scan status per chunk: (count, pairs) packed as low and high 32
                                   // bits of a 60-bit value, with its flags (kernels.cu, k_scan)
  uint32_t* idx_s;            // binning in the previous cell order: the point at position j [n]
  float2* pos_s;              // and its position after the prepass [n]
  uint32_t* bin_state;        // [0] = 1 once sorted_idx holds a cell order of the live points (zeroed at
                              // render); [1] = 1 when this tick's keys and ranks are by that order
  uint32_t* pair_start;       // exclusive scan of ceil(count / 2) per finest cell [G^2 + 1]
  uint32_t* pair_list;        // per pair of one cell's consecutive sorted positions (j, j + 1): j,
                              // with the top bit set when j is the cell's last point alone [<= n]
  unsigned long long* scan_seq;   // scan chunk tickets, counted up across ticks (zeroed with block_sums)
  uint32_t* error_word;       // host-mapped: kError* bits raised by a device wait that gave up
  float4* rec;                // cell records of all levels (cx, cy, count, nslot)
  uint32_t level_off[10];     // offset of level l in rec
  long long* acc;             // coarse-level integer sums (x, y, count) per cell, levels < tile level
  uint32_t acc_off[10];       // offset (in cells) of level l in acc
  uint32_t* cells_ticket;     // last-block ticket of the cell kernel
  uint32_t* big_list;         // [G^2] cells above kBigCell, then [G^2] warp cells: those above
                              // kWarpSmallCell from the front, the others above kSmallCell from the back
  uint32_t* big_count;        // [8] CTA cells, heavy and light warp cells this tick, warp-cell
                              // ticket, then [4] = 1 when a binned point lies outside [0, space]
                              // (zeroed at tick start)
  long long* big_sx;          // exact sums of big cells [G^2]
  long long* big_sy;
  uint32_t* big_ns;           // slots of big cells [G^2]
  long long* centroid;        // x, y, count sums for ForceCenter
  const TickParams* tick_params;
  uint32_t* tick_ctr;
  // link CSR (two directions)
  const uint32_t* rowptr_in;
  const uint4* ent_in;        // (col, rnd bits, bias bits, strength bits)
  const uint32_t* rowptr_out;
  const uint4* ent_out;
  const uint32_t* heavy_in;   // all points by incoming list length, longest first;
  const uint32_t* heavy_out;  // the first n_heavy_* have lists longer than kHeavyDegree
  uint32_t n_heavy_in, n_heavy_out;
  // Leading hubs run on an SM each on a second stream.  Incoming (early hubs):
  // the first n_early_hubs rows of heavy_in run their chains beside the
  // many-body pass.  Their points and link targets (early_pts, kEarly in
  // flags) take their many-body terms in a pass of their own first; inv then
  // holds each live point's sorted position.  Outgoing: the first n_first_out
  // rows of heavy_out run beside the rest of the pass, and the next
  // n_next_out on a third stream without SMs of their own.
  const uint32_t* early_pts;
  uint32_t n_early_pts, n_early_hubs, n_first_out, n_next_out;
  uint32_t* inv;              // sorted position of each live point [n]; null without early hubs
  // The rows after the first n_heavy_* of the order, by warps of 32: warp w's
  // entries at lane_ent[woff[w] .. woff[w + 1]), entry k of lane l at
  // 32 k + l, each lane's list padded to its warp's longest with absent entries.
  const uint32_t* woff_in;
  const uint4* lane_ent_in;
  const uint32_t* woff_out;
  const uint4* lane_ent_out;
  // collision
  const float* size;          // resolved point sizes [n]
  long long* cgrid_acc;       // 4 grids x G_c^2 x (x, y, size, count)
  float4* cgrid;              // 4 grids x G_c^2 (sx, sy, ssize, count)
  uint32_t* coll_mark;        // a bit per cell of the 4 grids: the 3x3 windows around the late points'
                              // cells (launch_collision_late); zero between ticks
  float2* pos_coll;           // collision results computed beside late points [n] (with leading
                              // outgoing hubs; the chains still read pos_alt)
  uint32_t* coll_redo;        // [0]: count, then the points whose collision result is computed again
                              // [1 + n] (launch_collision_fixup); the count is zero between ticks
  // clusters
  const uint32_t* cluster_of;     // cluster of each point, 0xFFFFFFFF if none [n]
  const float* cluster_coeff;     // pull coefficient of each point [n]
  const float2* cluster_custom;   // cluster position, negative = centre of mass [K]
  long long* cluster_acc;         // x, y, count sums per cluster [3K]
  uint32_t n_clusters;            // K
};

struct SimScalars {
  float space;                // adjustedSpaceSize (f32 uniform)
  float friction;
  float gravity;
  float center;
  float repulsion;
  float link_spring;
  float link_distance;
  float link_r0, link_r1;     // linkDistRandomVariationRange
  float coll_strength;
  float coll_radius;          // 0 when undefined
  float coll_padding;
  float coll_cell;            // collision cell size (f32 uniform)
  int coll_grid;
  int gf;                     // finest grid
  int levels;
  int tile;                   // cell-kernel tile edge
  float csf;                  // finest cell size
  FixedScale fx;
  PairUnits units;            // {1, -0}: operands of the paired sums and products
  float cluster;              // simulationCluster
  int pairs;                  // the many-body pass takes two points of a cell per thread (k_manybody_duo);
                              // the binning passes then also build its work list
  int mb_kernel;              // CGL_MANYBODY_* (include/cgl.h): the many-body pass's kernel
  int level_guard;            // finest cell >= 2 units and space <= 2^25: a level term's length is
                              // then in [1, 2^52] whenever every binned point lies in [0, space]
  int any_pinned;             // some live point is pinned
  int skip_early;             // this tick runs k_manybody_early: the many-body pass leaves kEarly points to it
};
constexpr uint32_t kErrorScan = 1;     // error_word bit: a scan block's look-back gave up waiting
constexpr uint32_t kOutsideFlag = 4;   // big_count word of the outside-the-space flag
constexpr uint32_t kSingleBit = 0x80000000u;


enum : int { kManybodyOnePoint = 0, kManybodySplit = 1, kManybodyTwoPoints = 2 };   // CGL_MANYBODY_*
enum PrepassMode : uint32_t { kPreGravity = 1, kPreCentroid = 2, kPreBin = 4 };

void launch_prepass(const DeviceView& d, const SimScalars& s, uint32_t mode, cudaStream_t st);
void launch_center(const DeviceView& d, const SimScalars& s, bool bin, cudaStream_t st);
void launch_scan(const DeviceView& d, const SimScalars& s, cudaStream_t st);
// The scans' bounded look-back against a status array nothing sets (2 words, zeroed).
void launch_wait_limit(const unsigned long long* status, uint32_t* error, cudaStream_t st);
void launch_scatter(const DeviceView& d, const SimScalars& s, cudaStream_t st);
void launch_cells(const DeviceView& d, const SimScalars& s, cudaStream_t st);
void launch_manybody(const DeviceView& d, const SimScalars& s, cudaStream_t st);
// The many-body terms of the early points alone (DeviceView::early_pts).
void launch_manybody_early(const DeviceView& d, const SimScalars& s, cudaStream_t st);
// direction 0 = incoming (reads pos, writes pos_alt), 1 = outgoing (pos_alt -> pos)
// The first n_heavy_* rows of the order each get a CTA of their own.
// A link pass: all of it (kLinkAll), or its hub CTAs or its light rows alone
// (the two halves write disjoint points and may run on two streams); or the
// leading hubs' CTAs (n_early_hubs incoming, n_first_out outgoing), an SM
// each, the next outgoing hubs' CTAs (n_next_out), and then the rest of the
// pass.
enum { kLinkAll = 0, kLinkHubs = 1, kLinkLight = 2, kLinkFirstHubs = 3, kLinkNextHubs = 4, kLinkAfterFirst = 5 };
void launch_link(const DeviceView& d, const SimScalars& s, int direction, bool swap_back, cudaStream_t st,
                 int part = kLinkAll);
// mark[order[t]] = 1 for t < nhub (the points whose list runs on a hub CTA)
void launch_mark_hubs(const uint32_t* order, uint32_t nhub, uint8_t* mark, cudaStream_t st);
// spans[t] = (rowptr[order[t]], rowptr[order[t] + 1]) for t < m
void launch_hub_spans(const uint32_t* order, const uint32_t* rowptr, uint32_t m, uint2* spans, cudaStream_t st);
// keys[t] = the finest cell (row-major) of pos[pts[t]] for t < m
void launch_cell_keys(const float2* pos, const uint32_t* pts, uint32_t m, float csf, int gf, uint32_t* keys,
                      cudaStream_t st);
// The warp layout of one direction's light rows (woff, lane_ent above):
// warp_lengths writes 32 x the longest list of each of the nw warps to
// woff[0 .. nw) and 0 to woff[nw] (an exclusive scan then gives the offsets);
// fill_lanes copies the lists into place.
void launch_warp_lengths(const uint32_t* order, const uint32_t* rowptr, uint32_t nhub, uint32_t n, uint32_t* woff,
                         cudaStream_t st);
void launch_fill_lanes(const uint32_t* order, const uint32_t* rowptr, const uint4* ent, uint32_t nhub, uint32_t n,
                       const uint32_t* woff, uint4* lane_ent, cudaStream_t st);
// `order`: the live points in cell order (sorted_idx of this tick's many-body
// pass, `count` of them), or nullptr to take all points in index order.
void launch_collision_grid(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                           cudaStream_t st);
// launch_collision_grid in two steps: the integer grid sums of the points in
// `order` not marked in `skip` (nullptr: all), then their conversion to the
// grids once every point is summed.
void launch_collision_sums(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                           const uint8_t* skip, cudaStream_t st);
// zero: clear the integer sums after converting (else they stay for later points)
void launch_collision_convert(const DeviceView& d, const SimScalars& s, cudaStream_t st, bool zero = true);
void launch_collision_force(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                            cudaStream_t st);
// Collision beside late points (chains still running): launch_collision_force
// of every point not marked `late`, from grids without the late points, into
// pos_coll.  After the late points' sums: launch_collision_late converts the
// late points' cells again and marks the 3x3 windows around them in coll_mark;
// launch_collision_fixup then moves every result into pos and lists the points
// that read a marked cell (and the late points) in coll_redo, whose results it
// computes again.  A point's force reads only its 3x3 windows, so every other
// result is already the final one.
void launch_collision_force_early(const DeviceView& d, const SimScalars& s, const uint32_t* order, uint32_t count,
                                  const uint8_t* late, cudaStream_t st);
void launch_collision_late(const DeviceView& d, const SimScalars& s, const uint32_t* late_list, uint32_t n_late,
                           cudaStream_t st);
void launch_collision_fixup(const DeviceView& d, const SimScalars& s, const uint8_t* late, cudaStream_t st);
// Sums of each cluster's live points (cluster_acc must be zero on entry).
void launch_cluster_sum(const DeviceView& d, const SimScalars& s, cudaStream_t st);
// The cluster pull and the update of every point.
void launch_cluster_force(const DeviceView& d, const SimScalars& s, cudaStream_t st);
void launch_tick_end(const DeviceView& d, cudaStream_t st);
// Right-click repulsion from the pointer (force-mouse.frag) and the update.
void launch_mouse(const DeviceView& d, const SimScalars& s, float2 mouse, float repulsion, cudaStream_t st);
// The dragged point follows the pointer (drag-point.frag).
void launch_drag(const DeviceView& d, uint32_t index, float2 mouse, cudaStream_t st);
// The renderer's points texture: texels [0, texels), (x, y, index, 0) below n.
void launch_position_texture(const DeviceView& d, float4* out, uint32_t texels, cudaStream_t st);

uint32_t scan_blocks(uint32_t cells);

}  // namespace cgl
