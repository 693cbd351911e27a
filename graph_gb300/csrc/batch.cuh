// batch.cuh — device interface of the batched engine (batch_kernels.cu).
//
// Many independent graphs advance together: every per-point array lives in a
// point arena, every per-cell array in a cell arena, and so on; graph g owns
// one contiguous range of each arena, described by GraphDesc.  Kernels run
// over the arenas' used prefixes and read each point's graph from `gid`, so a
// tick is one launch per kernel for all graphs.  Graphs can join and leave
// between ticks (ranges are allocated and freed on the host).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace cgl {

constexpr uint32_t kNoGraph = 0xFFFFFFFFu;
constexpr uint32_t kNoPoint = 0xFFFFFFFFu;
constexpr uint32_t kLinkWarpsPerBlock = 8;   // light-row link pass: warps of one graph per block
constexpr int kScanSub = 4;                  // scan: sub-chunks of kBlock x 4 cells per block
constexpr int kChunk = 1024 * kScanSub;      // scan: cells per block
constexpr uint32_t kBatchErrorScan = 1;      // error_word bit: a scan block's look-back gave up waiting
constexpr uint32_t kBatchOutside = 4;        // big_count word: a binned point outside its space
constexpr uint32_t kBatchSibs = 5;           // big_count word: the many-body pass's work items this tick

// Per graph per tick: the f32 alpha uniform, the peel seed, and whether the
// graph advances this tick (a graph that reached its tick budget, or whose
// run loop ended, keeps its positions).
struct BatchTick {
  float alpha;
  uint32_t seed_bits;
  uint32_t active;
  uint32_t pad;
};

enum : uint32_t { kGGravity = 1, kGCenter = 2, kGManybody = 4, kGLinkIn = 8, kGLinkOut = 16, kGCollision = 32 };

struct GraphDesc {
  uint32_t p_off, n;           // points [p_off, p_off + n) of the point arena
  uint32_t cell_off;           // finest cells [cell_off, cell_off + gf^2) of the cell arena
  uint32_t rec_off;            // level records: level l at rec_off + base(l)
  uint32_t acc_off;            // integer sums of the levels coarser than the cell-kernel tile
  uint32_t acc_cells;          // cells of those levels
  uint32_t rp_in, rp_out;      // rowptr arena offsets (n + 1 entries each, graph-local entry indices)
  uint32_t e_in, e_out;        // entry arena offsets of the two directions' lists
  // The light rows (lists of at most kHeavyDegree links) by warps, per
  // direction d: warp w's 32 rows are graph-local points at lrow[lr[d] + 32 w ..]
  // (kNoPoint: none), its entries lanes[ln[d] + lwoff[lw[d] + w] .. ln[d] +
  // lwoff[lw[d] + w + 1]), entry k of lane l at 32 k + l, each list padded with
  // absent entries to its warp's longest; rows by list length, longest first.
  uint32_t lr[2], lw[2], ln[2], nw[2];
  int32_t gf, levels, tile;
  uint32_t stages;             // kG* forces this graph runs
  float space, csf, friction, gravity, repulsion;
  float link_spring, link_distance, link_r0, link_r1;
  FixedScale fx;
  float center;                // simulationCenter (kGCenter)
  int32_t level_guard;         // finest cell >= 2 units, space <= 2^25 (the plain engine's level_guard)
  // collision (kGCollision): four coll_grid^2 grids from cell coll_off of the collision arena
  uint32_t coll_off;
  int32_t coll_grid;
  float coll_cell, coll_strength, coll_radius, coll_padding;
};

struct BatchView {
  uint32_t slots;              // descriptor slots (stride of the per-tick parameters)
  uint32_t point_hwm;          // arena points in use: [0, point_hwm)
  uint32_t cell_hwm;           // arena cells in use
  const GraphDesc* desc;
  const uint32_t* gid;         // graph of each arena point, kNoGraph if free
  const uint32_t* cell_gid;    // graph of each arena cell
  float2* pos;
  float2* pos_alt;
  const uint8_t* flags;
  const float2* jitter;
  uint32_t* key;
  uint32_t* rank;
  uint32_t* sorted_idx;        // absolute arena point indices, grouped by cell
  float2* sorted_pos;
  uint32_t* inv;               // null: a batch keeps no sorted-position map (no early pass)
  uint32_t* counts;            // [cell arena], zeroed by the scan
  uint32_t* cell_start;        // [cell arena + 1]
  unsigned long long* scan_status;   // one-pass scan: status word per chunk of kChunk cells
  unsigned long long* scan_seq;      // its chunk tickets, counted up across ticks (zeroed with scan_status)
  uint32_t* error_word;        // host-mapped: kBatchError* bits raised by a device wait that gave up
  uint32_t* big_list;          // [2 x cell arena] CTA cells, then warp cells: those above
                               // kWarpSmallCell from the front, the others from the back
  uint32_t* big_count;         // [8] CTA cells, heavy and light warp cells, warp-cell ticket, then [4] = 1
                               // when a binned point lies outside its graph's space, [5] the many-body
                               // pass's work items (zeroed each tick)
  uint2* sib_list;             // [point arena] many-body work items: sorted positions (jA, jB), jB = kNoPoint
                               // when jA is alone; the points of one parent cell (kb_cells)
  long long* big_sx;
  long long* big_sy;
  uint32_t* big_ns;
  float4* rec;
  long long* acc;
  const uint2* tiles;          // (graph, tile) work list of the cell kernel
  uint32_t n_tiles;
  const uint32_t* rowptr;
  const uint4* ent;            // neighbour = graph-local point index or kAbsentTarget
  const uint32_t* lrow;        // light rows by warps (GraphDesc::lr, lw, ln, nw)
  const uint32_t* lwoff;
  const uint4* lanes;
  const uint2* lwork[2];       // (graph, first warp) of each block of the light-row link pass, per direction
  uint32_t n_lwork[2];
  const uint32_t* heavy_in;    // absolute points with long incoming lists
  uint32_t n_heavy_in;
  const uint32_t* heavy_out;
  uint32_t n_heavy_out;
  const BatchTick* ticks;      // [tick][slot]
  uint32_t* tick_ctr;
  PairUnits units;             // {1, -0}: operands of the paired sums and products
  // center: exact (x, y, count) sums per slot, zeroed at tick start
  long long* centroid;
  // collision: resolved point sizes; grid sums and grids of the collision arena
  const float* size;           // [point arena]
  long long* cgrid_acc;        // 4 per collision cell, zero between ticks
  float4* cgrid;
  const uint32_t* coll_gid;    // graph of each collision cell, kNoGraph if free
  uint32_t coll_hwm;           // collision cells in use
  int any_center, any_collision;   // some job runs the force (its kernels are launched)
};

// Light rows by warps on the device (batch_kernels.cu): woff[w] = 32 x the
// length of row order[nh + 32 w] (w < nw), 0 at nw; lrow[t] = order[nh + t]
// (t < n - nh), kNoPoint up to 32 nw.
void batch_warp_lengths(const uint32_t* order, const uint32_t* len, uint32_t nh, uint32_t n, uint32_t* woff,
                        cudaStream_t st);
void batch_warp_rows(const uint32_t* order, uint32_t nh, uint32_t n, uint32_t* lrow, cudaStream_t st);

uint32_t batch_scan_blocks(uint32_t cells);   // blocks of the one-pass scan over `cells` cells

void batch_launch_tick(const BatchView& v, cudaStream_t st, cudaStream_t side, cudaEvent_t* fork, cudaEvent_t* join);
uint32_t batch_kernels_per_tick(const BatchView& v);

}  // namespace cgl
