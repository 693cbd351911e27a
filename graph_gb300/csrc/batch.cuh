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
  uint32_t rp_in, rp_out;      // rowptr arena offsets (n + 1 entries each, absolute entry indices)
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
  uint32_t* counts;            // [cell arena], zeroed by the scan
  uint32_t* cell_start;        // [cell arena + 1]
  uint32_t* scan1;             // scan partials per 1024 cells, then per 1024^2
  uint32_t* scan2;
  uint32_t* big_list;          // [2 x cell arena] CTA cells, then warp cells: those above
                               // kWarpSmallCell from the front, the others from the back
  uint32_t* big_count;         // [8] CTA cells, heavy and light warp cells, warp-cell ticket, then [4] = 1
                               // when a binned point lies outside its graph's space (zeroed each tick)
  long long* big_sx;
  long long* big_sy;
  uint32_t* big_ns;
  float4* rec;
  long long* acc;
  const uint2* tiles;          // (graph, tile) work list of the cell kernel
  uint32_t n_tiles;
  const uint32_t* rowptr;
  const uint4* ent;            // neighbour = absolute arena point index or kAbsentTarget
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

void batch_launch_tick(const BatchView& v, cudaStream_t st, cudaStream_t side, cudaEvent_t* fork, cudaEvent_t* join);
uint32_t batch_kernels_per_tick(const BatchView& v);

}  // namespace cgl
