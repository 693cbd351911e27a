// engine.cu — host side of the GB300 force-layout engine: the C ABI of
// include/cgl.h, data ingest (Graph.render), the simulation state machine
// (Store, Graph.start/stop/pause/unpause/step) and tick scheduling on one CUDA
// stream, one captured CUDA graph per tick topology.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/cgl.h"
#include "ingest.h"
#include "ingest_device.cuh"
#include "kernels.cuh"

using namespace cgl;

namespace {

constexpr double kAlphaMin = 0.001;   // ALPHA_MIN (Store/index.ts:8)
constexpr uint32_t kParamChunk = 4096; // ticks per parameter upload

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct cgl_engine {
  cgl_config cfg{};
  bool destroyed = false;
  std::string err;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t* h_error = nullptr;   // host-mapped error word (DeviceView::error_word)
  uint32_t* d_error = nullptr;
  // read-back beside the next ticks (cgl_enqueue_point_positions)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t snap_ready = nullptr, snap_done = nullptr;
  bool snap_pending = false;
  DevBuf b_snap;                 // the positions as queued, copied out from here
  cudaStream_t side2 = nullptr;  // the next outgoing hubs' chains (DeviceView::n_next_out)
  cudaEvent_t join2 = nullptr;
  cudaStream_t side = nullptr;   // the early hubs' chains beside the many-body pass; the outgoing hub
                                 // chains beside the collision sums
  cudaEvent_t fork = nullptr, join = nullptr;
  // many-body kernel tuning (cfg.manybody_kernel == CGL_MANYBODY_AUTO): the
  // candidates run kTuneTicks ticks each, timed, and the fastest is kept
  int mb_choice = -1;            // the kernel in use; -1: the size rule
  bool mb_tuned = false;
  std::vector<int> tune_cands;
  uint32_t tune_next = 0;        // timed ticks so far
  float tune_ms[3][3] = {};
  cudaEvent_t tune_ev[2] = {nullptr, nullptr};

  // staged input (copied at set_*, applied at render)
  bool have_pos_input = false, have_link_input = false, have_strength = false, have_sizes = false;
  std::vector<float> in_pos, in_links, in_strength, in_sizes;
  bool pinned_set = false;
  std::vector<double> pinned_input;
  bool pos_dirty = false, links_dirty = false, sizes_dirty = false;
  bool skip_rescale = false;   // Points.shouldSkipRescale (setPointPositions(…, dontRescale))
  bool have_clusters = false, have_cluster_pos = false, have_cluster_strength = false;
  std::vector<float> in_clusters, in_cluster_pos, in_cluster_strength;
  bool clusters_dirty = false;

  // applied data
  uint64_t N = 0, E = 0;
  uint32_t T = 0, W = 0;
  bool has_strength = false;
  std::vector<float> data_sizes;
  bool has_data_sizes = false;
  std::vector<uint8_t> absent, pinned;
  uint64_t live = 0;
  bool any_pinned = false;     // some live point is pinned (a tick-graph constant)
  uint64_t entries = 0;
  uint32_t max_deg_in = 0, max_deg_out = 0;
  bool mb_ready = false;
  int Gf = 0, L = 0, tile = 0;
  int fixed_bits = 0;
  FixedScale fx{};

  // collision
  bool collision_ready = false;
  int cgrid = 0;
  float ccell = 0.f;

  // clusters (Clusters/index.ts)
  bool point_clusters = false, cluster_positions = false;
  uint32_t n_clusters = 0;

  // interaction: Store.mousePosition, Graph.isRightClickMouse, the dragged point
  double mouse_x = 0, mouse_y = 0;
  bool right_button = false;
  int64_t drag_index = -1;

  // simulation state (Store)
  double adjusted_space = 4096;
  double alpha = 1.0;
  double progress = 0.0;
  bool running = false;
  ingest::Rng rng;             // Store.random: the graph's random draws
  std::string seed_text;       // the copied cgl_config.random_seed_text
  uint64_t tick = 0;

  // device state
  size_t dev_bytes = 0;
  DevBuf b_pos, b_pos_alt, b_flags, b_jitter, b_key, b_rank, b_sorted_idx, b_sorted_pos;
  DevBuf b_counts, b_cell_start, b_block_sums, b_tickets, b_rec, b_acc, b_centroid, b_pair_start, b_pair_list;
  DevBuf b_idx_s, b_pos_s, b_bin_state;
  DevBuf b_big_list, b_big_count, b_big_sx, b_big_sy, b_big_ns;
  DevBuf b_params, b_tick_ctr;
  DevBuf b_rowptr_in, b_rowptr_out, b_ent_in, b_ent_out, b_heavy_in, b_heavy_out;
  DevBuf b_hub_out;   // 1 for the points whose outgoing list runs on a hub CTA
  DevBuf b_woff_in, b_woff_out, b_lane_ent_in, b_lane_ent_out;   // light rows by warps (kernels.cuh)
  uint32_t n_heavy_in = 0, n_heavy_out = 0;
  // early hubs (DeviceView::n_early_hubs): their points and link targets
  DevBuf b_early_pts, b_inv;
  uint32_t n_early_hubs = 0, n_early_pts = 0;
  uint32_t n_first_out = 0, n_next_out = 0;   // leading outgoing hubs (DeviceView::n_first_out, n_next_out)
  std::vector<uint8_t> early;   // kEarly per point (empty: none)
  int32_t lead_limit[2] = {-1, -1};   // at most this many leading hubs each way (cgl_debug_set_leading_hubs);
                                      // -1: the rule
  DevBuf b_size, b_cgrid_acc, b_cgrid;
  DevBuf b_coll_mark, b_pos_coll, b_coll_redo;   // DeviceView::coll_mark, pos_coll, coll_redo
  DevBuf b_cl_of, b_cl_coeff, b_cl_custom, b_cl_acc;
  DevBuf b_texture;                        // staging for pageable texture read-back
  DeviceView view{};
  uint32_t level_off[10] = {};
  uint32_t acc_off[10] = {};

  TickParams* h_params = nullptr;          // pinned staging
  cudaEvent_t params_copied = nullptr;
  bool params_pending = false;

  cudaGraphExec_t graph = nullptr;
  bool graph_dirty = true;
  bool use_graph = true;

  double rnd(double mn, double mx) { return rng.uniform(mn, mx); }
};

namespace {

cgl_status fail(cgl_engine* e, cgl_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (e) e->err = buf;
  return st;
}

#define CU(call)                                                                              \
  do {                                                                                        \
    cudaError_t _err = (call);                                                                \
    if (_err != cudaSuccess)                                                                  \
      return fail(e, _err == cudaErrorMemoryAllocation ? CGL_OOM : CGL_CUDA_ERROR, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(_err), __FILE__, __LINE__);                       \
  } while (0)

// After a synchronisation: a device wait that gave up (error_word) is
// reported once, as a CUDA error of the call that found it.
cgl_status device_error(cgl_engine* e) {
  const uint32_t bits = *(volatile uint32_t*)e->h_error;
  if (!bits) return CGL_OK;
  *(volatile uint32_t*)e->h_error = 0;
  return fail(e, CGL_CUDA_ERROR, "a device wait gave up (error bits 0x%x): the last ticks' cell scan is not valid",
              bits);
}

cgl_status dev_reserve(cgl_engine* e, DevBuf& b, size_t bytes, bool zero) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) {
    if (zero) CU(cudaMemsetAsync(b.p, 0, bytes, e->stream));
    return CGL_OK;
  }
  const double budget = e->cfg.hbm_budget_bytes;
  if (budget > 0 && (double)(e->dev_bytes - b.bytes + bytes) > budget)
    return fail(e, CGL_OOM, "device memory budget %.0f bytes exceeded (need %zu more)", budget, bytes - b.bytes);
  if (b.p) {
    CU(cudaStreamSynchronize(e->stream));
    CU(cudaFree(b.p));
    e->dev_bytes -= b.bytes;
    b.p = nullptr;
    b.bytes = 0;
  }
  CU(cudaMalloc(&b.p, bytes));
  b.bytes = bytes;
  e->dev_bytes += bytes;
  if (zero) CU(cudaMemsetAsync(b.p, 0, bytes, e->stream));
  return CGL_OK;
}

void dev_release(cgl_engine* e, DevBuf& b) {
  if (!b.p) return;
  cudaStreamSynchronize(e->stream);
  cudaFree(b.p);
  e->dev_bytes -= b.bytes;
  b.p = nullptr;
  b.bytes = 0;
}

void dev_free_all(cgl_engine* e) {
  DevBuf* all[] = {&e->b_pos, &e->b_pos_alt, &e->b_flags, &e->b_jitter, &e->b_key, &e->b_rank,
                   &e->b_sorted_idx, &e->b_sorted_pos, &e->b_counts, &e->b_cell_start, &e->b_block_sums,
                   &e->b_tickets, &e->b_rec, &e->b_acc, &e->b_centroid, &e->b_params, &e->b_tick_ctr,
                   &e->b_rowptr_in, &e->b_rowptr_out, &e->b_ent_in, &e->b_ent_out, &e->b_size,
                   &e->b_cgrid_acc, &e->b_cgrid, &e->b_big_list, &e->b_big_count,
                   &e->b_big_sx, &e->b_big_sy, &e->b_big_ns, &e->b_heavy_in, &e->b_heavy_out, &e->b_hub_out,
                   &e->b_cl_of, &e->b_cl_coeff, &e->b_cl_custom, &e->b_cl_acc, &e->b_texture,
                   &e->b_woff_in, &e->b_woff_out, &e->b_lane_ent_in, &e->b_lane_ent_out, &e->b_pair_start,
                   &e->b_pair_list, &e->b_idx_s, &e->b_pos_s, &e->b_bin_state, &e->b_early_pts, &e->b_inv,
                   &e->b_coll_mark, &e->b_pos_coll, &e->b_coll_redo, &e->b_snap};
  for (DevBuf* b : all) {
    if (b->p) cudaFree(b->p);
    b->p = nullptr;
    b->bytes = 0;
  }
  e->dev_bytes = 0;
}

void adjust_space_size(cgl_engine* e) { e->adjusted_space = ingest::adjusted_space(e->cfg); }

void setup_fixed(cgl_engine* e) { e->fx = ingest::fixed_for(e->N, e->adjusted_space, &e->fixed_bits); }

float resolved_size(const cgl_engine* e, uint64_t i) {
  // GraphData.getResolvedPointSize (GraphData/index.ts:189-194); EXIT_DEFAULT_SIZE = 0
  if (e->has_data_sizes && i < e->data_sizes.size()) {
    const float r = e->data_sizes[i];
    if (!std::isnan(r)) return r;
  }
  if (e->absent[i]) return 0.f;
  return (float)e->cfg.point_default_size;
}

void refresh_view(cgl_engine* e) {
  DeviceView& d = e->view;
  d.n = (uint32_t)e->N;
  d.pos = (float2*)e->b_pos.p;
  d.pos_alt = (float2*)e->b_pos_alt.p;
  d.flags = (const uint8_t*)e->b_flags.p;
  d.jitter = (const float2*)e->b_jitter.p;
  d.key = (uint32_t*)e->b_key.p;
  d.rank = (uint32_t*)e->b_rank.p;
  d.sorted_idx = (uint32_t*)e->b_sorted_idx.p;
  d.sorted_pos = (float2*)e->b_sorted_pos.p;
  d.counts = (uint32_t*)e->b_counts.p;
  d.cell_start = (uint32_t*)e->b_cell_start.p;
  d.block_sums = (unsigned long long*)e->b_block_sums.p;
  d.pair_start = (uint32_t*)e->b_pair_start.p;
  d.idx_s = (uint32_t*)e->b_idx_s.p;
  d.pos_s = (float2*)e->b_pos_s.p;
  d.bin_state = (uint32_t*)e->b_bin_state.p;
  d.pair_list = (uint32_t*)e->b_pair_list.p;
  d.scan_seq = (unsigned long long*)e->b_tickets.p;
  d.cells_ticket = e->b_tickets.p ? (uint32_t*)e->b_tickets.p + 2 : nullptr;
  d.error_word = e->d_error;
  d.big_list = (uint32_t*)e->b_big_list.p;
  d.big_count = (uint32_t*)e->b_big_count.p;
  d.big_sx = (long long*)e->b_big_sx.p;
  d.big_sy = (long long*)e->b_big_sy.p;
  d.big_ns = (uint32_t*)e->b_big_ns.p;
  d.rec = (float4*)e->b_rec.p;
  d.acc = (long long*)e->b_acc.p;
  std::memcpy(d.level_off, e->level_off, sizeof(d.level_off));
  std::memcpy(d.acc_off, e->acc_off, sizeof(d.acc_off));
  d.centroid = (long long*)e->b_centroid.p;
  d.tick_params = (const TickParams*)e->b_params.p;
  d.tick_ctr = (uint32_t*)e->b_tick_ctr.p;
  d.rowptr_in = (const uint32_t*)e->b_rowptr_in.p;
  d.ent_in = (const uint4*)e->b_ent_in.p;
  d.rowptr_out = (const uint32_t*)e->b_rowptr_out.p;
  d.ent_out = (const uint4*)e->b_ent_out.p;
  d.heavy_in = (const uint32_t*)e->b_heavy_in.p;
  d.heavy_out = (const uint32_t*)e->b_heavy_out.p;
  d.n_heavy_in = e->n_heavy_in;
  d.n_heavy_out = e->n_heavy_out;
  d.early_pts = (const uint32_t*)e->b_early_pts.p;
  d.n_early_pts = e->n_early_pts;
  d.n_early_hubs = e->n_early_hubs;
  d.n_first_out = e->n_first_out;
  d.n_next_out = e->n_next_out;
  d.inv = e->n_early_hubs ? (uint32_t*)e->b_inv.p : nullptr;
  d.woff_in = (const uint32_t*)e->b_woff_in.p;
  d.lane_ent_in = (const uint4*)e->b_lane_ent_in.p;
  d.woff_out = (const uint32_t*)e->b_woff_out.p;
  d.lane_ent_out = (const uint4*)e->b_lane_ent_out.p;
  d.size = (const float*)e->b_size.p;
  d.cgrid_acc = (long long*)e->b_cgrid_acc.p;
  d.cgrid = (float4*)e->b_cgrid.p;
  d.coll_mark = (uint32_t*)e->b_coll_mark.p;
  d.pos_coll = (float2*)e->b_pos_coll.p;
  d.coll_redo = (uint32_t*)e->b_coll_redo.p;
  d.cluster_of = (const uint32_t*)e->b_cl_of.p;
  d.cluster_coeff = (const float*)e->b_cl_coeff.p;
  d.cluster_custom = (const float2*)e->b_cl_custom.p;
  d.cluster_acc = (long long*)e->b_cl_acc.p;
  d.n_clusters = e->n_clusters;
}

uint32_t device_sms() {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? (uint32_t)sms : 1u;
}

// Without timing: two points of a cell per thread once the cells hold one
// point on average and the graph fills the GPU with one thread per point; a
// point over 16 threads below that size; else a thread per point.
int size_rule_kernel(const cgl_engine* e) {
  const uint64_t full = 2ull * 256 * device_sms();
  if (e->Gf > 0 && e->live >= (uint64_t)e->Gf * e->Gf && e->N >= full) return kManybodyTwoPoints;
  return e->N < full ? kManybodySplit : kManybodyOnePoint;
}

SimScalars make_scalars(const cgl_engine* e) {
  SimScalars s{};
  s.space = (float)e->adjusted_space;
  s.friction = (float)e->cfg.simulation_friction;
  s.gravity = (float)e->cfg.simulation_gravity;
  s.center = (float)e->cfg.simulation_center;
  s.repulsion = (float)e->cfg.simulation_repulsion;
  s.link_spring = (float)e->cfg.simulation_link_spring;
  s.link_distance = (float)e->cfg.simulation_link_distance;
  s.link_r0 = (float)e->cfg.simulation_link_dist_random_variation_range[0];
  s.link_r1 = (float)e->cfg.simulation_link_dist_random_variation_range[1];
  s.coll_strength = (float)e->cfg.simulation_collision;
  const double cr = e->cfg.simulation_collision_radius;
  s.coll_radius = std::isnan(cr) ? 0.f : (float)cr;
  s.coll_padding = (float)e->cfg.simulation_collision_padding;
  s.coll_cell = e->ccell;
  s.coll_grid = e->cgrid;
  s.gf = e->Gf;
  s.levels = e->L;
  s.tile = e->tile;
  s.csf = e->Gf ? (float)(e->adjusted_space / e->Gf) : 1.f;
  s.fx = e->fx;
  s.units = PairUnits{1.0f, -0.0f};
  s.cluster = (float)e->cfg.simulation_cluster;
  // the many-body kernel: the configured one, else the one the tuner kept
  // for this graph, else the size rule
  const int32_t forced = e->cfg.manybody_kernel;
  s.mb_kernel = forced >= 0 ? forced : e->mb_choice >= 0 ? e->mb_choice : size_rule_kernel(e);
  s.pairs = s.mb_kernel == kManybodyTwoPoints;
  s.level_guard = s.csf >= 2.0f && s.space <= 33554432.0f;   // 2^25
  s.any_pinned = e->any_pinned;
  return s;
}

// ------------------------------------------------------------------ tick --
struct TickPlan {
  bool grav, cent, mb, link_in, link_out, coll;
  bool clus, clus_sum;   // the cluster pass runs / needs the centres of mass
};

TickPlan plan_tick(const cgl_engine* e) {
  const uint32_t m = e->cfg.stage_mask;
  TickPlan p{};
  p.grav = e->cfg.simulation_gravity != 0 && (m & CGL_STAGE_GRAVITY) && e->N > 0;
  p.cent = e->cfg.simulation_center != 0 && (m & CGL_STAGE_CENTER) && e->N > 0;
  p.mb = (m & CGL_STAGE_MANYBODY) && e->mb_ready && e->N > 0;
  const bool links = e->W > 0 && e->N > 0;
  p.link_in = links && (m & CGL_STAGE_LINK_IN);
  p.link_out = links && (m & CGL_STAGE_LINK_OUT);
  p.coll = e->cfg.simulation_collision != 0 && (m & CGL_STAGE_COLLISION) && e->N > 0;
  // src/index.ts:2057-2061: runs whenever per-point clusters or cluster positions are set
  p.clus = (e->point_clusters || e->cluster_positions) && (m & CGL_STAGE_CLUSTERS) && e->N > 0;
  p.clus_sum = p.clus && e->point_clusters;
  return p;
}

// Enqueue one tick.  ev (optional) = 2 events per stage for profiling.
cgl_status enqueue_tick(cgl_engine* e, cudaStream_t st, cudaEvent_t* ev) {
  const TickPlan p = plan_tick(e);
  const DeviceView& d = e->view;
  // With early hubs, their points take their many-body terms first; their
  // incoming chains then run on a second stream beside the rest of the
  // many-body pass and of the incoming pass.  Not in a stage profile (ev).
  const bool early = p.mb && p.link_in && !ev && d.n_early_hubs > 0 && d.n_early_pts > 0 && d.inv;
  SimScalars s = make_scalars(e);
  s.skip_early = early;
  auto mark = [&](int stage, int which) {
    if (ev) cudaEventRecord(ev[2 * stage + which], st);
  };
  // With collision right after the link passes (no cluster pass between), the
  // outgoing pass's hub chains run on a second stream while its light rows and
  // then the collision sums of every other point run on this one; the hubs'
  // points are summed once their chains end.  Not in a stage profile (ev).
  const bool overlap =
      p.link_in && p.link_out && p.coll && !p.clus && p.mb && !ev && d.n_heavy_out > 0 && e->b_hub_out.p;
  if (p.cent) CU(cudaMemsetAsync(d.centroid, 0, 3 * sizeof(long long), st));
  if (p.mb) CU(cudaMemsetAsync(d.big_count, 0, 8 * sizeof(uint32_t), st));
  uint32_t mode = 0;
  if (p.grav) mode |= kPreGravity;
  if (p.cent) mode |= kPreCentroid;
  else if (p.mb) mode |= kPreBin;
  mark(0, 0);
  if (mode) launch_prepass(d, s, mode, st);
  mark(0, 1);
  mark(1, 0);
  if (p.cent) launch_center(d, s, p.mb, st);
  mark(1, 1);
  if (p.mb) {
    mark(2, 0); launch_scan(d, s, st); mark(2, 1);
    mark(3, 0); launch_scatter(d, s, st); mark(3, 1);
    mark(4, 0); launch_cells(d, s, st); mark(4, 1);
    mark(5, 0);
    if (early) {
      launch_manybody_early(d, s, st);
      CU(cudaEventRecord(e->fork, st));
      CU(cudaStreamWaitEvent(e->side, e->fork, 0));
      launch_link(d, s, 0, false, e->side, kLinkFirstHubs);
      CU(cudaEventRecord(e->join, e->side));
    }
    launch_manybody(d, s, st);
    mark(5, 1);
  }
  if (p.link_in || p.link_out) {
    mark(6, 0);
    if (p.link_in) launch_link(d, s, 0, false, st, early ? kLinkAfterFirst : kLinkAll);
    if (early) CU(cudaStreamWaitEvent(st, e->join, 0));
    mark(6, 1);
    mark(7, 0);
    if (p.link_out) {
      // The leading outgoing hubs on the second stream, an SM each, beside the
      // rest of the pass; with the overlap all hub CTAs go there when no list
      // leads, beside the light rows.
      const bool first_out = !ev && d.n_first_out > 0;
      const bool next_out = first_out && d.n_next_out > 0;
      const bool split = first_out || overlap;
      if (split) {
        CU(cudaEventRecord(e->fork, st));
        CU(cudaStreamWaitEvent(e->side, e->fork, 0));
        launch_link(d, s, 1, p.link_in, e->side, first_out ? kLinkFirstHubs : kLinkHubs);
        CU(cudaEventRecord(e->join, e->side));
        if (next_out) {   // the next hubs on a third stream: their chains leave this one to the sums
          CU(cudaStreamWaitEvent(e->side2, e->fork, 0));
          launch_link(d, s, 1, p.link_in, e->side2, kLinkNextHubs);
          CU(cudaEventRecord(e->join2, e->side2));
        }
      }
      launch_link(d, s, 1, p.link_in, st, first_out ? kLinkAfterFirst : overlap ? kLinkLight : kLinkAll);
      if (overlap) {
        // the points on the second stream ("late": the leading hubs, else every
        // hub) are marked in b_hub_out and summed once their chains end
        const uint8_t* late = (const uint8_t*)e->b_hub_out.p;
        const uint32_t n_late = first_out ? d.n_first_out + d.n_next_out : d.n_heavy_out;
        launch_collision_sums(d, s, d.sorted_idx, (uint32_t)e->live, late, st);
        if (first_out && d.pos_coll && d.coll_mark && d.coll_redo) {
          // every other point's result beside the chains; then the late points'
          // and those of the points whose windows hold a late point's cell
          launch_collision_convert(d, s, st, false);
          launch_collision_force_early(d, s, d.sorted_idx, (uint32_t)e->live, late, st);
          CU(cudaStreamWaitEvent(st, e->join, 0));
          if (next_out) CU(cudaStreamWaitEvent(st, e->join2, 0));
          launch_collision_sums(d, s, d.heavy_out, n_late, nullptr, st);
          launch_collision_late(d, s, d.heavy_out, n_late, st);
          launch_collision_fixup(d, s, late, st);
          CU(cudaMemsetAsync(d.cgrid_acc, 0, e->b_cgrid_acc.bytes, st));
          CU(cudaMemsetAsync(d.coll_mark, 0, e->b_coll_mark.bytes, st));
          CU(cudaMemsetAsync(d.coll_redo, 0, sizeof(uint32_t), st));
        } else {
          CU(cudaStreamWaitEvent(st, e->join, 0));
          if (next_out) CU(cudaStreamWaitEvent(st, e->join2, 0));
          launch_collision_sums(d, s, d.heavy_out, n_late, nullptr, st);
          launch_collision_convert(d, s, st);
          launch_collision_force(d, s, d.sorted_idx, (uint32_t)e->live, st);
        }
      } else if (split) {
        CU(cudaStreamWaitEvent(st, e->join, 0));
        if (next_out) CU(cudaStreamWaitEvent(st, e->join2, 0));
      }
    }
    mark(7, 1);
    if (!(p.link_in && p.link_out))
      CU(cudaMemcpyAsync(d.pos, d.pos_alt, e->N * sizeof(float2), cudaMemcpyDeviceToDevice, st));
  }
  if (p.clus) {
    mark(10, 0);
    if (p.clus_sum) {
      CU(cudaMemsetAsync(d.cluster_acc, 0, 3 * (size_t)e->n_clusters * sizeof(long long), st));
      launch_cluster_sum(d, s, st);
    }
    launch_cluster_force(d, s, st);
    mark(10, 1);
  }
  if (p.coll && !overlap) {
    // the many-body pass left every live point in sorted_idx, grouped by cell
    const uint32_t* order = p.mb ? d.sorted_idx : nullptr;
    mark(8, 0); launch_collision_grid(d, s, order, (uint32_t)e->live, st); mark(8, 1);
    mark(9, 0); launch_collision_force(d, s, order, (uint32_t)e->live, st); mark(9, 1);
  }
  launch_tick_end(d, st);
  CU(cudaGetLastError());
  return CGL_OK;
}

cgl_status collision_create(cgl_engine* e) {
  // ForceCollision.create (ForceCollision/index.ts:61-148)
  double max_size = e->cfg.point_default_size;
  std::vector<float> sizes(e->N);
  for (uint64_t i = 0; i < e->N; ++i) {
    sizes[i] = resolved_size(e, i);
    if (e->has_data_sizes) max_size = std::max(max_size, (double)sizes[i]);
  }
  const double cr = std::isnan(e->cfg.simulation_collision_radius) ? 0 : e->cfg.simulation_collision_radius;
  const double pad = e->cfg.simulation_collision_padding;
  const double eff = (cr > 0 ? cr : max_size * 0.5) + pad;
  const double cell = std::max(eff * 2, 8.0);
  const int grid = (int)std::min(512.0, std::max(1.0, std::floor(e->adjusted_space / cell)));
  e->cgrid = grid;
  e->ccell = (float)(e->adjusted_space / grid);
  const size_t cells = 4 * (size_t)grid * grid;
  cgl_status st;
  if ((st = dev_reserve(e, e->b_size, e->N * sizeof(float), false))) return st;
  if ((st = dev_reserve(e, e->b_cgrid_acc, cells * 4 * sizeof(long long), true))) return st;
  if ((st = dev_reserve(e, e->b_cgrid, cells * sizeof(float4), false))) return st;
  if ((st = dev_reserve(e, e->b_coll_mark, (cells + 31) / 32 * sizeof(uint32_t), true))) return st;
  if (e->N) CU(cudaMemcpyAsync(e->b_size.p, sizes.data(), e->N * sizeof(float), cudaMemcpyHostToDevice, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  e->collision_ready = true;
  refresh_view(e);
  return CGL_OK;
}

cgl_status prepare_tick(cgl_engine* e) {
  const TickPlan p = plan_tick(e);
  if (p.coll && !e->collision_ready) {
    cgl_status st = collision_create(e);
    if (st) return st;
    e->graph_dirty = true;
  }
  if (!e->use_graph) return CGL_OK;
  if (!e->graph_dirty && e->graph) return CGL_OK;
  if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
  cudaGraph_t g = nullptr;
  CU(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  cgl_status st = enqueue_tick(e, e->stream, nullptr);
  cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
  if (st) { if (g) cudaGraphDestroy(g); return st; }
  if (ce != cudaSuccess) return fail(e, CGL_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(ce));
  // node priorities as captured: the hub chains' stream goes first (enqueue_tick)
  ce = cudaGraphInstantiate(&e->graph, g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) { e->graph = nullptr; return fail(e, CGL_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(ce)); }
  e->graph_dirty = false;
  return CGL_OK;
}

// Host side of one tick: the f32 alpha uniform and the peel seed draw
// (ForceManyBody/index.ts:521), then Store.addAlpha (Store/index.ts:328-332).
// Right-click repulsion is on (src/index.ts:2011, 2083)
bool mouse_active(const cgl_engine* e) { return e->right_button && e->cfg.enable_right_click_repulsion; }
bool dragging(const cgl_engine* e) {
  return e->drag_index >= 0 && e->drag_index < (int64_t)e->N && e->cfg.enable_drag;   // the index of this graph
}
bool interactive(const cgl_engine* e) { return mouse_active(e) || dragging(e); }

void launch_pointer_force(cgl_engine* e) {
  launch_mouse(e->view, make_scalars(e), make_float2((float)e->mouse_x, (float)e->mouse_y),
               (float)e->cfg.simulation_repulsion_from_mouse, e->stream);
}

TickParams host_tick(cgl_engine* e, bool draws_seed) {
  TickParams tp;
  tp.alpha = (float)e->alpha;
  tp.seed_bits = 0;
  if (draws_seed) {
    const float seed = (float)e->rnd(0, 1);
    std::memcpy(&tp.seed_bits, &seed, 4);
  }
  e->alpha += (0 - e->alpha) * (1 - std::pow(kAlphaMin, 1 / e->cfg.simulation_decay));
  if (mouse_active(e)) e->alpha = std::max(e->alpha, 0.1);   // src/index.ts:2083-2085
  e->progress = std::sqrt(std::min(1.0, kAlphaMin / e->alpha));
  e->tick++;
  return tp;
}

// The many-body kernels a graph is timed with: a thread per point always; a
// point over 16 threads while the graph is under four GPU-fulls of 512
// points a SM; two points of a cell per thread from half a point a cell.
std::vector<int> tune_candidates(const cgl_engine* e) {
  std::vector<int> c{kManybodyOnePoint};
  if (e->N < 4ull * 2 * 256 * device_sms()) c.push_back(kManybodySplit);
  if (e->Gf > 0 && 2 * e->live >= (uint64_t)e->Gf * e->Gf) c.push_back(kManybodyTwoPoints);
  return c;
}

bool tuning(const cgl_engine* e, const cudaEvent_t* ev) {
  return e->cfg.manybody_kernel == CGL_MANYBODY_AUTO && !e->mb_tuned && e->use_graph && !ev && plan_tick(e).mb;
}

// Ticks per candidate; the first after a candidate's graph is built carries
// its first launch and is not counted.  A candidate replaces the size rule's
// kernel only when it is kTuneMargin faster: two kernels within the margin
// are kept as the rule has them, not swapped on timing noise.
constexpr uint32_t kTuneTicks = 3;
constexpr float kTuneMargin = 0.97f;

// One tick of the tuning: the next candidate's graph, timed with events.
// *ran: whether a tick ran (with a single candidate there is nothing to time).
cgl_status tune_tick(cgl_engine* e, bool* ran) {
  *ran = false;
  if (e->tune_cands.empty()) {
    e->tune_cands = tune_candidates(e);
    e->tune_next = 0;
    if (e->tune_cands.size() == 1) {   // nothing to choose
      e->mb_choice = e->tune_cands[0];
      e->mb_tuned = true;
      e->graph_dirty = true;
      return CGL_OK;
    }
  }
  const uint32_t idx = e->tune_next / kTuneTicks;
  if (e->mb_choice != e->tune_cands[idx]) {
    e->mb_choice = e->tune_cands[idx];
    e->graph_dirty = true;
  }
  cgl_status st = prepare_tick(e);
  if (st) return st;
  if (e->params_pending) { CU(cudaEventSynchronize(e->params_copied)); e->params_pending = false; }
  e->h_params[0] = host_tick(e, plan_tick(e).mb);
  CU(cudaMemcpyAsync(e->b_params.p, e->h_params, sizeof(TickParams), cudaMemcpyHostToDevice, e->stream));
  CU(cudaEventRecord(e->params_copied, e->stream));
  e->params_pending = true;
  CU(cudaMemsetAsync(e->b_tick_ctr.p, 0, sizeof(uint32_t), e->stream));
  if (mouse_active(e)) launch_pointer_force(e);
  CU(cudaEventRecord(e->tune_ev[0], e->stream));
  CU(cudaGraphLaunch(e->graph, e->stream));
  CU(cudaEventRecord(e->tune_ev[1], e->stream));
  CU(cudaEventSynchronize(e->tune_ev[1]));
  float ms = 0.f;
  CU(cudaEventElapsedTime(&ms, e->tune_ev[0], e->tune_ev[1]));
  e->tune_ms[idx][e->tune_next % kTuneTicks] = ms;
  *ran = true;
  if (++e->tune_next == kTuneTicks * e->tune_cands.size()) {
    auto best_of = [&](size_t k) { return std::min(e->tune_ms[k][1], e->tune_ms[k][2]); };   // [0]: first launch
    const int rule = size_rule_kernel(e);
    size_t pick = 0, fastest = 0;
    for (size_t k = 0; k < e->tune_cands.size(); ++k) {
      if (e->tune_cands[k] == rule) pick = k;
      if (best_of(k) < best_of(fastest)) fastest = k;
    }
    if (best_of(fastest) < kTuneMargin * best_of(pick)) pick = fastest;
    if (e->mb_choice != e->tune_cands[pick]) e->graph_dirty = true;
    e->mb_choice = e->tune_cands[pick];
    e->mb_tuned = true;
  }
  return CGL_OK;
}

cgl_status run_ticks(cgl_engine* e, uint32_t ticks, cudaEvent_t* ev, double* stage_ms) {
  while (ticks > 0 && tuning(e, ev)) {   // a graph's first ticks time the many-body kernels
    bool ran = false;
    cgl_status st = tune_tick(e, &ran);
    if (st) return st;
    if (ran) --ticks;
  }
  if (ticks == 0) return CGL_OK;
  cgl_status st = prepare_tick(e);
  if (st) return st;
  const bool seed = plan_tick(e).mb;
  const bool mouse = mouse_active(e);   // ForceMouse pass before each tick's forces
  uint32_t done = 0;
  while (done < ticks) {
    const uint32_t n = std::min(kParamChunk, ticks - done);
    if (e->params_pending) { CU(cudaEventSynchronize(e->params_copied)); e->params_pending = false; }
    for (uint32_t t = 0; t < n; ++t) e->h_params[t] = host_tick(e, seed);
    CU(cudaMemcpyAsync(e->b_params.p, e->h_params, n * sizeof(TickParams), cudaMemcpyHostToDevice, e->stream));
    CU(cudaEventRecord(e->params_copied, e->stream));
    e->params_pending = true;
    CU(cudaMemsetAsync(e->b_tick_ctr.p, 0, sizeof(uint32_t), e->stream));
    for (uint32_t t = 0; t < n; ++t) {
      if (mouse) launch_pointer_force(e);
      if (ev) {
        st = enqueue_tick(e, e->stream, ev);
        if (st) return st;
        CU(cudaStreamSynchronize(e->stream));
        for (int k = 0; k < CGL_NUM_STAGE_TIMES; ++k) {
          float ms = 0.f;
          if (cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]) == cudaSuccess) stage_ms[k] += ms;
        }
        cudaGetLastError();
      } else if (e->use_graph) {
        CU(cudaGraphLaunch(e->graph, e->stream));
      } else {
        st = enqueue_tick(e, e->stream, nullptr);
        if (st) return st;
      }
    }
    done += n;
  }
  return CGL_OK;
}

// ForceLink.create(INCOMING) then (OUTGOING) built on the device
// (ingest_device.cu); the same lists, draws and order as ingest::build_links.
cgl_status build_links_device(cgl_engine* e, uint64_t E64, size_t n) {
  using namespace dingest;
  cudaStream_t st = e->stream;
  const uint32_t E = (uint32_t)E64, N = (uint32_t)n;
  DevBuf t_links, t_str, t_valid, t_len_in, t_len_out, t_kin, t_kout, t_vin, t_vout, t_tmp, t_stats, t_draws;
  DevBuf* temps[] = {&t_links, &t_str, &t_valid, &t_len_in, &t_len_out, &t_kin, &t_kout, &t_vin, &t_vout, &t_tmp,
                     &t_stats, &t_draws};
  auto done = [&](cgl_status rc) {
    for (DevBuf* b : temps) dev_release(e, *b);
    return rc;
  };
  cgl_status rc;
  // a CUDA error releases the temporaries before returning
#define TCU(call)                                                                              \
  do {                                                                                         \
    cudaError_t _err = (call);                                                                 \
    if (_err != cudaSuccess)                                                                   \
      return done(fail(e, _err == cudaErrorMemoryAllocation ? CGL_OOM : CGL_CUDA_ERROR, "%s: %s", #call, \
                       cudaGetErrorString(_err)));                                             \
  } while (0)
  const uint64_t big = std::max<uint64_t>(E64 + 1, n + 1);
  const size_t tmp_words = std::max(sort_temp_words(big), scan_temp_words(big));
  if ((rc = dev_reserve(e, t_links, E64 * sizeof(float2), false)) ||
      (rc = dev_reserve(e, t_valid, (E64 + 1) * sizeof(uint32_t), true)) ||
      (rc = dev_reserve(e, t_len_in, (n + 1) * sizeof(uint32_t), true)) ||
      (rc = dev_reserve(e, t_len_out, (n + 1) * sizeof(uint32_t), true)) ||
      (rc = dev_reserve(e, t_tmp, tmp_words * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, t_stats, 4 * sizeof(uint32_t), true)))
    return done(rc);
  if (cudaMemcpyAsync(t_links.p, e->in_links.data(), E64 * sizeof(float2), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return done(fail(e, CGL_CUDA_ERROR, "link upload failed"));
  const float* strength = nullptr;
  if (e->has_strength) {
    if ((rc = dev_reserve(e, t_str, E64 * sizeof(float), false))) return done(rc);
    if (cudaMemcpyAsync(t_str.p, e->in_strength.data(), E64 * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return done(fail(e, CGL_CUDA_ERROR, "link strength upload failed"));
    strength = (const float*)t_str.p;
  }
  const float2* links = (const float2*)t_links.p;
  uint32_t* valid = (uint32_t*)t_valid.p;
  uint32_t* len_in = (uint32_t*)t_len_in.p;
  uint32_t* len_out = (uint32_t*)t_len_out.p;
  uint32_t* tmp = (uint32_t*)t_tmp.p;
  uint32_t* stats = (uint32_t*)t_stats.p;
  count_links(links, E, N, valid, len_in, len_out, st);
  scan_exclusive(valid, E + 1, tmp, st);
  len_stats(len_in, N, stats, st);
  len_stats(len_out, N, stats + 2, st);
  uint32_t h[5];
  TCU(cudaMemcpyAsync(h, valid + E, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  TCU(cudaMemcpyAsync(h + 1, stats, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  TCU(cudaStreamSynchronize(st));
  const uint32_t M = h[0];
  const size_t pairs = std::max<size_t>(M, n);   // the pair buffers also hold the length sort
  if ((rc = dev_reserve(e, t_kin, pairs * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, t_kout, pairs * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, t_vin, pairs * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, t_vout, pairs * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, e->b_ent_in, (size_t)M * sizeof(uint4), false)) ||
      (rc = dev_reserve(e, e->b_ent_out, (size_t)M * sizeof(uint4), false)) ||
      (rc = dev_reserve(e, e->b_rowptr_in, (n + 1) * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, e->b_rowptr_out, (n + 1) * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, e->b_heavy_in, n * sizeof(uint32_t), false)) ||
      (rc = dev_reserve(e, e->b_heavy_out, n * sizeof(uint32_t), false)))
    return done(rc);
  uint32_t *kin = (uint32_t*)t_kin.p, *kout = (uint32_t*)t_kout.p, *vin = (uint32_t*)t_vin.p, *vout = (uint32_t*)t_vout.p;
  compact_links(links, E, valid, kin, kout, vin, vout, st);
  const int row_bits = key_bits(n ? n - 1 : 0);
  sort_pairs(kin, vin, M, row_bits, tmp, st);
  sort_pairs(kout, vout, M, row_bits, tmp, st);
  const uint64_t base = e->rng.ctr;
  const float* draws_in = nullptr;
  const float* draws_out = nullptr;
  if (!e->rng.counter && M) {
    // The reference's stream is sequential: draw both directions' values on the
    // host (entry order, incoming first) while the sorts run, then upload them.
    std::vector<float> h_draws(2 * (size_t)M);
    e->rng.fill_unit_f32(h_draws.data(), 2 * (uint64_t)M);
    if ((rc = dev_reserve(e, t_draws, 2 * (size_t)M * sizeof(float), false))) return done(rc);
    TCU(cudaMemcpyAsync(t_draws.p, h_draws.data(), 2 * (size_t)M * sizeof(float), cudaMemcpyHostToDevice, st));
    TCU(cudaStreamSynchronize(st));   // h_draws is pageable and about to go
    draws_in = (const float*)t_draws.p;
    draws_out = draws_in + M;
  } else {
    e->rng.ctr += 2 * (uint64_t)M;
  }
  fill_csr(kin, vin, M, links, true, len_in, len_out, strength, (const uint8_t*)e->b_flags.p, draws_in, e->rng.seed,
           base, 0, (uint4*)e->b_ent_in.p, st);
  fill_csr(kout, vout, M, links, false, len_in, len_out, strength, (const uint8_t*)e->b_flags.p, draws_out,
           e->rng.seed, base + M, 0, (uint4*)e->b_ent_out.p, st);
  // rowptr = exclusive scan of the list lengths (len[n] = 0 makes rowptr[n] = M)
  copy_u32(len_in, (uint32_t*)e->b_rowptr_in.p, N + 1, st);
  scan_exclusive((uint32_t*)e->b_rowptr_in.p, N + 1, tmp, st);
  copy_u32(len_out, (uint32_t*)e->b_rowptr_out.p, N + 1, st);
  scan_exclusive((uint32_t*)e->b_rowptr_out.p, N + 1, tmp, st);
  // points by list length, longest first, ties by index
  len_keys(len_in, N, stats, kin, (uint32_t*)e->b_heavy_in.p, st);
  sort_pairs(kin, (uint32_t*)e->b_heavy_in.p, N, key_bits(h[1]), tmp, st);
  len_keys(len_out, N, stats + 2, kout, (uint32_t*)e->b_heavy_out.p, st);
  sort_pairs(kout, (uint32_t*)e->b_heavy_out.p, N, key_bits(h[3]), tmp, st);
  TCU(cudaGetLastError());
  TCU(cudaStreamSynchronize(st));
  e->entries = M;
  e->max_deg_in = h[1];
  e->n_heavy_in = h[2];
  e->max_deg_out = h[3];
  e->n_heavy_out = h[4];
  return done(CGL_OK);
}
#undef TCU

// The light rows of both directions by warps (DeviceView::woff_*, lane_ent_*),
// from the CSR and the order: a warp's block holds entry k of its 32 lists at
// 32 k + lane, so the link pass loads one entry of every lane at once.
cgl_status build_link_warps(cgl_engine* e) {
  const uint32_t n = (uint32_t)e->N;
  cudaStream_t st = e->stream;
  DevBuf t_tmp;
  cgl_status rc = CGL_OK;
  for (int dir = 0; dir < 2 && rc == CGL_OK; ++dir) {
    const uint32_t nhub = dir == 0 ? e->n_heavy_in : e->n_heavy_out;
    const uint32_t nw = (n - nhub + 31) / 32;
    DevBuf& woff = dir == 0 ? e->b_woff_in : e->b_woff_out;
    DevBuf& lanes = dir == 0 ? e->b_lane_ent_in : e->b_lane_ent_out;
    const uint32_t* order = (const uint32_t*)(dir == 0 ? e->b_heavy_in.p : e->b_heavy_out.p);
    const uint32_t* rowptr = (const uint32_t*)(dir == 0 ? e->b_rowptr_in.p : e->b_rowptr_out.p);
    const uint4* ent = (const uint4*)(dir == 0 ? e->b_ent_in.p : e->b_ent_out.p);
    if ((rc = dev_reserve(e, woff, (nw + 1) * sizeof(uint32_t), true))) break;
    if ((rc = dev_reserve(e, t_tmp, dingest::scan_temp_words(nw + 1) * sizeof(uint32_t), false))) break;
    uint32_t total = 0;
    if (nw) {
      launch_warp_lengths(order, rowptr, nhub, n, (uint32_t*)woff.p, st);
      dingest::scan_exclusive((uint32_t*)woff.p, nw + 1, (uint32_t*)t_tmp.p, st);
      cudaError_t err = cudaMemcpyAsync(&total, (uint32_t*)woff.p + nw, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
      if (err == cudaSuccess) err = cudaStreamSynchronize(st);
      if (err != cudaSuccess) { rc = fail(e, CGL_CUDA_ERROR, "link warp layout: %s", cudaGetErrorString(err)); break; }
    }
    if ((rc = dev_reserve(e, lanes, std::max<size_t>(total, 1) * sizeof(uint4), false))) break;
    if (total) launch_fill_lanes(order, rowptr, ent, nhub, n, (const uint32_t*)woff.p, (uint4*)lanes.p, st);
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) rc = fail(e, CGL_CUDA_ERROR, "link warp layout: %s", cudaGetErrorString(err));
  }
  if (rc == CGL_OK) {
    const cudaError_t err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) rc = fail(e, CGL_CUDA_ERROR, "link warp layout: %s", cudaGetErrorString(err));
  }
  dev_release(e, t_tmp);
  return rc;
}

// Device flags from the pinned, absent and early marks.
cgl_status upload_flags(cgl_engine* e) {
  if (!e->N) return CGL_OK;
  const bool with_early = e->early.size() == e->N;
  std::vector<uint8_t> flags(e->N);
  for (uint64_t i = 0; i < e->N; ++i)
    flags[i] = (e->pinned[i] ? kPinned : 0) | (e->absent[i] ? kAbsent : 0) | (with_early && e->early[i] ? kEarly : 0);
  CU(cudaMemcpyAsync(e->b_flags.p, flags.data(), e->N, cudaMemcpyHostToDevice, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return CGL_OK;
}

// Leading hubs: the first lists of a direction's order (longest first) of at
// least kLeadMinLinks links and a fraction of the longest, at most
// kLeadCandidates of them (or the test hook's limit).  Their chains each run
// on an SM of their own on the second stream.  Incoming (early hubs): half the
// longest, while their links total at most an eighth of the points.  Their
// chains need the many-body results of their own points and link targets
// only; those run first, and the chains then start beside the rest of the
// many-body pass instead of after it.  More of them take SMs from that pass
// (R-MAT 2^23: 24 early hubs, 0.15-0.2 ms a tick slower than 1 to 4).
// Outgoing: half the longest on SMs of their own, then down to a quarter of
// the longest on a third stream (their SMs shared): the rest of the pass and
// the collision results of every other point run beside them.
constexpr uint32_t kLeadCandidates = 32;
constexpr uint32_t kLeadMinLinks = 4096;

// spans (rowptr[p], rowptr[p + 1]) and points p of the leading hubs of a
// direction; returns their count (0 when none qualifies).
cgl_status leading_hubs(cgl_engine* e, int dir, uint32_t fraction, uint64_t max_total, std::vector<uint2>& spans,
                        std::vector<uint32_t>& hubs, uint32_t* count) {
  *count = 0;
  const uint32_t nheavy = dir == 0 ? e->n_heavy_in : e->n_heavy_out;
  const uint32_t* order = (const uint32_t*)(dir == 0 ? e->b_heavy_in.p : e->b_heavy_out.p);
  const uint32_t* rowptr = (const uint32_t*)(dir == 0 ? e->b_rowptr_in.p : e->b_rowptr_out.p);
  uint32_t m = std::min(nheavy, kLeadCandidates);
  if (e->lead_limit[dir] >= 0) m = std::min(m, (uint32_t)e->lead_limit[dir]);
  if (!m) return CGL_OK;
  DevBuf t_spans;
  cgl_status rc;
  if ((rc = dev_reserve(e, t_spans, m * sizeof(uint2), false))) return rc;
  spans.resize(m);
  hubs.resize(m);
  launch_hub_spans(order, rowptr, m, (uint2*)t_spans.p, e->stream);
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(spans.data(), t_spans.p, m * sizeof(uint2), cudaMemcpyDeviceToHost, e->stream);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(hubs.data(), order, m * sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
  dev_release(e, t_spans);
  if (err != cudaSuccess) return fail(e, CGL_CUDA_ERROR, "leading hubs: %s", cudaGetErrorString(err));
  // the test hook's limit takes the leading lists whatever their lengths
  const uint32_t least =
      e->lead_limit[dir] >= 0 ? 1u : std::max(kLeadMinLinks, (spans[0].y - spans[0].x) / fraction);
  uint64_t total = 0;
  uint32_t k = 0;
  for (; k < m; ++k) {
    const uint32_t len = spans[k].y - spans[k].x;
    if (len < least || total + len > max_total) break;
    total += len;
  }
  *count = k;
  return CGL_OK;
}

cgl_status build_early(cgl_engine* e) {
  e->n_early_hubs = e->n_early_pts = e->n_first_out = e->n_next_out = 0;
  e->early.clear();
  const uint32_t n = (uint32_t)e->N;
  cgl_status rc = CGL_OK;
  std::vector<uint2> spans;
  std::vector<uint32_t> hubs;
  uint32_t k = 0, k4 = 0;
  if (e->T && (rc = leading_hubs(e, 1, 2, ~0ull, spans, hubs, &k))) return rc;
  if (e->T && (rc = leading_hubs(e, 1, 4, ~0ull, spans, hubs, &k4))) return rc;
  e->n_first_out = k;
  e->n_next_out = k ? k4 - k : 0;
  k = 0;
  if (e->T && (rc = leading_hubs(e, 0, 2, n / 8, spans, hubs, &k))) return rc;
  if (k) {
    uint64_t total = 0;
    for (uint32_t t = 0; t < k; ++t) total += spans[t].y - spans[t].x;
    std::vector<uint4> ent(total);
    size_t at = 0;
    cudaError_t err = cudaSuccess;
    for (uint32_t t = 0; t < k && err == cudaSuccess; ++t) {
      const uint32_t len = spans[t].y - spans[t].x;
      err = cudaMemcpyAsync(ent.data() + at, (const uint4*)e->b_ent_in.p + spans[t].x, len * sizeof(uint4),
                            cudaMemcpyDeviceToHost, e->stream);
      at += len;
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
    if (err != cudaSuccess) return fail(e, CGL_CUDA_ERROR, "early hubs: %s", cudaGetErrorString(err));
    e->early.assign(n, 0);
    for (uint32_t t = 0; t < k; ++t)
      if (!e->absent[hubs[t]]) e->early[hubs[t]] = 1;
    for (const uint4& en : ent)
      if (en.x < n && !e->absent[en.x]) e->early[en.x] = 1;
    std::vector<uint32_t> pts;
    for (uint32_t i = 0; i < n; ++i)
      if (e->early[i]) pts.push_back(i);
    if ((rc = dev_reserve(e, e->b_early_pts, std::max<size_t>(pts.size(), 1) * sizeof(uint32_t), false)) ||
        (rc = dev_reserve(e, e->b_inv, (size_t)n * sizeof(uint32_t), false))) {
      e->early.clear();
      return rc;
    }
    const uint32_t np = (uint32_t)pts.size();
    if (np) {
      CU(cudaMemcpyAsync(e->b_early_pts.p, pts.data(), np * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
      // by finest cell of their positions now: the early pass then walks them
      // in (roughly) the order the cells hold them
      DevBuf t_keys, t_tmp;
      if ((rc = dev_reserve(e, t_keys, np * sizeof(uint32_t), false)) ||
          (rc = dev_reserve(e, t_tmp, dingest::sort_temp_words(np) * sizeof(uint32_t), false))) {
        dev_release(e, t_keys);
        e->early.clear();
        return rc;
      }
      const SimScalars s = make_scalars(e);
      launch_cell_keys((const float2*)e->b_pos.p, (const uint32_t*)e->b_early_pts.p, np, s.csf, s.gf,
                       (uint32_t*)t_keys.p, e->stream);
      dingest::sort_pairs((uint32_t*)t_keys.p, (uint32_t*)e->b_early_pts.p, np,
                          dingest::key_bits((uint64_t)e->Gf * e->Gf), (uint32_t*)t_tmp.p, e->stream);
      err = cudaGetLastError();
      if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
      dev_release(e, t_keys);
      dev_release(e, t_tmp);
      if (err != cudaSuccess) return fail(e, CGL_CUDA_ERROR, "early points: %s", cudaGetErrorString(err));
    }
    e->n_early_hubs = k;
    e->n_early_pts = np;
  }
  if (!e->n_early_hubs) {
    dev_release(e, e->b_early_pts);
    dev_release(e, e->b_inv);
  }
  // the points whose outgoing chains run on the second stream (the leading
  // hubs, else every hub): their collision sums wait for those chains
  if ((rc = dev_reserve(e, e->b_hub_out, std::max<size_t>(n, 1), false))) return rc;
  CU(cudaMemsetAsync(e->b_hub_out.p, 0, std::max<size_t>(n, 1), e->stream));
  launch_mark_hubs((const uint32_t*)e->b_heavy_out.p,
                   e->n_first_out ? e->n_first_out + e->n_next_out : e->n_heavy_out, (uint8_t*)e->b_hub_out.p,
                   e->stream);
  CU(cudaGetLastError());
  if (e->n_first_out) {
    if ((rc = dev_reserve(e, e->b_pos_coll, std::max<size_t>(n, 1) * sizeof(float2), false)) ||
        (rc = dev_reserve(e, e->b_coll_redo, ((size_t)n + 1) * sizeof(uint32_t), true)))
      return rc;
  } else {
    dev_release(e, e->b_pos_coll);
    dev_release(e, e->b_coll_redo);
  }
  return upload_flags(e);
}

cgl_status apply_pinned(cgl_engine* e) {
  // Points.updatePinnedStatus (Points/index.ts:1264-1277) -> device flags
  e->pinned.assign(e->N, 0);
  if (e->pinned_set)
    for (double v : e->pinned_input)
      if (v >= 0 && v < (double)e->N && v == std::floor(v)) e->pinned[(size_t)v] = 1;
  bool any = false;
  for (uint64_t i = 0; i < e->N; ++i) any |= e->pinned[i] && !e->absent[i];
  if (any != e->any_pinned) e->graph_dirty = true;   // the tick kernels take it as a constant
  e->any_pinned = any;
  if (!e->N) return CGL_OK;
  return upload_flags(e);
}

// A render that fails part way (a refused or failed allocation, a CUDA error)
// can leave buffers of the old graph's sizes under the new graph's counts.
// The engine then forgets the graph, as before its first render: no tick,
// read-back or texture touches a buffer until a render succeeds, and every
// staged input stays dirty, so the next render builds all of it again.  The
// random stream goes back to where the failed render found it, so the next
// render draws what an uninterrupted one would have.
void forget_graph(cgl_engine* e) {
  e->N = e->E = 0;
  e->T = e->W = 0;
  e->Gf = e->L = 0;
  e->live = 0;
  e->entries = 0;
  e->max_deg_in = e->max_deg_out = 0;
  e->n_heavy_in = e->n_heavy_out = 0;
  e->n_early_hubs = e->n_early_pts = e->n_first_out = e->n_next_out = 0;
  e->early.clear();
  e->mb_ready = false;
  e->collision_ready = false;
  e->point_clusters = e->cluster_positions = false;
  e->n_clusters = 0;
  e->running = false;
  e->pos_dirty = e->links_dirty = e->sizes_dirty = e->clusters_dirty = true;
  e->graph_dirty = true;
  refresh_view(e);
}

cgl_status build_graph(cgl_engine* e, double alpha, uint64_t N, uint64_t E);

cgl_status do_render(cgl_engine* e, double alpha) {
  // GraphData.update (GraphData/index.ts:443-462)
  const uint64_t N = e->have_pos_input ? e->in_pos.size() / 2 : 0;
  const uint64_t E = e->have_link_input ? e->in_links.size() / 2 : 0;
  if (N == 0 && E == 0) return CGL_OK;   // empty render (src/index.ts:941-955)
  if (N > (1ull << 24)) return fail(e, CGL_INVALID_ARG, "%llu points: point indices must stay exact in f32 (max 2^24)", (unsigned long long)N);
  if (E > 0xFFFFFFF0ull) return fail(e, CGL_INVALID_ARG, "too many links");
  const ingest::Rng rng = e->rng;
  const cgl_status st = build_graph(e, alpha, N, E);
  if (st != CGL_OK) {
    e->rng = rng;
    forget_graph(e);
  }
  return st;
}

cgl_status build_graph(cgl_engine* e, double alpha, uint64_t N, uint64_t E) {
  const bool pos_changed = e->pos_dirty;
  const bool links_changed = e->links_dirty || pos_changed;
  cgl_status st;
  if (links_changed) {   // the leading hubs are chosen again from the new lists
    e->n_early_hubs = e->n_early_pts = e->n_first_out = e->n_next_out = 0;
    e->early.clear();
  }
  if (pos_changed) e->N = N;
  e->E = E;
  e->has_strength = e->have_strength && e->in_strength.size() == E;
  e->has_data_sizes = e->have_sizes;
  e->data_sizes = e->in_sizes;
  // Graph.update (src/index.ts:1987-1994)
  e->T = (uint32_t)std::ceil(std::sqrt((double)e->N));
  e->W = (uint32_t)std::ceil(std::sqrt((double)e->E * 2));
  const size_t n = e->N;
  if (pos_changed) {
    e->graph_dirty = true;
    // Points.updatePositions (Points/index.ts:390-592): the optional rescale
    // (:396-413), then absence and the position texture
    std::vector<float2> pos;
    if (ingest::should_rescale(e->cfg, e->skip_rescale)) {
      std::vector<float> xy(e->in_pos);
      ingest::rescale_positions(xy.data(), n, e->cfg.space_size);
      e->live = ingest::canonical_positions(xy.data(), n, pos, e->absent);
    } else {
      e->live = ingest::canonical_positions(e->in_pos.data(), n, pos, e->absent);
    }
    if ((st = dev_reserve(e, e->b_pos, n * sizeof(float2), false))) return st;
    if ((st = dev_reserve(e, e->b_pos_alt, n * sizeof(float2), false))) return st;
    if ((st = dev_reserve(e, e->b_flags, n, false))) return st;
    if ((st = dev_reserve(e, e->b_jitter, n * sizeof(float2), false))) return st;
    if ((st = dev_reserve(e, e->b_key, n * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_rank, n * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_sorted_idx, n * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_sorted_pos, n * sizeof(float2), false))) return st;
    if ((st = dev_reserve(e, e->b_idx_s, n * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_pos_s, n * sizeof(float2), false))) return st;
    // a new point set: the first tick bins in index order (no cell order yet)
    if ((st = dev_reserve(e, e->b_bin_state, 4 * sizeof(uint32_t), true))) return st;
    if (n) CU(cudaMemcpyAsync(e->b_pos.p, pos.data(), n * sizeof(float2), cudaMemcpyHostToDevice, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    refresh_view(e);
    if ((st = apply_pinned(e))) return st;
    setup_fixed(e);
    // ForceManyBody.create (ForceManyBody/index.ts:124-185): pyramid sizes and
    // the jitter texture (2 draws per texel of pointsTextureSize^2, :133-138)
    e->mb_ready = false;
    // a new point set: its many-body kernel is timed again
    e->mb_choice = -1;
    e->mb_tuned = false;
    e->tune_cands.clear();
    e->tune_next = 0;
    if (e->T) {
      const ingest::Grid grid = ingest::grid_for(e->N);
      e->Gf = grid.gf;
      e->L = grid.levels;
      e->tile = std::min(16, e->Gf);
      uint32_t off = 0;
      for (int l = 0; l < e->L; ++l) { e->level_off[l] = off; off += (uint32_t)((4 << l) * (4 << l)); }
      uint32_t aoff = 0;
      for (int l = 0; l < e->L; ++l) { e->acc_off[l] = aoff; aoff += (uint32_t)((4 << l) * (4 << l)); }
      const uint32_t cells = (uint32_t)(e->Gf * e->Gf);
      if ((st = dev_reserve(e, e->b_counts, cells * sizeof(uint32_t), true))) return st;
      if ((st = dev_reserve(e, e->b_cell_start, (cells + 1) * sizeof(uint32_t), false))) return st;
      // the scan's status words and tickets start from zero together
      if ((st = dev_reserve(e, e->b_block_sums, (scan_blocks(cells) + 1) * sizeof(unsigned long long), true)))
        return st;
      if ((st = dev_reserve(e, e->b_pair_start, (cells + 1) * sizeof(uint32_t), true))) return st;
      if ((st = dev_reserve(e, e->b_pair_list, std::max<size_t>(n, 1) * sizeof(uint32_t), false))) return st;
      if ((st = dev_reserve(e, e->b_tickets, 4 * sizeof(uint32_t), true))) return st;
      if ((st = dev_reserve(e, e->b_rec, off * sizeof(float4), true))) return st;
      if ((st = dev_reserve(e, e->b_acc, 3 * (size_t)aoff * sizeof(long long), true))) return st;
      if ((st = dev_reserve(e, e->b_centroid, 3 * sizeof(long long), true))) return st;
      if ((st = dev_reserve(e, e->b_big_list, 2 * (size_t)cells * sizeof(uint32_t), false))) return st;
      if ((st = dev_reserve(e, e->b_big_count, 8 * sizeof(uint32_t), true))) return st;
      if ((st = dev_reserve(e, e->b_big_sx, cells * sizeof(long long), false))) return st;
      if ((st = dev_reserve(e, e->b_big_sy, cells * sizeof(long long), false))) return st;
      if ((st = dev_reserve(e, e->b_big_ns, cells * sizeof(uint32_t), false))) return st;
      const uint64_t texels = (uint64_t)e->T * e->T;
      if (e->rng.counter && !(e->cfg.device_ingest_min_links > (double)n)) {   // drawn on the device, same draws
        dingest::jitter(e->rng.seed, e->rng.ctr, (uint32_t)n, (float2*)e->b_jitter.p, e->stream);
        CU(cudaGetLastError());
        e->rng.ctr += 2 * texels;
      } else {
        std::vector<float2> jit;
        ingest::jitter(e->rng, n, jit);
        if (n) CU(cudaMemcpyAsync(e->b_jitter.p, jit.data(), n * sizeof(float2), cudaMemcpyHostToDevice, e->stream));
      }
      CU(cudaStreamSynchronize(e->stream));
      e->mb_ready = true;
    }
    e->collision_ready = false;
  }
  if (e->sizes_dirty) e->collision_ready = false;
  if (links_changed) {
    e->graph_dirty = true;
    // ForceLink.create(INCOMING) then (OUTGOING) (src/index.ts:1663-1666)
    const double dmin = e->cfg.device_ingest_min_links;
    if (e->T && e->W && E > 0 && !(dmin > (double)E)) {
      if ((st = build_links_device(e, E, n))) return st;
    } else {
    ingest::Csr cin, cout_;
    if (e->T && e->W) {
      ingest::build_links(e->in_links.data(), E, n, e->has_strength ? e->in_strength.data() : nullptr, e->absent,
                          e->rng, cin, cout_);
    } else {
      cin.rowptr.assign(n + 1, 0);
      cout_.rowptr.assign(n + 1, 0);
    }
    std::vector<uint32_t>& rp_in = cin.rowptr;
    std::vector<uint32_t>& rp_out = cout_.rowptr;
    std::vector<uint4>& en_in = cin.ent;
    std::vector<uint4>& en_out = cout_.ent;
    if (cin.order.empty()) { cin.order.resize(n); for (size_t p = 0; p < n; ++p) cin.order[p] = (uint32_t)p; }
    if (cout_.order.empty()) { cout_.order.resize(n); for (size_t p = 0; p < n; ++p) cout_.order[p] = (uint32_t)p; }
    std::vector<uint32_t>& hv_in = cin.order;
    std::vector<uint32_t>& hv_out = cout_.order;
    e->max_deg_in = cin.max_degree;
    e->max_deg_out = cout_.max_degree;
    e->entries = en_in.size();
    e->n_heavy_in = (uint32_t)cin.heavy.size();
    e->n_heavy_out = (uint32_t)cout_.heavy.size();
    if ((st = dev_reserve(e, e->b_heavy_in, hv_in.size() * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_heavy_out, hv_out.size() * sizeof(uint32_t), false))) return st;
    if (!hv_in.empty())
      CU(cudaMemcpyAsync(e->b_heavy_in.p, hv_in.data(), hv_in.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
    if (!hv_out.empty())
      CU(cudaMemcpyAsync(e->b_heavy_out.p, hv_out.data(), hv_out.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
    if ((st = dev_reserve(e, e->b_rowptr_in, (n + 1) * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_rowptr_out, (n + 1) * sizeof(uint32_t), false))) return st;
    if ((st = dev_reserve(e, e->b_ent_in, en_in.size() * sizeof(uint4), false))) return st;
    if ((st = dev_reserve(e, e->b_ent_out, en_out.size() * sizeof(uint4), false))) return st;
    CU(cudaMemcpyAsync(e->b_rowptr_in.p, rp_in.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
    CU(cudaMemcpyAsync(e->b_rowptr_out.p, rp_out.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
    if (!en_in.empty())
      CU(cudaMemcpyAsync(e->b_ent_in.p, en_in.data(), en_in.size() * sizeof(uint4), cudaMemcpyHostToDevice, e->stream));
    if (!en_out.empty())
      CU(cudaMemcpyAsync(e->b_ent_out.p, en_out.data(), en_out.size() * sizeof(uint4), cudaMemcpyHostToDevice, e->stream));
    CU(cudaStreamSynchronize(e->stream));
    }
    if ((st = build_link_warps(e))) return st;
    if ((st = build_early(e))) return st;
  }
  if (e->clusters_dirty || pos_changed) {
    // Clusters.create (Clusters/index.ts:54-100), src/index.ts:1668
    e->graph_dirty = true;
    ingest::Clusters c;
    ingest::build_clusters(n, e->have_clusters, e->in_clusters, e->have_cluster_pos, e->in_cluster_pos,
                           e->have_cluster_strength, e->in_cluster_strength, c);
    e->point_clusters = c.point_clusters;
    e->cluster_positions = c.positions;
    e->n_clusters = (c.point_clusters || c.positions) ? c.count : 0;
    if (e->n_clusters) {
      if ((st = dev_reserve(e, e->b_cl_of, n * sizeof(uint32_t), false))) return st;
      if ((st = dev_reserve(e, e->b_cl_coeff, n * sizeof(float), false))) return st;
      if ((st = dev_reserve(e, e->b_cl_custom, e->n_clusters * sizeof(float2), false))) return st;
      if ((st = dev_reserve(e, e->b_cl_acc, 3 * (size_t)e->n_clusters * sizeof(long long), true))) return st;
      CU(cudaMemcpyAsync(e->b_cl_of.p, c.of.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
      CU(cudaMemcpyAsync(e->b_cl_coeff.p, c.coeff.data(), n * sizeof(float), cudaMemcpyHostToDevice, e->stream));
      CU(cudaMemcpyAsync(e->b_cl_custom.p, c.custom.data(), e->n_clusters * sizeof(float2), cudaMemcpyHostToDevice,
                         e->stream));
      CU(cudaStreamSynchronize(e->stream));
    }
  }
  refresh_view(e);
  e->pos_dirty = e->links_dirty = e->sizes_dirty = e->clusters_dirty = false;
  if (pos_changed) e->skip_rescale = false;   // Points/index.ts:412-413
  if (!std::isnan(alpha)) e->alpha = alpha;
  return CGL_OK;
}

}  // namespace

// ================================================================ C ABI ====
extern "C" {

void cgl_config_defaults(cgl_config* c) {
  // src/variables.ts:10,15,19,69-82,147-148
  std::memset(c, 0, sizeof(*c));
  c->space_size = 4096;
  c->simulation_decay = 5000;
  c->simulation_gravity = 0.25;
  c->simulation_center = 0;
  c->simulation_repulsion = 1.0;
  c->simulation_repulsion_theta = 1.15;
  c->simulation_link_spring = 1;
  c->simulation_link_distance = 10;
  c->simulation_link_dist_random_variation_range[0] = 1;
  c->simulation_link_dist_random_variation_range[1] = 1.2;
  c->simulation_friction = 0.85;
  c->simulation_collision = 0;
  c->simulation_collision_radius = NAN;
  c->simulation_collision_padding = 0;
  c->point_default_size = 4;
  c->enable_simulation = 1;
  c->has_random_seed = 0;
  c->random_seed = 0;
  c->max_texture_dimension = 0;
  c->stage_mask = CGL_STAGE_ALL;
  c->device = 0;
  c->hbm_budget_bytes = 0;
  c->simulation_cluster = 0.1;
  c->simulation_repulsion_from_mouse = 2;
  c->enable_right_click_repulsion = 0;
  c->enable_drag = 0;
  c->device_ingest_min_links = 65536;
  c->random_stream = CGL_RANDOM_REFERENCE;
  c->rescale_positions = -1;
  c->random_seed_text = nullptr;
  c->manybody_kernel = CGL_MANYBODY_AUTO;
}

cgl_status cgl_create(const cgl_config* cfg, cgl_engine** out) {
  if (!cfg || !out) return CGL_INVALID_ARG;
  if (cfg->manybody_kernel < CGL_MANYBODY_AUTO || cfg->manybody_kernel > CGL_MANYBODY_TWO_POINTS)
    return CGL_INVALID_ARG;
  *out = nullptr;
  cgl_engine* e = new cgl_engine();
  e->cfg = *cfg;
  e->device = cfg->device;
  // Store.addRandomSeed (src/index.ts:452): the seed text is copied and kept
  if (cfg->has_random_seed && cfg->random_seed_text) e->seed_text = cfg->random_seed_text;
  e->cfg.random_seed_text = (cfg->has_random_seed && cfg->random_seed_text) ? e->seed_text.c_str() : nullptr;
  ingest::seed_rng(e->cfg, e->rng);
  adjust_space_size(e);
  const char* g = getenv("CGL_NO_GRAPH");
  e->use_graph = !(g && g[0] == '1');
  cudaError_t ce = cudaSetDevice(e->device);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaMallocHost((void**)&e->h_params, kParamChunk * sizeof(TickParams));
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->params_copied, cudaEventDisableTiming);
  if (ce == cudaSuccess) {   // the hub chains' stream first in line for the SMs: the longest chain starts at once
    int lo = 0, hi = 0;
    ce = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithPriority(&e->side, cudaStreamNonBlocking, hi);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithPriority(&e->side2, cudaStreamNonBlocking, lo);
  }
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e->tune_ev[0]);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e->tune_ev[1]);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->join2, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->snap_ready, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->snap_done, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaHostAlloc((void**)&e->h_error, sizeof(uint32_t), cudaHostAllocMapped);
  if (ce == cudaSuccess) ce = cudaHostGetDevicePointer((void**)&e->d_error, e->h_error, 0);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    static thread_local std::string create_err;
    create_err = cudaGetErrorString(ce);
    if (e->own_stream) cudaStreamDestroy(e->own_stream);
    if (e->side) cudaStreamDestroy(e->side);
    if (e->side2) cudaStreamDestroy(e->side2);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->join) cudaEventDestroy(e->join);
    if (e->join2) cudaEventDestroy(e->join2);
    if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
    if (e->snap_ready) cudaEventDestroy(e->snap_ready);
    if (e->snap_done) cudaEventDestroy(e->snap_done);
    for (cudaEvent_t x : e->tune_ev) if (x) cudaEventDestroy(x);
    if (e->h_params) cudaFreeHost(e->h_params);
    if (e->h_error) cudaFreeHost(e->h_error);
    delete e;
    return ce == cudaErrorMemoryAllocation ? CGL_OOM : CGL_CUDA_ERROR;
  }
  *e->h_error = 0;
  e->stream = e->own_stream;
  cgl_status st;
  if ((st = dev_reserve(e, e->b_params, kParamChunk * sizeof(TickParams), true)) ||
      (st = dev_reserve(e, e->b_tick_ctr, sizeof(uint32_t), true))) {
    cgl_destroy(e);
    return st;
  }
  refresh_view(e);
  *out = e;
  return CGL_OK;
}

cgl_status cgl_destroy(cgl_engine* e) {
  if (!e) return CGL_INVALID_ARG;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->copy_stream) cudaStreamSynchronize(e->copy_stream);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  dev_free_all(e);
  if (e->params_copied) cudaEventDestroy(e->params_copied);
  if (e->h_params) cudaFreeHost(e->h_params);
  if (e->h_error) cudaFreeHost(e->h_error);
  if (e->side) cudaStreamDestroy(e->side);
  if (e->side2) cudaStreamDestroy(e->side2);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->join) cudaEventDestroy(e->join);
  if (e->join2) cudaEventDestroy(e->join2);
  if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
  if (e->snap_ready) cudaEventDestroy(e->snap_ready);
  if (e->snap_done) cudaEventDestroy(e->snap_done);
  for (cudaEvent_t x : e->tune_ev) if (x) cudaEventDestroy(x);
  if (e->own_stream) cudaStreamDestroy(e->own_stream);
  delete e;
  return CGL_OK;
}

#define CHECK_E(e)                                  \
  do {                                              \
    if (!(e)) return CGL_INVALID_ARG;               \
    if ((e)->destroyed) return CGL_DESTROYED;       \
    (e)->err.clear();                               \
    if (cudaSetDevice((e)->device) != cudaSuccess) return fail(e, CGL_CUDA_ERROR, "cudaSetDevice"); \
  } while (0)

cgl_status cgl_set_config(cgl_engine* e, const cgl_config* cfg) {
  CHECK_E(e);
  if (!cfg) return CGL_INVALID_ARG;
  if (cfg->manybody_kernel < CGL_MANYBODY_AUTO || cfg->manybody_kernel > CGL_MANYBODY_TWO_POINTS)
    return fail(e, CGL_INVALID_ARG, "manybody_kernel %d: not a CGL_MANYBODY_* value", cfg->manybody_kernel);
  const cgl_config prev = e->cfg;
  e->cfg = *cfg;
  e->cfg.has_random_seed = prev.has_random_seed;   // init-only (src/index.ts:1720-1724)
  e->cfg.random_seed = prev.random_seed;
  e->cfg.random_seed_text = prev.random_seed_text;
  e->cfg.random_stream = prev.random_stream;
  e->cfg.device = prev.device;
  e->graph_dirty = true;
  if (prev.space_size != e->cfg.space_size) {
    // src/index.ts:1844-1851
    adjust_space_size(e);
    e->collision_ready = false;
    if (e->N) setup_fixed(e);
    e->alpha = e->running ? e->alpha : 0;
  }
  return CGL_OK;
}

cgl_status cgl_get_config(cgl_engine* e, cgl_config* out) {
  CHECK_E(e);
  if (!out) return CGL_INVALID_ARG;
  *out = e->cfg;
  return CGL_OK;
}

cgl_status cgl_set_point_positions(cgl_engine* e, const float* xy, uint64_t n) {
  return cgl_set_point_positions_ex(e, xy, n, 0);
}

cgl_status cgl_set_point_positions_ex(cgl_engine* e, const float* xy, uint64_t n, int32_t dont_rescale) {
  CHECK_E(e);
  if (!xy && n) return CGL_INVALID_ARG;
  cgl_status st = CGL_OK;
  if (n % 2) {
    n -= 1;
    st = fail(e, CGL_WARNING, "Invalid point positions length: %llu. The trailing value was ignored.",
              (unsigned long long)(n + 1));
  }
  e->in_pos.assign(xy, xy + n);
  e->have_pos_input = true;
  e->skip_rescale = dont_rescale != 0;   // src/index.ts:553
  e->pos_dirty = e->links_dirty = e->sizes_dirty = true;
  e->clusters_dirty = true;   // src/index.ts:570
  return st;
}

cgl_status cgl_set_links(cgl_engine* e, const float* st_, uint64_t n) {
  CHECK_E(e);
  if (!st_ && n) return CGL_INVALID_ARG;
  cgl_status st = CGL_OK;
  if (n % 2) {
    n -= 1;
    st = fail(e, CGL_WARNING, "Invalid links length: %llu. The trailing value was ignored.", (unsigned long long)(n + 1));
  }
  e->in_links.assign(st_, st_ + n);
  e->have_link_input = true;
  e->links_dirty = true;
  return st;
}

cgl_status cgl_set_link_strength(cgl_engine* e, const float* v, uint64_t n) {
  CHECK_E(e);
  if (!v || n == 0) { e->in_strength.clear(); e->have_strength = false; }
  else { e->in_strength.assign(v, v + n); e->have_strength = true; }
  e->links_dirty = true;
  return CGL_OK;
}

cgl_status cgl_set_point_sizes(cgl_engine* e, const float* v, uint64_t n) {
  CHECK_E(e);
  if (!v) { e->in_sizes.clear(); e->have_sizes = false; }
  else { e->in_sizes.assign(v, v + n); e->have_sizes = true; }
  e->sizes_dirty = true;
  return CGL_OK;
}

cgl_status cgl_set_point_clusters(cgl_engine* e, const float* v, uint64_t n) {
  CHECK_E(e);
  if (!v || n == 0) { e->in_clusters.clear(); e->have_clusters = false; }
  else { e->in_clusters.assign(v, v + n); e->have_clusters = true; }
  e->clusters_dirty = true;
  return CGL_OK;
}

cgl_status cgl_set_cluster_positions(cgl_engine* e, const float* v, uint64_t n) {
  CHECK_E(e);
  if (!v) { e->in_cluster_pos.clear(); e->have_cluster_pos = false; }
  else { e->in_cluster_pos.assign(v, v + n); e->have_cluster_pos = true; }
  e->clusters_dirty = true;
  return CGL_OK;
}

cgl_status cgl_set_point_cluster_strength(cgl_engine* e, const float* v, uint64_t n) {
  CHECK_E(e);
  if (!v || n == 0) { e->in_cluster_strength.clear(); e->have_cluster_strength = false; }
  else { e->in_cluster_strength.assign(v, v + n); e->have_cluster_strength = true; }
  e->clusters_dirty = true;
  return CGL_OK;
}

cgl_status cgl_get_cluster_positions(cgl_engine* e, double* out, uint64_t cap, uint64_t* n_out) {
  CHECK_E(e);
  // Clusters.getCentroidPositions (Clusters/index.ts:389-423): sum / count in
  // FP64 of the f32 sums, from the current positions
  const uint64_t n = e->point_clusters ? 2 * (uint64_t)e->n_clusters : 0;
  if (n_out) *n_out = n;
  if (!out || n == 0) return CGL_OK;
  if (cap < n) return fail(e, CGL_INVALID_ARG, "output holds %llu doubles, need %llu", (unsigned long long)cap,
                           (unsigned long long)n);
  const DeviceView& d = e->view;
  const SimScalars s = make_scalars(e);
  CU(cudaMemsetAsync(d.cluster_acc, 0, 3 * (size_t)e->n_clusters * sizeof(long long), e->stream));
  launch_cluster_sum(d, s, e->stream);
  CU(cudaGetLastError());
  std::vector<long long> acc(3 * (size_t)e->n_clusters);
  CU(cudaMemcpyAsync(acc.data(), d.cluster_acc, acc.size() * sizeof(long long), cudaMemcpyDeviceToHost, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  for (uint32_t c = 0; c < e->n_clusters; ++c) {
    const float sx = (float)acc[3 * (size_t)c] * e->fx.inv, sy = (float)acc[3 * (size_t)c + 1] * e->fx.inv;
    const float cnt = (float)acc[3 * (size_t)c + 2];
    out[2 * (size_t)c] = (double)sx / (double)cnt;
    out[2 * (size_t)c + 1] = (double)sy / (double)cnt;
  }
  return CGL_OK;
}

namespace {
// Device address of `out` when the engine's device can write it directly:
// device memory of that device, managed memory, or pinned host memory (mapped
// into the device's address space).  nullptr for pageable host memory.
cgl_status texture_target(cgl_engine* e, float* out, float4** dev) {
  *dev = nullptr;
  cudaPointerAttributes a{};
  cudaError_t ce = cudaPointerGetAttributes(&a, out);
  if (ce != cudaSuccess) { cudaGetLastError(); return CGL_OK; }   // unknown to CUDA: pageable
  if (a.type == cudaMemoryTypeDevice) {
    if (a.device != e->device) return fail(e, CGL_INVALID_ARG, "texture buffer is on device %d, engine on %d", a.device, e->device);
    *dev = (float4*)a.devicePointer;
  } else if (a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeHost) {
    *dev = (float4*)a.devicePointer;
  }
  return CGL_OK;
}

cgl_status texture_common(cgl_engine* e, float* out, uint64_t cap, uint64_t* texels) {
  *texels = (uint64_t)e->T * e->T;
  if (!out && *texels) return fail(e, CGL_INVALID_ARG, "null texture buffer");
  if (cap < 4 * *texels)
    return fail(e, CGL_INVALID_ARG, "texture buffer holds %llu floats, need %llu", (unsigned long long)cap,
                (unsigned long long)(4 * *texels));
  return CGL_OK;
}
}  // namespace

cgl_status cgl_get_position_texture(cgl_engine* e, float* out, uint64_t cap) {
  CHECK_E(e);
  uint64_t texels;
  cgl_status st = texture_common(e, out, cap, &texels);
  if (st || !texels) return st;
  float4* dev;
  if ((st = texture_target(e, out, &dev))) return st;
  if (dev) {
    launch_position_texture(e->view, dev, (uint32_t)texels, e->stream);
    CU(cudaGetLastError());
  } else {
    if ((st = dev_reserve(e, e->b_texture, texels * sizeof(float4), false))) return st;
    launch_position_texture(e->view, (float4*)e->b_texture.p, (uint32_t)texels, e->stream);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(out, e->b_texture.p, texels * sizeof(float4), cudaMemcpyDeviceToHost, e->stream));
  }
  CU(cudaStreamSynchronize(e->stream));
  return CGL_OK;
}

cgl_status cgl_enqueue_position_texture(cgl_engine* e, float* out, uint64_t cap) {
  CHECK_E(e);
  uint64_t texels;
  cgl_status st = texture_common(e, out, cap, &texels);
  if (st || !texels) return st;
  float4* dev;
  if ((st = texture_target(e, out, &dev))) return st;
  if (!dev) return fail(e, CGL_INVALID_ARG, "queued texture read-back needs device or pinned host memory");
  launch_position_texture(e->view, dev, (uint32_t)texels, e->stream);
  CU(cudaGetLastError());
  return CGL_OK;
}

cgl_status cgl_set_pinned_points(cgl_engine* e, const double* idx, uint64_t n) {
  CHECK_E(e);
  e->pinned_set = idx && n > 0;
  if (e->pinned_set) e->pinned_input.assign(idx, idx + n);
  else e->pinned_input.clear();
  if (e->N) return apply_pinned(e);
  return CGL_OK;
}

cgl_status cgl_render(cgl_engine* e, double alpha) {
  CHECK_E(e);
  return do_render(e, alpha);
}

cgl_status cgl_start(cgl_engine* e, double alpha) {
  CHECK_E(e);
  if (!e->cfg.enable_simulation || e->N == 0) return CGL_OK;
  e->running = true;
  e->progress = 0;
  e->alpha = alpha;
  return CGL_OK;
}

cgl_status cgl_stop(cgl_engine* e) {
  CHECK_E(e);
  e->running = false;
  e->progress = 0;
  e->alpha = 0;
  return CGL_OK;
}

cgl_status cgl_pause(cgl_engine* e) {
  CHECK_E(e);
  e->running = false;
  return CGL_OK;
}

cgl_status cgl_unpause(cgl_engine* e) {
  CHECK_E(e);
  if (e->cfg.enable_simulation) e->running = true;
  return CGL_OK;
}

cgl_status cgl_step(cgl_engine* e, uint32_t ticks) {
  CHECK_E(e);
  if (!e->cfg.enable_simulation || e->T == 0) return CGL_OK;
  return run_ticks(e, ticks, nullptr, nullptr);
}

namespace {
// One animation frame (src/index.ts:2161-2175, renderFrame :2237-2317).
cgl_status one_frame(cgl_engine* e, uint32_t* ticks) {
  if (e->alpha < kAlphaMin && e->running) { e->running = false; e->progress = 1; }   // end()
  if (e->cfg.enable_simulation && e->T) {   // runSimulationStep(false)
    if (e->running) {
      cgl_status st = run_ticks(e, 1, nullptr, nullptr);   // includes the pointer pass
      if (st) return st;
      ++*ticks;
    } else if (mouse_active(e)) {
      launch_pointer_force(e);
      CU(cudaGetLastError());
    }
  }
  if (dragging(e)) {
    launch_drag(e->view, (uint32_t)e->drag_index, make_float2((float)e->mouse_x, (float)e->mouse_y), e->stream);
    CU(cudaGetLastError());
  }
  return CGL_OK;
}
}  // namespace

cgl_status cgl_set_pointer(cgl_engine* e, double x, double y, int32_t right_button_down) {
  CHECK_E(e);
  e->mouse_x = x;
  e->mouse_y = y;
  e->right_button = right_button_down != 0;
  return CGL_OK;
}

cgl_status cgl_set_drag(cgl_engine* e, int64_t index) {
  CHECK_E(e);
  if (!e->cfg.enable_drag) return CGL_OK;
  if (index >= (int64_t)e->N) return fail(e, CGL_INVALID_ARG, "drag index %lld outside %llu points", (long long)index,
                                          (unsigned long long)e->N);
  e->drag_index = index < 0 ? -1 : index;
  return CGL_OK;
}

cgl_status cgl_frame(cgl_engine* e, uint32_t frames, uint32_t* ticks_done) {
  CHECK_E(e);
  uint32_t n = 0;
  if (!e->T) { if (ticks_done) *ticks_done = 0; return CGL_OK; }   // frame() needs points (:2159)
  if (!interactive(e)) {
    // alpha evolves on the host only: the frames that tick are known up front
    if (e->cfg.enable_simulation && e->running) {
      double a = e->alpha;
      const double f = 1 - std::pow(kAlphaMin, 1 / e->cfg.simulation_decay);
      while (n < frames && !(a < kAlphaMin)) { a += (0 - a) * f; ++n; }
      cgl_status st = run_ticks(e, n, nullptr, nullptr);
      if (st) return st;
      if (n < frames && e->alpha < kAlphaMin) { e->running = false; e->progress = 1; }
    }
  } else {
    for (uint32_t k = 0; k < frames; ++k) {
      cgl_status st = one_frame(e, &n);
      if (st) return st;
    }
  }
  if (ticks_done) *ticks_done = n;
  return CGL_OK;
}

cgl_status cgl_run(cgl_engine* e, uint32_t max_ticks, uint32_t* ticks_done) {
  CHECK_E(e);
  uint32_t n = 0;
  if (e->cfg.enable_simulation && e->T && e->running && interactive(e)) {
    while (n < max_ticks && e->running) {
      cgl_status st = one_frame(e, &n);
      if (st) return st;
    }
    if (ticks_done) *ticks_done = n;
    return CGL_OK;
  }
  if (e->cfg.enable_simulation && e->T && e->running) {
    // alpha evolves on the host only, so the tick count is known up front
    double a = e->alpha;
    const double f = 1 - std::pow(kAlphaMin, 1 / e->cfg.simulation_decay);
    while (n < max_ticks && !(a < kAlphaMin)) { a += (0 - a) * f; ++n; }
    cgl_status st = run_ticks(e, n, nullptr, nullptr);
    if (st) return st;
    if (n < max_ticks && e->alpha < kAlphaMin) { e->running = false; e->progress = 1; }
  }
  if (ticks_done) *ticks_done = n;
  return CGL_OK;
}

cgl_status cgl_get_point_positions(cgl_engine* e, float* out, uint64_t cap) {
  CHECK_E(e);
  if (cap < 2 * e->N || (!out && e->N)) return fail(e, CGL_INVALID_ARG, "output holds %llu floats, need %llu",
                                                      (unsigned long long)cap, (unsigned long long)(2 * e->N));
  if (!e->N) return CGL_OK;
  CU(cudaMemcpyAsync(out, e->b_pos.p, e->N * sizeof(float2), cudaMemcpyDeviceToHost, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return device_error(e);
}

cgl_status cgl_enqueue_point_positions(cgl_engine* e, float* out, uint64_t cap) {
  CHECK_E(e);
  if (cap < 2 * e->N || (!out && e->N)) return fail(e, CGL_INVALID_ARG, "output holds %llu floats, need %llu",
                                                      (unsigned long long)cap, (unsigned long long)(2 * e->N));
  if (!e->N) return CGL_OK;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, out) != cudaSuccess) cudaGetLastError();
  if (a.type == cudaMemoryTypeUnregistered || (a.type == cudaMemoryTypeDevice && a.device != e->device))
    return fail(e, CGL_INVALID_ARG, "queued position read-back needs pinned host memory or memory of device %d",
                e->device);
  if (e->snap_pending) {   // the previous copy has landed: its buffer is the caller's again, its staging ours
    CU(cudaEventSynchronize(e->snap_done));
    e->snap_pending = false;
  }
  const size_t bytes = e->N * sizeof(float2);
  cgl_status st;
  if ((st = dev_reserve(e, e->b_snap, bytes, false))) return st;
  CU(cudaMemcpyAsync(e->b_snap.p, e->b_pos.p, bytes, cudaMemcpyDeviceToDevice, e->stream));
  CU(cudaEventRecord(e->snap_ready, e->stream));
  CU(cudaStreamWaitEvent(e->copy_stream, e->snap_ready, 0));
  CU(cudaMemcpyAsync(out, e->b_snap.p, bytes, cudaMemcpyDefault, e->copy_stream));
  CU(cudaEventRecord(e->snap_done, e->copy_stream));
  e->snap_pending = true;
  return device_error(e);
}

cgl_status cgl_get_state(cgl_engine* e, cgl_state* s) {
  if (!e || !s) return CGL_INVALID_ARG;
  std::memset(s, 0, sizeof(*s));
  s->destroyed = e->destroyed;
  s->alpha = e->alpha;
  s->progress = e->progress;
  s->is_simulation_running = e->running;
  s->tick = e->tick;
  s->points_number = e->N;
  s->links_number = e->E;
  s->rng_draws = e->rng.ctr;
  return CGL_OK;
}

const char* cgl_last_error(cgl_engine* e) { return e ? e->err.c_str() : "null engine"; }

cgl_status cgl_random_draws(const char* seed_text, uint64_t n, double* out) {
  if (!seed_text || (!out && n)) return CGL_INVALID_ARG;
  RandomStream r;
  r.seed_utf8(seed_text);
  for (uint64_t k = 0; k < n; ++k) out[k] = r.next();
  return CGL_OK;
}

cgl_status cgl_check_wait_limit(int32_t device, uint32_t* error_bits) {
  if (!error_bits) return CGL_INVALID_ARG;
  *error_bits = 0;
  if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return CGL_CUDA_ERROR; }
  unsigned long long* status = nullptr;
  uint32_t *h_err = nullptr, *d_err = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaMalloc((void**)&status, 2 * sizeof(unsigned long long));
  if (ce == cudaSuccess) ce = cudaMemsetAsync(status, 0, 2 * sizeof(unsigned long long), st);
  if (ce == cudaSuccess) ce = cudaHostAlloc((void**)&h_err, sizeof(uint32_t), cudaHostAllocMapped);
  if (ce == cudaSuccess) ce = cudaHostGetDevicePointer((void**)&d_err, h_err, 0);
  if (ce == cudaSuccess) {
    *h_err = 0;
    launch_wait_limit(status, d_err, st);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce == cudaSuccess) *error_bits = *(volatile uint32_t*)h_err;
  }
  if (status) cudaFree(status);
  if (h_err) cudaFreeHost(h_err);
  if (st) cudaStreamDestroy(st);
  if (ce != cudaSuccess) { cudaGetLastError(); return CGL_CUDA_ERROR; }
  return CGL_OK;
}

cgl_status cgl_set_stream(cgl_engine* e, void* cuda_stream) {
  CHECK_E(e);
  CU(cudaStreamSynchronize(e->stream));
  e->stream = cuda_stream ? (cudaStream_t)cuda_stream : e->own_stream;
  return CGL_OK;
}

cgl_status cgl_synchronize(cgl_engine* e) {
  CHECK_E(e);
  CU(cudaStreamSynchronize(e->stream));
  if (e->snap_pending) {
    CU(cudaEventSynchronize(e->snap_done));
    e->snap_pending = false;
  }
  return device_error(e);
}

cgl_status cgl_profile_stages(cgl_engine* e, uint32_t ticks, double* ms_out) {
  CHECK_E(e);
  if (!ms_out) return CGL_INVALID_ARG;
  for (int k = 0; k < CGL_NUM_STAGE_TIMES; ++k) ms_out[k] = 0;
  if (!e->cfg.enable_simulation || e->T == 0 || ticks == 0) return CGL_OK;
  cudaEvent_t ev[2 * CGL_NUM_STAGE_TIMES];
  for (auto& x : ev) CU(cudaEventCreate(&x));
  cgl_status st = run_ticks(e, ticks, ev, ms_out);
  for (auto& x : ev) cudaEventDestroy(x);
  if (st) return st;
  for (int k = 0; k < CGL_NUM_STAGE_TIMES; ++k) ms_out[k] /= ticks;
  return CGL_OK;
}

cgl_status cgl_get_layout(cgl_engine* e, cgl_layout* o) {
  CHECK_E(e);
  if (!o) return CGL_INVALID_ARG;
  std::memset(o, 0, sizeof(*o));
  o->points_number = e->N;
  o->live_points = e->live;
  o->links_number = e->E;
  o->link_entries_in = e->entries;
  o->points_texture_size = e->T;
  o->finest_grid = (uint32_t)e->Gf;
  o->levels = (uint32_t)e->L;
  o->max_degree_in = e->max_deg_in;
  o->max_degree_out = e->max_deg_out;
  o->fixed_point_bits = e->fixed_bits;
  o->fixed_point_bound = e->fx.bound;
  o->collision_grid = (uint32_t)e->cgrid;
  o->collision_cell_size = e->ccell;
  o->device_bytes = e->dev_bytes;
  if (e->mb_ready && e->N) {
    o->manybody_kernel = (uint32_t)make_scalars(e).mb_kernel;
    o->manybody_tuned = e->mb_tuned && e->cfg.manybody_kernel == CGL_MANYBODY_AUTO;
  }
  const TickPlan p = plan_tick(e);
  uint32_t k = 1;                                      // tick end
  if (p.grav || p.cent || p.mb) k += 1;                // prepass
  if (p.cent) k += 1;
  if (p.mb) k += 5;                                    // scan, scatter, big cells, cells, manybody
  k += (uint32_t)p.link_in + (uint32_t)p.link_out;
  if (p.coll) k += 3;                                  // grid, convert, force
  // the outgoing hub chains beside the collision sums: two link launches, two sums
  if (p.link_in && p.link_out && p.coll && !p.clus && p.mb && e->n_heavy_out > 0) k += 2;
  if (p.clus) k += 1 + (uint32_t)p.clus_sum;           // sums, pull + update
  // the early points' many-body terms and the early hubs' chains
  if (p.mb && p.link_in && e->n_early_hubs > 0 && e->n_early_pts > 0) k += 2;
  // the leading outgoing hubs apart from the rest of their pass (counted above with the overlap);
  // with the overlap, the collision results beside their chains: the late cells, the fix-up, the redo
  const bool overlap = p.link_in && p.link_out && p.coll && !p.clus && p.mb && e->n_heavy_out > 0;
  if (p.link_out && e->n_first_out > 0 && !overlap) k += 1;
  if (p.link_out && e->n_first_out > 0 && e->n_next_out > 0) k += 1;   // the next hubs' launch
  if (overlap && e->n_first_out > 0 && e->b_pos_coll.p && e->b_coll_mark.p && e->b_coll_redo.p) k += 3;
  o->kernels_per_tick = k;
  o->early_hubs = e->n_early_hubs;
  o->early_points = e->n_early_pts;
  o->leading_out_hubs = e->n_first_out + e->n_next_out;
  return CGL_OK;
}

cgl_status cgl_debug_get_cells(cgl_engine* e, uint32_t level, float* out, uint64_t cap) {
  CHECK_E(e);
  if (!e->mb_ready || level >= (uint32_t)e->L) return fail(e, CGL_INVALID_ARG, "no level %u", level);
  const uint64_t cells = (uint64_t)(4u << level) * (4u << level);
  if (cap < 4 * cells) return CGL_INVALID_ARG;
  CU(cudaMemcpyAsync(out, (float4*)e->b_rec.p + e->level_off[level], cells * sizeof(float4), cudaMemcpyDeviceToHost,
                     e->stream));
  CU(cudaStreamSynchronize(e->stream));
  return CGL_OK;
}

cgl_status cgl_debug_set_leading_hubs(cgl_engine* e, int32_t max_in, int32_t max_out) {
  CHECK_E(e);
  if (max_in < -1 || max_out < -1) return fail(e, CGL_INVALID_ARG, "max_in %d, max_out %d", max_in, max_out);
  e->lead_limit[0] = max_in;
  e->lead_limit[1] = max_out;
  if (e->N && !e->links_dirty && !e->pos_dirty) {
    const cgl_status st = build_early(e);
    if (st) return st;
  }
  refresh_view(e);
  e->graph_dirty = true;
  return CGL_OK;
}

cgl_status cgl_debug_get_slots(cgl_engine* e, int32_t* out, uint64_t cap) {
  CHECK_E(e);
  if (!e->mb_ready) return CGL_INVALID_ARG;
  const uint64_t cells = (uint64_t)e->Gf * e->Gf;
  if (cap < kSlots * cells) return CGL_INVALID_ARG;
  std::vector<float4> fine(cells);
  std::vector<uint32_t> start(cells + 1);
  std::vector<uint32_t> sidx(e->live);
  CU(cudaMemcpyAsync(fine.data(), (float4*)e->b_rec.p + e->level_off[e->L - 1], cells * sizeof(float4),
                     cudaMemcpyDeviceToHost, e->stream));
  CU(cudaMemcpyAsync(start.data(), e->b_cell_start.p, (cells + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
  if (e->live)
    CU(cudaMemcpyAsync(sidx.data(), e->b_sorted_idx.p, e->live * sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
  CU(cudaStreamSynchronize(e->stream));
  for (uint64_t c = 0; c < cells; ++c) {
    const int ns = (int)fine[c].w;
    for (int q = 0; q < kSlots; ++q)
      out[c * kSlots + q] = (q < ns && start[c] + q < e->live) ? (int32_t)sidx[start[c] + q] : -1;
  }
  return CGL_OK;
}

}  // extern "C"
