// batch.cu — host side of the batched engine (cgl_batch_* in include/cgl.h).
//
// Independent layout jobs share one set of device arenas and advance
// together: one CUDA-graph launch per tick for every graph in the batch.
// Jobs join (cgl_batch_add) and leave (cgl_batch_remove) between ticks;
// each keeps its own alpha, random stream and tick budget, so its trajectory
// is the one it would have in a plain engine.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <string>
#include <vector>

#include "../../include/cgl.h"
#include "batch.cuh"
#include "ingest.h"
#include "ingest_device.cuh"
#include "kernels.cuh"

using namespace cgl;

namespace {

constexpr double kAlphaMin = 0.001;
constexpr uint32_t kTickChunk = 64;   // ticks per parameter upload

// First-fit range allocator over [0, cap): free ranges below the high-water mark.
struct Arena {
  uint64_t cap = 0, hwm = 0;
  std::map<uint64_t, uint64_t> free_;   // offset -> length
  bool alloc(uint64_t n, uint64_t* off) {
    if (n == 0) { *off = 0; return true; }
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        const uint64_t rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    }
    if (hwm + n > cap) return false;
    *off = hwm;
    hwm += n;
    return true;
  }
  void release(uint64_t off, uint64_t n) {
    if (n == 0) return;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); it = pv; }
    }
    if (it->first + it->second == hwm) { hwm = it->first; free_.erase(it); }
  }
};

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct Job {
  bool used = false;
  cgl_config cfg{};
  uint64_t n = 0, live = 0, E = 0, m_in = 0, m_out = 0;
  uint64_t p_off = 0, cell_off = 0, cells = 0, rec_off = 0, recs = 0, acc_off = 0, accs = 0;
  uint64_t rp_in = 0, rp_out = 0, e_in = 0, e_out = 0;
  uint64_t coll_off = 0, coll_cells = 0;   // collision grids: 4 x coll_grid^2 cells
  int gf = 0, levels = 0, tile = 0;
  uint32_t stages = 0;
  ingest::Rng rng;
  double alpha = 1.0, progress = 0.0, decay_factor = 0.0;
  bool running = true;
  uint64_t tick = 0;
  uint32_t max_ticks = 0;
  bool stop_below_min = false;
  std::vector<uint32_t> heavy_in, heavy_out;   // local
  // the lists as rows (CSR) in the row and entry arenas: every row when the
  // device builds them, else only for a direction with long lists (the light
  // rows are read from the warp layout)
  uint64_t rows_n[2] = {0, 0}, ents_n[2] = {0, 0};
  // the light rows by warps (GraphDesc::lr, lw, ln, nw), both directions in one
  // range of each arena: rows, warp offsets, entries
  uint64_t lr_off = 0, lrs = 0, lw_off = 0, lws = 0, ln_off = 0, lns = 0;
  uint32_t nw[2] = {0, 0};
  uint64_t lane_ents[2] = {0, 0};
  GraphDesc desc{};
};

}  // namespace

struct cgl_batch {
  int device = 0;
  double budget = 0;
  std::string err;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t fork[2] = {}, join[2] = {}, params_copied = nullptr;
  bool params_pending = false;
  Arena pts, cells, recs, accs, rows, ents, colls, lrows, lwoffs, lanes_a;
  std::vector<Job> jobs;
  size_t dev_bytes = 0;
  // point arena
  Buf gid, pos, pos_alt, flags, jitter, key, rank, sorted_idx, sorted_pos, sib_list;
  // cell arena
  Buf counts, cell_start, cell_gid, big_list, big_sx, big_sy, big_ns, scan_status, scan_seq;
  Buf big_count, tick_ctr;
  Buf rec, acc, rowptr, ent, desc, tiles, heavy_in, heavy_out, ticks;
  Buf size, cgrid_acc, cgrid, coll_gid, centroid;   // collision and center
  Buf lrow, lwoff, lanes, lwork[2];                   // light rows by warps
  uint32_t n_lwork[2] = {0, 0};
  bool any_center = false, any_collision = false;
  uint32_t n_tiles = 0, n_heavy_in = 0, n_heavy_out = 0, slots_cap = 0;
  BatchTick* h_ticks = nullptr;
  uint32_t* h_error = nullptr;   // host-mapped error word (BatchView::error_word)
  uint32_t* d_error = nullptr;
  float2* h_stage = nullptr;   // pinned read-back staging of the point arena
  uint64_t stage_cap = 0;
  cudaGraphExec_t graph = nullptr;
  bool dirty = true;
  BatchView view{};
};

namespace {

// Transient device buffers of one cgl_batch_add, freed when it returns.
struct Temp {
  cgl_batch* b;
  std::vector<void*> ptrs;
  ~Temp();
  template <class T>
  T* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n * sizeof(T), 16)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    ptrs.push_back(p);
    return (T*)p;
  }
};

cgl_status bfail(cgl_batch* b, cgl_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return st;
}

Temp::~Temp() {
  if (ptrs.empty()) return;
  cudaStreamSynchronize(b->stream);
  for (void* p : ptrs) cudaFree(p);
}

#define BCU(call)                                                                                     \
  do {                                                                                                \
    cudaError_t _e = (call);                                                                          \
    if (_e != cudaSuccess)                                                                            \
      return bfail(b, _e == cudaErrorMemoryAllocation ? CGL_OOM : CGL_CUDA_ERROR, "%s: %s", #call,   \
                   cudaGetErrorString(_e));                                                           \
  } while (0)

// Grow a device buffer to `bytes`, keeping its first `keep` bytes; new bytes
// are filled with `fill` (-1: leave undefined).
cgl_status grow(cgl_batch* b, Buf& x, size_t bytes, size_t keep, int fill) {
  if (bytes <= x.bytes) return CGL_OK;
  if (b->budget > 0 && (double)(b->dev_bytes + bytes - x.bytes) > b->budget)
    return bfail(b, CGL_OOM, "device memory budget %.0f bytes: cannot grow to %zu more", b->budget, bytes - x.bytes);
  void* p = nullptr;
  BCU(cudaMalloc(&p, bytes));
  if (fill >= 0) BCU(cudaMemsetAsync(p, fill, bytes, b->stream));
  if (x.p && keep) BCU(cudaMemcpyAsync(p, x.p, std::min(keep, x.bytes), cudaMemcpyDeviceToDevice, b->stream));
  BCU(cudaStreamSynchronize(b->stream));
  if (x.p) cudaFree(x.p);
  b->dev_bytes += bytes - x.bytes;
  x.p = p;
  x.bytes = bytes;
  return CGL_OK;
}

// After a synchronisation: a device wait that gave up (error_word) is
// reported once, as a CUDA error of the call that found it.
cgl_status batch_device_error(cgl_batch* b) {
  if (!b->h_error) return CGL_OK;
  const uint32_t bits = *(volatile uint32_t*)b->h_error;
  if (!bits) return CGL_OK;
  *(volatile uint32_t*)b->h_error = 0;
  return bfail(b, CGL_CUDA_ERROR, "a device wait gave up (error bits 0x%x): the last ticks' cell scan is not valid",
               bits);
}

uint64_t grown(uint64_t cap, uint64_t need) { return std::max<uint64_t>(need, cap + cap / 2 + 1024); }

cgl_status reserve_points(cgl_batch* b, uint64_t cap) {
  if (cap <= b->pts.cap) return CGL_OK;
  const uint64_t keep = b->pts.hwm;
  cgl_status st;
  if ((st = grow(b, b->gid, cap * 4, keep * 4, 0xFF)) || (st = grow(b, b->pos, cap * 8, keep * 8, -1)) ||
      (st = grow(b, b->pos_alt, cap * 8, keep * 8, -1)) || (st = grow(b, b->flags, cap, keep, 0)) ||
      (st = grow(b, b->jitter, cap * 8, keep * 8, -1)) || (st = grow(b, b->key, cap * 4, 0, -1)) ||
      (st = grow(b, b->rank, cap * 4, 0, -1)) || (st = grow(b, b->sorted_idx, cap * 4, 0, -1)) ||
      (st = grow(b, b->sorted_pos, cap * 8, 0, -1)) || (st = grow(b, b->size, cap * 4, keep * 4, 0)) ||
      (st = grow(b, b->sib_list, cap * 8, 0, -1)))
    return st;
  b->pts.cap = cap;
  return CGL_OK;
}

cgl_status reserve_cells(cgl_batch* b, uint64_t cap) {
  if (cap <= b->cells.cap) return CGL_OK;
  const uint64_t keep = b->cells.hwm;
  cgl_status st;
  const uint64_t chunks = batch_scan_blocks((uint32_t)std::min<uint64_t>(cap, 0xFFFFFFFFull)) + 1;
  if ((st = grow(b, b->counts, cap * 4, keep * 4, 0)) || (st = grow(b, b->cell_start, (cap + 1) * 4, 0, 0)) ||
      (st = grow(b, b->cell_gid, cap * 4, keep * 4, 0xFF)) || (st = grow(b, b->big_list, 2 * cap * 4, 0, -1)) ||
      (st = grow(b, b->big_sx, cap * 8, 0, -1)) || (st = grow(b, b->big_sy, cap * 8, 0, -1)) ||
      (st = grow(b, b->big_ns, cap * 4, 0, -1)) || (st = grow(b, b->scan_status, chunks * 8, 0, 0)) ||
      (st = grow(b, b->scan_seq, 8, 0, 0)))
    return st;
  b->cells.cap = cap;
  return CGL_OK;
}

// The collision arena: integer sums (zero between ticks), grids, graph of each cell.
cgl_status reserve_colls(cgl_batch* b, uint64_t cap) {
  if (cap <= b->colls.cap) return CGL_OK;
  const uint64_t keep = b->colls.hwm;
  cgl_status st;
  if ((st = grow(b, b->cgrid_acc, cap * 32, keep * 32, 0)) || (st = grow(b, b->cgrid, cap * 16, 0, 0)) ||
      (st = grow(b, b->coll_gid, cap * 4, keep * 4, 0xFF)))
    return st;
  b->colls.cap = cap;
  return CGL_OK;
}

void refresh_view(cgl_batch* b) {
  BatchView& v = b->view;
  v.slots = (uint32_t)b->jobs.size();
  v.point_hwm = (uint32_t)b->pts.hwm;
  v.units = PairUnits{1.0f, -0.0f};
  v.cell_hwm = (uint32_t)b->cells.hwm;
  v.desc = (const GraphDesc*)b->desc.p;
  v.gid = (const uint32_t*)b->gid.p;
  v.cell_gid = (const uint32_t*)b->cell_gid.p;
  v.pos = (float2*)b->pos.p;
  v.pos_alt = (float2*)b->pos_alt.p;
  v.flags = (const uint8_t*)b->flags.p;
  v.jitter = (const float2*)b->jitter.p;
  v.key = (uint32_t*)b->key.p;
  v.rank = (uint32_t*)b->rank.p;
  v.sorted_idx = (uint32_t*)b->sorted_idx.p;
  v.sorted_pos = (float2*)b->sorted_pos.p;
  v.sib_list = (uint2*)b->sib_list.p;
  v.counts = (uint32_t*)b->counts.p;
  v.cell_start = (uint32_t*)b->cell_start.p;
  v.scan_status = (unsigned long long*)b->scan_status.p;
  v.scan_seq = (unsigned long long*)b->scan_seq.p;
  v.error_word = b->d_error;
  v.big_list = (uint32_t*)b->big_list.p;
  v.big_count = (uint32_t*)b->big_count.p;
  v.big_sx = (long long*)b->big_sx.p;
  v.big_sy = (long long*)b->big_sy.p;
  v.big_ns = (uint32_t*)b->big_ns.p;
  v.rec = (float4*)b->rec.p;
  v.acc = (long long*)b->acc.p;
  v.tiles = (const uint2*)b->tiles.p;
  v.n_tiles = b->n_tiles;
  v.rowptr = (const uint32_t*)b->rowptr.p;
  v.ent = (const uint4*)b->ent.p;
  v.lrow = (const uint32_t*)b->lrow.p;
  v.lwoff = (const uint32_t*)b->lwoff.p;
  v.lanes = (const uint4*)b->lanes.p;
  for (int d = 0; d < 2; ++d) {
    v.lwork[d] = (const uint2*)b->lwork[d].p;
    v.n_lwork[d] = b->n_lwork[d];
  }
  v.heavy_in = (const uint32_t*)b->heavy_in.p;
  v.n_heavy_in = b->n_heavy_in;
  v.heavy_out = (const uint32_t*)b->heavy_out.p;
  v.n_heavy_out = b->n_heavy_out;
  v.ticks = (const BatchTick*)b->ticks.p;
  v.tick_ctr = (uint32_t*)b->tick_ctr.p;
  v.centroid = (long long*)b->centroid.p;
  v.size = (const float*)b->size.p;
  v.cgrid_acc = (long long*)b->cgrid_acc.p;
  v.cgrid = (float4*)b->cgrid.p;
  v.coll_gid = (const uint32_t*)b->coll_gid.p;
  v.coll_hwm = (uint32_t)b->colls.hwm;
  v.any_center = b->any_center ? 1 : 0;
  v.any_collision = b->any_collision ? 1 : 0;
}

// Descriptors, the cell-kernel work list and the long-list rows of all jobs.
cgl_status rebuild_tables(cgl_batch* b) {
  BCU(cudaStreamSynchronize(b->stream));   // no parameter upload may still read h_ticks
  b->params_pending = false;
  const size_t slots = b->jobs.size();
  std::vector<GraphDesc> descs(slots);
  std::vector<uint2> tiles;
  std::vector<uint32_t> hin, hout;
  std::vector<uint2> lwork[2];
  b->any_center = b->any_collision = false;
  for (size_t g = 0; g < slots; ++g) {
    const Job& j = b->jobs[g];
    if (!j.used) { std::memset(&descs[g], 0, sizeof(GraphDesc)); continue; }
    descs[g] = j.desc;
    b->any_center |= (j.stages & kGCenter) != 0;
    b->any_collision |= (j.stages & kGCollision) != 0;
    if (j.stages & kGManybody) {
      const int per_row = j.gf / j.tile;
      for (int t = 0; t < per_row * per_row; ++t) tiles.push_back(make_uint2((uint32_t)g, (uint32_t)t));
    }
    for (uint32_t p : j.heavy_in) hin.push_back((uint32_t)j.p_off + p);
    for (uint32_t p : j.heavy_out) hout.push_back((uint32_t)j.p_off + p);
    for (int d = 0; d < 2; ++d)
      for (uint32_t w = 0; w < j.nw[d]; w += kLinkWarpsPerBlock) lwork[d].push_back(make_uint2((uint32_t)g, w));
  }
  cgl_status st;
  if ((st = grow(b, b->desc, std::max<size_t>(slots, 1) * sizeof(GraphDesc), 0, 0))) return st;
  if ((st = grow(b, b->tiles, std::max<size_t>(tiles.size(), 1) * sizeof(uint2), 0, -1))) return st;
  if ((st = grow(b, b->heavy_in, std::max<size_t>(hin.size(), 1) * 4, 0, -1))) return st;
  if ((st = grow(b, b->heavy_out, std::max<size_t>(hout.size(), 1) * 4, 0, -1))) return st;
  if ((st = grow(b, b->centroid, std::max<size_t>(slots, 1) * 3 * sizeof(long long), 0, 0))) return st;
  for (int d = 0; d < 2; ++d) {
    if ((st = grow(b, b->lwork[d], std::max<size_t>(lwork[d].size(), 1) * sizeof(uint2), 0, -1))) return st;
    if (!lwork[d].empty())
      BCU(cudaMemcpyAsync(b->lwork[d].p, lwork[d].data(), lwork[d].size() * sizeof(uint2), cudaMemcpyHostToDevice,
                          b->stream));
  }
  if (slots) BCU(cudaMemcpyAsync(b->desc.p, descs.data(), slots * sizeof(GraphDesc), cudaMemcpyHostToDevice, b->stream));
  if (!tiles.empty())
    BCU(cudaMemcpyAsync(b->tiles.p, tiles.data(), tiles.size() * sizeof(uint2), cudaMemcpyHostToDevice, b->stream));
  if (!hin.empty()) BCU(cudaMemcpyAsync(b->heavy_in.p, hin.data(), hin.size() * 4, cudaMemcpyHostToDevice, b->stream));
  if (!hout.empty()) BCU(cudaMemcpyAsync(b->heavy_out.p, hout.data(), hout.size() * 4, cudaMemcpyHostToDevice, b->stream));
  if (slots > b->slots_cap) {
    if ((st = grow(b, b->ticks, (size_t)kTickChunk * slots * sizeof(BatchTick), 0, 0))) return st;
    if (b->h_ticks) cudaFreeHost(b->h_ticks);
    b->h_ticks = nullptr;
    BCU(cudaMallocHost((void**)&b->h_ticks, (size_t)kTickChunk * slots * sizeof(BatchTick)));
    b->slots_cap = (uint32_t)slots;
  }
  BCU(cudaStreamSynchronize(b->stream));
  b->n_tiles = (uint32_t)tiles.size();
  b->n_heavy_in = (uint32_t)hin.size();
  b->n_heavy_out = (uint32_t)hout.size();
  for (int d = 0; d < 2; ++d) b->n_lwork[d] = (uint32_t)lwork[d].size();
  refresh_view(b);
  return CGL_OK;
}

cgl_status prepare(cgl_batch* b) {
  if (!b->dirty && b->graph) return CGL_OK;
  cgl_status st = rebuild_tables(b);
  if (st) return st;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  // the scan's status words and tickets start from zero together (its chunk count may have changed)
  if (b->scan_status.p) BCU(cudaMemsetAsync(b->scan_status.p, 0, b->scan_status.bytes, b->stream));
  if (b->scan_seq.p) BCU(cudaMemsetAsync(b->scan_seq.p, 0, b->scan_seq.bytes, b->stream));
  cudaGraph_t g = nullptr;
  BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  batch_launch_tick(b->view, b->stream, b->side, b->fork, b->join);
  cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  if (ce != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "batch graph capture: %s", cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) { b->graph = nullptr; return bfail(b, CGL_CUDA_ERROR, "batch graph: %s", cudaGetErrorString(ce)); }
  b->dirty = false;
  return CGL_OK;
}

// One tick of one job on the host: whether it runs, its f32 alpha and peel
// seed, then Store.addAlpha (Store/index.ts:328-332).
BatchTick host_tick(Job& j) {
  BatchTick t{0.f, 0u, 0u, 0u};
  if (!j.used) return t;
  if (j.max_ticks && j.tick >= j.max_ticks) j.running = false;
  if (j.running && j.stop_below_min && j.alpha < kAlphaMin) { j.running = false; j.progress = 1; }
  if (!j.running) return t;
  t.active = 1;
  t.alpha = (float)j.alpha;
  if (j.stages & kGManybody) {
    const float seed = (float)j.rng.uniform(0, 1);
    std::memcpy(&t.seed_bits, &seed, 4);
  }
  j.alpha += (0 - j.alpha) * j.decay_factor;
  j.progress = std::sqrt(std::min(1.0, kAlphaMin / j.alpha));
  j.tick++;
  return t;
}

void release(cgl_batch* b, Job& j) {
  b->pts.release(j.p_off, j.n);
  b->cells.release(j.cell_off, j.cells);
  b->recs.release(j.rec_off, j.recs);
  b->accs.release(j.acc_off, j.accs);
  b->rows.release(j.rp_in, j.rows_n[0]);
  b->rows.release(j.rp_out, j.rows_n[1]);
  b->ents.release(j.e_in, j.ents_n[0]);
  b->ents.release(j.e_out, j.ents_n[1]);
  b->lrows.release(j.lr_off, j.lrs);
  b->lwoffs.release(j.lw_off, j.lws);
  b->lanes_a.release(j.ln_off, j.lns);
  b->colls.release(j.coll_off, j.coll_cells);
}

// ---------------------------------------------------------------- ingest --
// A job's ingest in two steps.  prepare_job is host work only (no CUDA call,
// nothing shared): positions and their rescale, the random draws (the
// reference's stream is sequential per job), the host link lists of small
// jobs, point sizes and collision grid.  Many jobs prepare on many host
// threads at once (cgl_batch_add_many).  commit_job then takes the arena
// ranges and uploads, in job order on the batch's stream.
struct HostJob {
  Job j;
  cgl_status status = CGL_OK;
  std::string err;
  double space = 0;
  FixedScale fx{};
  std::vector<float2> pos;
  std::vector<uint8_t> absent;
  bool dev_jitter = false;     // counter stream: the device draws the jitter
  uint64_t jitter_base = 0;
  std::vector<float2> jit;
  const float* links = nullptr;   // the caller's array (read again at commit)
  bool has_links = false;
  bool dev_links = false;      // the device builds the link lists (commit may fall back)
  uint32_t m = 0;              // valid links
  ingest::Rng rng_links;       // the stream where the link draws start
  std::vector<float> draws;    // reference stream, device build: 2m rest-length draws
  ingest::Csr cin, cout_;      // host build
  std::vector<uint32_t> lrow, lwoff;   // host build: the light rows by warps, incoming then outgoing
  std::vector<uint4> lanes;
  std::vector<float> sizes;    // collision: resolved point sizes
};

// The light rows of one direction by warps (GraphDesc::lr, lw, ln): rows
// order[nh..n) in that order (every point in index order when there are no
// lists), warp w's 32 lists interleaved by lane from woff[w], each padded with
// absent entries to the warp's first (longest) list.  Appended to the vectors;
// returns the warps.
uint32_t host_warp_layout(const ingest::Csr& c, uint32_t n, uint32_t nh, std::vector<uint32_t>& lrow,
                          std::vector<uint32_t>& woff, std::vector<uint4>& lanes, uint64_t* lane_ents) {
  const uint32_t nw = (n - nh + 31) / 32;
  const bool lists = !c.order.empty();
  auto row = [&](uint32_t t) { return lists ? c.order[t] : t; };
  auto len = [&](uint32_t p) { return c.rowptr[p + 1] - c.rowptr[p]; };
  const size_t r0 = lrow.size(), w0 = woff.size(), l0 = lanes.size();
  lrow.resize(r0 + 32ull * nw, kNoPoint);
  woff.resize(w0 + nw + 1);
  uint64_t total = 0;
  for (uint32_t w = 0; w < nw; ++w) {
    woff[w0 + w] = (uint32_t)total;
    total += 32ull * len(row(nh + 32 * w));
  }
  woff[w0 + nw] = (uint32_t)total;
  lanes.resize(l0 + total, make_uint4(kAbsentTarget, 0u, 0u, 0u));
  for (uint32_t t = 0; t < n - nh; ++t) {
    const uint32_t p = row(nh + t);
    lrow[r0 + t] = p;
    const uint32_t e0 = c.rowptr[p], m = len(p);
    uint4* col = lanes.data() + l0 + woff[w0 + t / 32] + (t & 31);
    for (uint32_t k = 0; k < m; ++k) col[32 * (size_t)k] = c.ent[e0 + k];
  }
  *lane_ents = total;
  return nw;
}

// A job whose lists the host built: their sizes, long lists and warp layout.
// Rows are kept as CSR only for a direction with long lists.
void host_links_layout(HostJob& h) {
  Job& j = h.j;
  j.m_in = h.cin.ent.size();
  j.m_out = h.cout_.ent.size();
  j.heavy_in = h.cin.heavy;
  j.heavy_out = h.cout_.heavy;
  h.lrow.clear();
  h.lwoff.clear();
  h.lanes.clear();
  j.nw[0] = host_warp_layout(h.cin, (uint32_t)j.n, (uint32_t)j.heavy_in.size(), h.lrow, h.lwoff, h.lanes,
                             &j.lane_ents[0]);
  j.nw[1] = host_warp_layout(h.cout_, (uint32_t)j.n, (uint32_t)j.heavy_out.size(), h.lrow, h.lwoff, h.lanes,
                             &j.lane_ents[1]);
  for (int d = 0; d < 2; ++d) {
    const bool heavy = !(d == 0 ? j.heavy_in : j.heavy_out).empty();
    j.rows_n[d] = heavy ? j.n + 1 : 0;
    j.ents_n[d] = heavy ? (d == 0 ? j.m_in : j.m_out) : 0;
  }
  j.lrs = 32ull * (j.nw[0] + j.nw[1]);
  j.lws = (uint64_t)j.nw[0] + 1 + j.nw[1] + 1;
  j.lns = j.lane_ents[0] + j.lane_ents[1];
}

cgl_status prep_fail(HostJob& h, cgl_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  h.err = buf;
  h.status = st;
  return st;
}

cgl_status prepare_job(const cgl_batch_job& in, HostJob& h) {
  const cgl_config* cfg = in.cfg;
  if (!cfg || (!in.xy && in.n_floats) || (!in.links && in.n_link_floats) || (!in.sizes && in.n_sizes))
    return prep_fail(h, CGL_INVALID_ARG, "null array");
  if (!cfg->enable_simulation) return prep_fail(h, CGL_INVALID_ARG, "enableSimulation is off");
  Job& j = h.j;
  j.used = true;
  j.cfg = *cfg;
  j.cfg.random_seed_text = nullptr;   // the seed is used here only
  j.n = in.n_floats / 2;
  j.E = in.n_link_floats / 2;
  if (j.n == 0) return prep_fail(h, CGL_INVALID_ARG, "a job needs points");
  if (j.n > (1ull << 24)) return prep_fail(h, CGL_INVALID_ARG, "%llu points exceed 2^24", (unsigned long long)j.n);
  const uint32_t mask = cfg->stage_mask;
  ingest::seed_rng(*cfg, j.rng);
  h.space = ingest::adjusted_space(*cfg);
  // Points.updatePositions (Points/index.ts:390-413), as cgl_render for a fresh engine
  if (ingest::should_rescale(*cfg, false)) {
    std::vector<float> scaled(in.xy, in.xy + 2 * j.n);
    ingest::rescale_positions(scaled.data(), j.n, cfg->space_size);
    j.live = ingest::canonical_positions(scaled.data(), j.n, h.pos, h.absent);
  } else {
    j.live = ingest::canonical_positions(in.xy, j.n, h.pos, h.absent);
  }
  int fbits = 0;
  h.fx = ingest::fixed_for(j.n, h.space, &fbits);
  const ingest::Grid grid = ingest::grid_for(j.n);
  j.gf = grid.gf;
  j.levels = grid.levels;
  j.tile = std::min(32, j.gf);   // kb_cells: 2 x 2 cells per thread
  // the jitter draws come first (ForceManyBody.create), then the link draws
  const uint64_t T = (uint64_t)std::ceil(std::sqrt((double)j.n));
  h.dev_jitter = j.rng.counter && !(cfg->device_ingest_min_links > (double)j.n);
  h.jitter_base = j.rng.ctr;
  if (h.dev_jitter) j.rng.ctr += 2 * T * T;
  else ingest::jitter(j.rng, j.n, h.jit);
  h.links = in.links;
  h.has_links = j.E > 0;
  h.dev_links = h.has_links && j.E < 0xFFFFFFF0ull && !(cfg->device_ingest_min_links > (double)j.E);
  h.rng_links = j.rng;
  if (h.dev_links) {
    // GraphData.isPointIndex of both ends (GraphData/index.ts:286-289): one draw per list entry
    uint64_t m = 0;
    for (uint64_t i = 0; i < j.E; ++i)
      m += ingest::is_point_index(in.links[2 * i], j.n) && ingest::is_point_index(in.links[2 * i + 1], j.n);
    h.m = (uint32_t)m;
    if (!j.rng.counter && m) {
      h.draws.resize(2 * (size_t)m);
      j.rng.fill_unit_f32(h.draws.data(), 2 * m);
    } else {
      j.rng.ctr += 2 * m;
    }
    j.m_in = j.m_out = m;
    j.rows_n[0] = j.rows_n[1] = j.n + 1;
    j.ents_n[0] = j.ents_n[1] = m;
  } else {
    if (h.has_links) ingest::build_links(in.links, j.E, j.n, nullptr, h.absent, j.rng, h.cin, h.cout_);
    else { h.cin.rowptr.assign(j.n + 1, 0); h.cout_.rowptr.assign(j.n + 1, 0); }
    host_links_layout(h);
  }
  j.stages = 0;
  if (cfg->simulation_gravity != 0 && (mask & CGL_STAGE_GRAVITY)) j.stages |= kGGravity;
  if (cfg->simulation_center != 0 && (mask & CGL_STAGE_CENTER)) j.stages |= kGCenter;
  if (mask & CGL_STAGE_MANYBODY) j.stages |= kGManybody;
  if (h.has_links && (mask & CGL_STAGE_LINK_IN)) j.stages |= kGLinkIn;
  if (h.has_links && (mask & CGL_STAGE_LINK_OUT)) j.stages |= kGLinkOut;
  if (cfg->simulation_collision != 0 && (mask & CGL_STAGE_COLLISION)) j.stages |= kGCollision;
  j.decay_factor = 1 - std::pow(kAlphaMin, 1 / cfg->simulation_decay);
  j.max_ticks = in.max_ticks;
  j.stop_below_min = in.stop_below_alpha_min != 0;
  j.cells = (uint64_t)j.gf * j.gf;
  j.recs = ingest::level_base(j.levels);
  int lv_tile = j.levels - 1;
  for (int g = j.tile; g > 1 && lv_tile > 0; g >>= 1) --lv_tile;
  j.accs = ingest::level_base(lv_tile);
  GraphDesc& D = j.desc;
  std::memset(&D, 0, sizeof(D));
  if (j.stages & kGCollision) {
    // GraphData.getResolvedPointSize (GraphData/index.ts:189-194) and
    // ForceCollision.create (ForceCollision/index.ts:61-95)
    const bool has = in.sizes != nullptr;
    h.sizes.resize(j.n);
    double max_size = cfg->point_default_size;
    for (uint64_t i = 0; i < j.n; ++i) {
      float r = NAN;
      if (has && i < in.n_sizes) r = in.sizes[i];
      if (std::isnan(r)) r = h.absent[i] ? 0.f : (float)cfg->point_default_size;
      h.sizes[i] = r;
      if (has) max_size = std::max(max_size, (double)r);
    }
    const double cr = std::isnan(cfg->simulation_collision_radius) ? 0 : cfg->simulation_collision_radius;
    const double eff = (cr > 0 ? cr : max_size * 0.5) + cfg->simulation_collision_padding;
    const double cell = std::max(eff * 2, 8.0);
    const int cgrid = (int)std::min(512.0, std::max(1.0, std::floor(h.space / cell)));
    D.coll_grid = cgrid;
    D.coll_cell = (float)(h.space / cgrid);
    D.coll_strength = (float)cfg->simulation_collision;
    D.coll_radius = (float)cr;
    D.coll_padding = (float)cfg->simulation_collision_padding;
    j.coll_cells = 4ull * (uint64_t)cgrid * (uint64_t)cgrid;
  }
  return CGL_OK;
}

cgl_status commit_job(cgl_batch* b, HostJob& h, uint32_t* id) {
  Job& j = h.j;
  const cgl_config* cfg = &j.cfg;
  // link lists on the device when asked for and when its transient buffers fit the budget
  Temp tmp{b};
  bool dev_links = h.dev_links;
  const uint64_t big = std::max<uint64_t>(j.E + 1, j.n + 1);
  const size_t tmp_words = std::max(dingest::sort_temp_words(big), dingest::scan_temp_words(big));
  if (dev_links && b->budget > 0 &&
      (double)b->dev_bytes + 8.0 * j.E + 4.0 * (j.E + 1) + 8.0 * (j.n + 1) + 16.0 * big + 4.0 * tmp_words +
              4.0 * h.draws.size() > b->budget)
    dev_links = false;
  float2* d_links = nullptr;
  float* d_draws = nullptr;
  uint32_t *d_valid = nullptr, *d_len_in = nullptr, *d_len_out = nullptr, *d_tmp = nullptr, *d_stats = nullptr;
  uint32_t *d_kin = nullptr, *d_kout = nullptr, *d_vin = nullptr, *d_vout = nullptr;
  uint32_t* d_ord[2] = {nullptr, nullptr};   // rows by list length
  uint32_t* d_wo[2] = {nullptr, nullptr};    // warp layout offsets
  if (dev_links) {
    d_links = tmp.get<float2>(j.E);
    d_valid = tmp.get<uint32_t>(j.E + 1);
    d_len_in = tmp.get<uint32_t>(j.n + 1);
    d_len_out = tmp.get<uint32_t>(j.n + 1);
    d_tmp = tmp.get<uint32_t>(tmp_words);
    d_stats = tmp.get<uint32_t>(4);
    d_kin = tmp.get<uint32_t>(big);
    d_kout = tmp.get<uint32_t>(big);
    d_vin = tmp.get<uint32_t>(big);
    d_vout = tmp.get<uint32_t>(big);
    if (!h.draws.empty()) d_draws = tmp.get<float>(h.draws.size());
    dev_links = d_links && d_valid && d_len_in && d_len_out && d_tmp && d_stats && d_kin && d_kout && d_vin &&
                d_vout && (h.draws.empty() || d_draws);
  }
  if (h.dev_links && !dev_links) {
    // the device build did not fit: the host build, from the same point of the
    // stream (it draws the same 2m values prepare_job drew)
    j.rng = h.rng_links;
    ingest::build_links(h.links, j.E, j.n, nullptr, h.absent, j.rng, h.cin, h.cout_);
    host_links_layout(h);
  }
  uint32_t dev_stats[4] = {0, 0, 0, 0};
  if (dev_links) {
    cudaStream_t s = b->stream;
    const uint32_t E32 = (uint32_t)j.E, N32 = (uint32_t)j.n;
    uint32_t dev_m = 0;
    BCU(cudaMemcpyAsync(d_links, h.links, j.E * sizeof(float2), cudaMemcpyHostToDevice, s));
    if (d_draws) BCU(cudaMemcpyAsync(d_draws, h.draws.data(), h.draws.size() * 4, cudaMemcpyHostToDevice, s));
    BCU(cudaMemsetAsync(d_valid, 0, (j.E + 1) * 4, s));
    BCU(cudaMemsetAsync(d_len_in, 0, (j.n + 1) * 4, s));
    BCU(cudaMemsetAsync(d_len_out, 0, (j.n + 1) * 4, s));
    BCU(cudaMemsetAsync(d_stats, 0, 16, s));
    dingest::count_links(d_links, E32, N32, d_valid, d_len_in, d_len_out, s);
    dingest::scan_exclusive(d_valid, E32 + 1, d_tmp, s);
    dingest::len_stats(d_len_in, N32, d_stats, s);
    dingest::len_stats(d_len_out, N32, d_stats + 2, s);
    BCU(cudaMemcpyAsync(&dev_m, d_valid + j.E, 4, cudaMemcpyDeviceToHost, s));
    BCU(cudaMemcpyAsync(dev_stats, d_stats, 16, cudaMemcpyDeviceToHost, s));
    BCU(cudaStreamSynchronize(s));
    if (dev_m != h.m) return bfail(b, CGL_CUDA_ERROR, "link count %u on the device, %u on the host", dev_m, h.m);
    // each direction's rows by list length, longest first (the long lists are
    // its first stats[1] / stats[3]), and the warp layout's offsets: sizes
    // known before the arena ranges are taken
    uint32_t lane_tot[2] = {0, 0};
    for (int d = 0; d < 2; ++d) {
      const uint32_t nh = dev_stats[2 * d + 1];
      j.nw[d] = (N32 - nh + 31) / 32;
      d_ord[d] = tmp.get<uint32_t>(j.n);
      d_wo[d] = tmp.get<uint32_t>(j.nw[d] + 1);
      if (!d_ord[d] || !d_wo[d]) return bfail(b, CGL_OOM, "link warp layout: no device memory for its temporaries");
      uint32_t* len = d == 0 ? d_len_in : d_len_out;
      dingest::len_keys(len, N32, d_stats + 2 * d, d_kout, d_ord[d], s);
      dingest::sort_pairs(d_kout, d_ord[d], N32, dingest::key_bits(dev_stats[2 * d]), d_tmp, s);
      batch_warp_lengths(d_ord[d], len, nh, N32, d_wo[d], s);
      dingest::scan_exclusive(d_wo[d], j.nw[d] + 1, d_tmp, s);
      BCU(cudaMemcpyAsync(&lane_tot[d], d_wo[d] + j.nw[d], 4, cudaMemcpyDeviceToHost, s));
      std::vector<uint32_t>& hv = d == 0 ? j.heavy_in : j.heavy_out;
      hv.resize(nh);
      if (nh) BCU(cudaMemcpyAsync(hv.data(), d_ord[d], nh * 4, cudaMemcpyDeviceToHost, s));
    }
    BCU(cudaGetLastError());
    BCU(cudaStreamSynchronize(s));
    j.lane_ents[0] = lane_tot[0];
    j.lane_ents[1] = lane_tot[1];
    j.lrs = 32ull * (j.nw[0] + j.nw[1]);
    j.lws = (uint64_t)j.nw[0] + 1 + j.nw[1] + 1;
    j.lns = j.lane_ents[0] + j.lane_ents[1];
  }
  // arena ranges (grow the arenas when full)
  cgl_status st;
  auto take = [&](Arena& a, uint64_t n, uint64_t* off, int kind) -> cgl_status {
    if (a.alloc(n, off)) return CGL_OK;
    const uint64_t cap = grown(a.cap, a.hwm + n);
    cgl_status s2 = CGL_OK;
    if (kind == 0) s2 = reserve_points(b, cap);
    else if (kind == 1) s2 = reserve_cells(b, cap);
    else if (kind == 2) s2 = grow(b, b->rec, cap * sizeof(float4), a.hwm * sizeof(float4), 0);
    else if (kind == 3) s2 = grow(b, b->acc, cap * 3 * sizeof(long long), a.hwm * 3 * sizeof(long long), 0);
    else if (kind == 4) s2 = grow(b, b->rowptr, cap * 4, a.hwm * 4, -1);
    else if (kind == 5) s2 = grow(b, b->ent, cap * sizeof(uint4), a.hwm * sizeof(uint4), -1);
    else if (kind == 6) s2 = reserve_colls(b, cap);
    else if (kind == 7) s2 = grow(b, b->lrow, cap * 4, a.hwm * 4, -1);
    else if (kind == 8) s2 = grow(b, b->lwoff, cap * 4, a.hwm * 4, -1);
    else s2 = grow(b, b->lanes, cap * sizeof(uint4), a.hwm * sizeof(uint4), -1);
    if (s2) return s2;
    if ((kind >= 2 && kind <= 5) || kind >= 7) a.cap = cap;
    b->dirty = true;
    return a.alloc(n, off) ? CGL_OK : bfail(b, CGL_OOM, "arena allocation failed");
  };
  // Take every range; on a refusal give back exactly the ranges already taken.
  struct Want { Arena* a; uint64_t n; uint64_t* off; int kind; };
  const Want wants[] = {{&b->pts, j.n, &j.p_off, 0},        {&b->cells, j.cells, &j.cell_off, 1},
                        {&b->recs, j.recs, &j.rec_off, 2},   {&b->accs, j.accs, &j.acc_off, 3},
                        {&b->rows, j.rows_n[0], &j.rp_in, 4}, {&b->rows, j.rows_n[1], &j.rp_out, 4},
                        {&b->ents, j.ents_n[0], &j.e_in, 5}, {&b->ents, j.ents_n[1], &j.e_out, 5},
                        {&b->colls, j.coll_cells, &j.coll_off, 6}, {&b->lrows, j.lrs, &j.lr_off, 7},
                        {&b->lwoffs, j.lws, &j.lw_off, 8},   {&b->lanes_a, j.lns, &j.ln_off, 9}};
  int taken = 0;
  st = CGL_OK;
  for (const Want& w : wants) {
    if ((st = take(*w.a, w.n, w.off, w.kind))) break;
    ++taken;
  }
  if (!st && (b->pts.hwm > 0xFFFFFF00ull || b->cells.hwm > 0xFFFFFF00ull || b->ents.hwm > 0xFFFFFF00ull ||
              b->colls.hwm > 0xFFFFFF00ull || b->lrows.hwm > 0xFFFFFF00ull || b->lwoffs.hwm > 0xFFFFFF00ull ||
              b->lanes_a.hwm > 0xFFFFFF00ull))
    st = bfail(b, CGL_OOM, "arena index space (32 bits) exhausted");
  if (st) {
    for (int k = 0; k < taken; ++k) wants[k].a->release(*wants[k].off, wants[k].n);
    return st;
  }
  // From here on a CUDA error gives the job's arena ranges back before returning.
  auto give_back = [&]() {
    for (const Want& w : wants) w.a->release(*w.off, w.n);
  };
#define JCU(call)                                                                                    \
  do {                                                                                               \
    cudaError_t _e = (call);                                                                         \
    if (_e != cudaSuccess) {                                                                         \
      give_back();                                                                                   \
      return bfail(b, _e == cudaErrorMemoryAllocation ? CGL_OOM : CGL_CUDA_ERROR, "%s: %s", #call,  \
                   cudaGetErrorString(_e));                                                          \
    }                                                                                                \
  } while (0)
  // rows, entries and neighbours stay graph-local (the kernels add the job's offsets)
  std::vector<uint8_t> flags(j.n);
  for (uint64_t i = 0; i < j.n; ++i) flags[i] = h.absent[i] ? kAbsent : 0;
  const uint32_t g = [&]() {
    for (uint32_t sl = 0; sl < b->jobs.size(); ++sl)
      if (!b->jobs[sl].used) return sl;
    b->jobs.emplace_back();
    return (uint32_t)(b->jobs.size() - 1);
  }();
  std::vector<uint32_t> gids(j.n, g), cgids(j.cells, g);
  cudaStream_t s = b->stream;
  JCU(cudaMemcpyAsync((float2*)b->pos.p + j.p_off, h.pos.data(), j.n * 8, cudaMemcpyHostToDevice, s));
  if (h.dev_jitter) dingest::jitter(j.rng.seed, h.jitter_base, (uint32_t)j.n, (float2*)b->jitter.p + j.p_off, s);
  else JCU(cudaMemcpyAsync((float2*)b->jitter.p + j.p_off, h.jit.data(), j.n * 8, cudaMemcpyHostToDevice, s));
  JCU(cudaMemcpyAsync((uint8_t*)b->flags.p + j.p_off, flags.data(), j.n, cudaMemcpyHostToDevice, s));
  JCU(cudaMemcpyAsync((uint32_t*)b->gid.p + j.p_off, gids.data(), j.n * 4, cudaMemcpyHostToDevice, s));
  JCU(cudaMemcpyAsync((uint32_t*)b->cell_gid.p + j.cell_off, cgids.data(), j.cells * 4, cudaMemcpyHostToDevice, s));
  JCU(cudaMemsetAsync((uint32_t*)b->counts.p + j.cell_off, 0, j.cells * 4, s));
  JCU(cudaMemsetAsync((long long*)b->acc.p + 3 * j.acc_off, 0, j.accs * 3 * sizeof(long long), s));
  std::vector<uint32_t> coll_gids;
  if (j.coll_cells) {
    coll_gids.assign(j.coll_cells, g);
    JCU(cudaMemcpyAsync((float*)b->size.p + j.p_off, h.sizes.data(), j.n * 4, cudaMemcpyHostToDevice, s));
    JCU(cudaMemcpyAsync((uint32_t*)b->coll_gid.p + j.coll_off, coll_gids.data(), j.coll_cells * 4,
                        cudaMemcpyHostToDevice, s));
    JCU(cudaMemsetAsync((long long*)b->cgrid_acc.p + 4 * j.coll_off, 0, j.coll_cells * 32, s));
  }
  if (dev_links) {
    // (row, link) pairs sorted by row, entries filled in place with arena
    // indices; the flags of this job are already queued above
    const uint32_t E32 = (uint32_t)j.E, N32 = (uint32_t)j.n, M = h.m;
    const uint8_t* flags_j = (const uint8_t*)b->flags.p + j.p_off;
    dingest::compact_links(d_links, E32, d_valid, d_kin, d_kout, d_vin, d_vout, s);
    const int row_bits = dingest::key_bits(j.n - 1);
    dingest::sort_pairs(d_kin, d_vin, M, row_bits, d_tmp, s);
    dingest::sort_pairs(d_kout, d_vout, M, row_bits, d_tmp, s);
    const uint64_t links_base = h.rng_links.ctr;
    dingest::fill_csr(d_kin, d_vin, M, d_links, true, d_len_in, d_len_out, nullptr, flags_j, d_draws, j.rng.seed,
                      links_base, 0u, (uint4*)b->ent.p + j.e_in, s);
    dingest::fill_csr(d_kout, d_vout, M, d_links, false, d_len_in, d_len_out, nullptr, flags_j,
                      d_draws ? d_draws + M : nullptr, j.rng.seed, links_base + M, 0u, (uint4*)b->ent.p + j.e_out, s);
    // row pointers (exclusive scan of the lengths), then the light rows by warps from them
    for (int d = 0; d < 2; ++d) {
      uint32_t* len = d == 0 ? d_len_in : d_len_out;
      uint32_t* rp = (uint32_t*)b->rowptr.p + (d == 0 ? j.rp_in : j.rp_out);
      dingest::scan_exclusive(len, N32 + 1, d_tmp, s);
      dingest::copy_u32(len, rp, N32 + 1, s);
      const uint32_t nh = dev_stats[2 * d + 1];
      uint32_t* woff = (uint32_t*)b->lwoff.p + j.lw_off + (d == 0 ? 0 : j.nw[0] + 1);
      JCU(cudaMemcpyAsync(woff, d_wo[d], ((size_t)j.nw[d] + 1) * 4, cudaMemcpyDeviceToDevice, s));
      batch_warp_rows(d_ord[d], nh, N32, (uint32_t*)b->lrow.p + j.lr_off + (d == 0 ? 0 : 32ull * j.nw[0]), s);
      if (j.lane_ents[d])
        launch_fill_lanes(d_ord[d], rp, (const uint4*)b->ent.p + (d == 0 ? j.e_in : j.e_out), nh, N32, woff,
                          (uint4*)b->lanes.p + j.ln_off + (d == 0 ? 0 : j.lane_ents[0]), s);
    }
    JCU(cudaGetLastError());
  } else {
    if (j.rows_n[0]) {
      JCU(cudaMemcpyAsync((uint32_t*)b->rowptr.p + j.rp_in, h.cin.rowptr.data(), (j.n + 1) * 4, cudaMemcpyHostToDevice, s));
      JCU(cudaMemcpyAsync((uint4*)b->ent.p + j.e_in, h.cin.ent.data(), j.m_in * 16, cudaMemcpyHostToDevice, s));
    }
    if (j.rows_n[1]) {
      JCU(cudaMemcpyAsync((uint32_t*)b->rowptr.p + j.rp_out, h.cout_.rowptr.data(), (j.n + 1) * 4, cudaMemcpyHostToDevice, s));
      JCU(cudaMemcpyAsync((uint4*)b->ent.p + j.e_out, h.cout_.ent.data(), j.m_out * 16, cudaMemcpyHostToDevice, s));
    }
    JCU(cudaMemcpyAsync((uint32_t*)b->lrow.p + j.lr_off, h.lrow.data(), j.lrs * 4, cudaMemcpyHostToDevice, s));
    JCU(cudaMemcpyAsync((uint32_t*)b->lwoff.p + j.lw_off, h.lwoff.data(), j.lws * 4, cudaMemcpyHostToDevice, s));
    if (j.lns) JCU(cudaMemcpyAsync((uint4*)b->lanes.p + j.ln_off, h.lanes.data(), j.lns * 16, cudaMemcpyHostToDevice, s));
  }
  if (dev_links) JCU(cudaStreamSynchronize(s));   // the temporaries' kernels; pageable uploads are staged at the call
#undef JCU
  GraphDesc& D = j.desc;
  D.p_off = (uint32_t)j.p_off;
  D.n = (uint32_t)j.n;
  D.cell_off = (uint32_t)j.cell_off;
  D.rec_off = (uint32_t)j.rec_off;
  D.acc_off = (uint32_t)j.acc_off;
  D.acc_cells = (uint32_t)j.accs;
  D.rp_in = (uint32_t)j.rp_in;
  D.rp_out = (uint32_t)j.rp_out;
  D.e_in = (uint32_t)j.e_in;
  D.e_out = (uint32_t)j.e_out;
  D.lr[0] = (uint32_t)j.lr_off;
  D.lr[1] = (uint32_t)(j.lr_off + 32ull * j.nw[0]);
  D.lw[0] = (uint32_t)j.lw_off;
  D.lw[1] = (uint32_t)(j.lw_off + j.nw[0] + 1);
  D.ln[0] = (uint32_t)j.ln_off;
  D.ln[1] = (uint32_t)(j.ln_off + j.lane_ents[0]);
  D.nw[0] = j.nw[0];
  D.nw[1] = j.nw[1];
  D.gf = j.gf;
  D.levels = j.levels;
  D.tile = j.tile;
  D.stages = j.stages;
  D.space = (float)h.space;
  D.csf = (float)(h.space / j.gf);
  D.friction = (float)cfg->simulation_friction;
  D.gravity = (float)cfg->simulation_gravity;
  D.repulsion = (float)cfg->simulation_repulsion;
  D.link_spring = (float)cfg->simulation_link_spring;
  D.link_distance = (float)cfg->simulation_link_distance;
  D.link_r0 = (float)cfg->simulation_link_dist_random_variation_range[0];
  D.link_r1 = (float)cfg->simulation_link_dist_random_variation_range[1];
  D.fx = h.fx;
  D.center = (float)cfg->simulation_center;
  D.level_guard = D.csf >= 2.0f && D.space <= 33554432.0f;   // 2^25
  D.coll_off = (uint32_t)j.coll_off;
  b->jobs[g] = std::move(j);
  b->dirty = true;
  *id = g;
  return CGL_OK;
}

}  // namespace

extern "C" {

cgl_status cgl_batch_create(int32_t device, double hbm_budget_bytes, cgl_batch** out) {
  if (!out) return CGL_INVALID_ARG;
  *out = nullptr;
  cgl_batch* b = new cgl_batch();
  b->device = device;
  b->budget = hbm_budget_bytes;
  cudaError_t ce = cudaSetDevice(device);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
  for (int k = 0; k < 2 && ce == cudaSuccess; ++k) {
    ce = cudaEventCreateWithFlags(&b->fork[k], cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming);
  }
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->params_copied, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaHostAlloc((void**)&b->h_error, sizeof(uint32_t), cudaHostAllocMapped);
  if (ce == cudaSuccess) ce = cudaHostGetDevicePointer((void**)&b->d_error, b->h_error, 0);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    cgl_batch_destroy(b);
    return CGL_CUDA_ERROR;
  }
  *b->h_error = 0;
  cgl_status st;
  if ((st = grow(b, b->big_count, 32, 0, 0)) || (st = grow(b, b->tick_ctr, 4, 0, 0)) ||
      (st = reserve_cells(b, 1024)) || (st = reserve_points(b, 1024))) {
    cgl_batch_destroy(b);
    return st;
  }
  refresh_view(b);
  *out = b;
  return CGL_OK;
}

cgl_status cgl_batch_destroy(cgl_batch* b) {
  if (!b) return CGL_INVALID_ARG;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  Buf* all[] = {&b->sib_list, &b->gid, &b->pos, &b->pos_alt, &b->flags, &b->jitter, &b->key, &b->rank, &b->sorted_idx,
                &b->sorted_pos, &b->counts, &b->cell_start, &b->cell_gid, &b->big_list, &b->big_sx, &b->big_sy,
                &b->big_ns, &b->scan_status, &b->scan_seq, &b->big_count, &b->tick_ctr, &b->rec, &b->acc, &b->rowptr,
                &b->ent, &b->desc, &b->tiles, &b->heavy_in, &b->heavy_out, &b->ticks, &b->size, &b->cgrid_acc,
                &b->cgrid, &b->coll_gid, &b->centroid, &b->lrow, &b->lwoff, &b->lanes, &b->lwork[0],
                &b->lwork[1]};
  for (Buf* x : all)
    if (x->p) cudaFree(x->p);
  if (b->h_ticks) cudaFreeHost(b->h_ticks);
  if (b->h_error) cudaFreeHost(b->h_error);
  if (b->h_stage) cudaFreeHost(b->h_stage);
  for (int k = 0; k < 2; ++k) {
    if (b->fork[k]) cudaEventDestroy(b->fork[k]);
    if (b->join[k]) cudaEventDestroy(b->join[k]);
  }
  if (b->params_copied) cudaEventDestroy(b->params_copied);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CGL_OK;
}

const char* cgl_batch_last_error(cgl_batch* b) { return b ? b->err.c_str() : "null batch"; }

cgl_status cgl_batch_add(cgl_batch* b, const cgl_config* cfg, const float* xy, uint64_t n_floats, const float* links,
                         uint64_t n_link_floats, uint32_t max_ticks, int32_t stop_below_alpha_min, uint32_t* id) {
  if (!b || !cfg || !id || (!xy && n_floats) || (!links && n_link_floats)) return CGL_INVALID_ARG;
  b->err.clear();
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "cudaSetDevice");
  cgl_batch_job in{};
  in.cfg = cfg;
  in.xy = xy;
  in.n_floats = n_floats;
  in.links = links;
  in.n_link_floats = n_link_floats;
  in.max_ticks = max_ticks;
  in.stop_below_alpha_min = stop_below_alpha_min;
  HostJob h;
  if (prepare_job(in, h)) return bfail(b, h.status, "%s", h.err.c_str());
  return commit_job(b, h, id);
}

cgl_status cgl_batch_add_many(cgl_batch* b, uint32_t count, const cgl_batch_job* jobs, uint32_t* ids,
                              uint32_t threads, uint32_t* added) {
  if (added) *added = 0;
  if (!b || (!jobs && count) || (!ids && count)) return CGL_INVALID_ARG;
  b->err.clear();
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "cudaSetDevice");
  if (count == 0) return CGL_OK;
  unsigned nt = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, count);
  // Prepare in a sliding window of jobs (bounded host memory) on nt threads,
  // commit in job order as each becomes ready.
  const uint32_t window = std::max<uint32_t>(4 * nt, 16);
  std::vector<std::unique_ptr<HostJob>> ready(count);
  std::vector<std::atomic<bool>> done(count);
  for (auto& d : done) d.store(false);
  std::atomic<uint32_t> next{0};
  std::atomic<uint32_t> committed{0};
  std::atomic<bool> stop{false};
  std::mutex mu;
  std::condition_variable cv;
  auto worker = [&]() {
    for (;;) {
      uint32_t k = next.fetch_add(1);
      if (k >= count || stop.load()) return;
      {   // stay within the window ahead of the commits
        std::unique_lock<std::mutex> lock(mu);
        cv.wait(lock, [&] { return k < committed.load() + window || stop.load(); });
      }
      if (stop.load()) return;
      auto h = std::make_unique<HostJob>();
      prepare_job(jobs[k], *h);
      {
        std::lock_guard<std::mutex> lock(mu);
        ready[k] = std::move(h);
        done[k].store(true);
      }
      cv.notify_all();
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t) pool.emplace_back(worker);
  cgl_status st = CGL_OK;
  for (uint32_t k = 0; k < count; ++k) {
    std::unique_ptr<HostJob> h;
    {
      std::unique_lock<std::mutex> lock(mu);
      cv.wait(lock, [&] { return done[k].load(); });
      h = std::move(ready[k]);
    }
    if (h->status) st = bfail(b, h->status, "job %u: %s", k, h->err.c_str());
    else st = commit_job(b, *h, &ids[k]);
    if (st) break;
    committed.store(k + 1);
    if (added) *added = k + 1;
    cv.notify_all();
  }
  stop.store(true);
  cv.notify_all();
  for (auto& t : pool) t.join();
  return st;
}


cgl_status cgl_batch_remove(cgl_batch* b, uint32_t id) {
  if (!b || id >= b->jobs.size() || !b->jobs[id].used) return CGL_INVALID_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "cudaSetDevice");
  Job& j = b->jobs[id];
  BCU(cudaStreamSynchronize(b->stream));
  BCU(cudaMemsetAsync((uint32_t*)b->gid.p + j.p_off, 0xFF, j.n * 4, b->stream));
  release(b, j);
  j = Job();
  b->dirty = true;
  return CGL_OK;
}

cgl_status cgl_batch_step(cgl_batch* b, uint32_t ticks) {
  if (!b) return CGL_INVALID_ARG;
  b->err.clear();
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "cudaSetDevice");
  if (b->jobs.empty() || ticks == 0) return CGL_OK;
  cgl_status st = prepare(b);
  if (st) return st;
  const size_t slots = b->jobs.size();
  uint32_t done = 0;
  while (done < ticks) {
    const uint32_t n = std::min(kTickChunk, ticks - done);
    if (b->params_pending) { BCU(cudaEventSynchronize(b->params_copied)); b->params_pending = false; }
    for (uint32_t t = 0; t < n; ++t)
      for (size_t g = 0; g < slots; ++g) b->h_ticks[(size_t)t * slots + g] = host_tick(b->jobs[g]);
    BCU(cudaMemcpyAsync(b->ticks.p, b->h_ticks, (size_t)n * slots * sizeof(BatchTick), cudaMemcpyHostToDevice,
                        b->stream));
    BCU(cudaEventRecord(b->params_copied, b->stream));
    b->params_pending = true;
    BCU(cudaMemsetAsync(b->tick_ctr.p, 0, 4, b->stream));
    for (uint32_t t = 0; t < n; ++t) BCU(cudaGraphLaunch(b->graph, b->stream));
    done += n;
  }
  return CGL_OK;
}

cgl_status cgl_batch_synchronize(cgl_batch* b) {
  if (!b) return CGL_INVALID_ARG;
  BCU(cudaStreamSynchronize(b->stream));
  return batch_device_error(b);
}

cgl_status cgl_batch_get_point_positions(cgl_batch* b, uint32_t id, float* out, uint64_t cap) {
  if (!b || id >= b->jobs.size() || !b->jobs[id].used) return CGL_INVALID_ARG;
  const Job& j = b->jobs[id];
  if (cap < 2 * j.n || !out) return bfail(b, CGL_INVALID_ARG, "output holds %llu floats, need %llu",
                                          (unsigned long long)cap, (unsigned long long)(2 * j.n));
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "cudaSetDevice");
  BCU(cudaMemcpyAsync(out, (float2*)b->pos.p + j.p_off, j.n * 8, cudaMemcpyDeviceToHost, b->stream));
  BCU(cudaStreamSynchronize(b->stream));
  return batch_device_error(b);
}

cgl_status cgl_batch_get_positions_many(cgl_batch* b, uint32_t count, const uint32_t* ids, float* const* outs,
                                        const uint64_t* capacity_floats) {
  if (!b || (count && (!ids || !outs || !capacity_floats))) return CGL_INVALID_ARG;
  b->err.clear();
  for (uint32_t k = 0; k < count; ++k) {
    if (ids[k] >= b->jobs.size() || !b->jobs[ids[k]].used) return bfail(b, CGL_INVALID_ARG, "job %u: no such job", ids[k]);
    const Job& j = b->jobs[ids[k]];
    if (!outs[k] || capacity_floats[k] < 2 * j.n)
      return bfail(b, CGL_INVALID_ARG, "job %u: output holds %llu floats, need %llu", ids[k],
                   (unsigned long long)capacity_floats[k], (unsigned long long)(2 * j.n));
  }
  if (count == 0) return CGL_OK;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, CGL_CUDA_ERROR, "cudaSetDevice");
  // the used point arena in one copy, then each job's range on host threads
  const uint64_t hwm = b->pts.hwm;
  if (hwm > b->stage_cap) {
    if (b->h_stage) cudaFreeHost(b->h_stage);
    b->h_stage = nullptr;
    b->stage_cap = 0;
    BCU(cudaMallocHost((void**)&b->h_stage, hwm * sizeof(float2)));
    b->stage_cap = hwm;
  }
  BCU(cudaMemcpyAsync(b->h_stage, b->pos.p, hwm * sizeof(float2), cudaMemcpyDeviceToHost, b->stream));
  BCU(cudaStreamSynchronize(b->stream));
  const unsigned nt = std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), count);
  std::atomic<uint32_t> next{0};
  auto worker = [&]() {
    for (uint32_t k; (k = next.fetch_add(1)) < count;) {
      const Job& j = b->jobs[ids[k]];
      std::memcpy(outs[k], b->h_stage + j.p_off, j.n * sizeof(float2));
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  return batch_device_error(b);
}

cgl_status cgl_batch_get_state(cgl_batch* b, uint32_t id, cgl_state* s) {
  if (!b || !s || id >= b->jobs.size() || !b->jobs[id].used) return CGL_INVALID_ARG;
  const Job& j = b->jobs[id];
  std::memset(s, 0, sizeof(*s));
  s->alpha = j.alpha;
  s->progress = j.progress;
  s->is_simulation_running = j.running && !(j.max_ticks && j.tick >= j.max_ticks) &&
                             !(j.stop_below_min && j.alpha < kAlphaMin);
  s->tick = j.tick;
  s->points_number = j.n;
  s->links_number = j.E;
  s->rng_draws = j.rng.ctr;
  return CGL_OK;
}

cgl_status cgl_batch_get_info(cgl_batch* b, cgl_batch_info* out) {
  if (!b || !out) return CGL_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  if (b->dirty) {   // the tables the next tick runs with (its kernel count)
    const cgl_status st = rebuild_tables(b);
    if (st) return st;
  }
  for (const Job& j : b->jobs) {
    if (!j.used) continue;
    out->jobs++;
    out->points += j.n;
    out->link_entries += j.m_in;
    if (j.running && !(j.max_ticks && j.tick >= j.max_ticks) && !(j.stop_below_min && j.alpha < kAlphaMin))
      out->running_jobs++;
  }
  out->point_arena = b->pts.cap;
  out->cell_arena = b->cells.cap;
  out->device_bytes = b->dev_bytes;
  refresh_view(b);
  out->kernels_per_tick = batch_kernels_per_tick(b->view);
  return CGL_OK;
}

}  // extern "C"
