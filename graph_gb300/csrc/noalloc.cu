// noalloc.cu — the many-body grid pyramid for callers that cannot allocate
// device memory.
//
// Some hosts must not see a library call cudaMalloc: an application that owns
// the whole GPU memory budget through its own allocator (a browser GPU process,
// a renderer with a fixed arena), code recording a CUDA graph (cudaMalloc is
// illegal during stream capture), or a frame loop where the implicit
// synchronisation of cudaMalloc/cudaFree would stall.  cgl_levels_noalloc
// computes the same level cells as the engine's many-body pass (exact integer
// cell sums rounded once to f32, all levels) for positions the caller already
// holds on the device, and writes them to a caller buffer.  Its scratch — the
// integer sums of every level — is the file-scope array below, 8.4 MB, enough
// for the largest pyramid the engine builds (finest grid 512, 8 levels), held
// by every GPU that loads the library until the process exits.
//
// Every call shares that array and it keeps the last call's contents; the
// first kernel of each call clears what must start at zero.  Calls whose work
// overlaps on the GPU (different streams, or different host threads without
// ordering) race on the array.  The array's device address is looked up once
// per device and kept; a device reset (cudaDeviceReset) unloads the library's
// device code, after which that address is stale, so a process that resets a
// device must not call this entry point on that device again.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/cgl.h"
#include "common.cuh"
#include "ingest.h"

namespace cgl {
namespace {

constexpr int kNaLevelsMax = 8;                          // finest grid 512 = 4 << 7
constexpr uint32_t kNaCellsMax = 349520;                 // sum over l < 8 of (4 << l)^2
constexpr uint64_t kNaPointsMax = 1ull << 24;            // point indices exact in f32
constexpr int kNaBlock = 256;
constexpr int kNaMaxDevices = 64;

// Integer sums (x, y, count) of every cell of every level, level 0 first.
static __device__ __align__(256) long long g_levels_scratch[3 * (size_t)kNaCellsMax];

std::mutex g_setup_mutex;
void* g_scratch_addr[kNaMaxDevices] = {};

__global__ void k_na_clear(long long* acc, uint32_t words) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < words; k += gridDim.x * blockDim.x) acc[k] = 0;
}

__global__ void k_na_bin(const float2* __restrict__ xy, uint32_t n, float csf, int gf, FixedScale fx,
                         long long* __restrict__ fine) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 p = xy[i];
  if (isnan(p.x) || isnan(p.y)) return;   // absent points stay out of the grid (calculate-level.vert:33-40)
  const int cx = cell_index(p.x, csf, gf), cy = cell_index(p.y, csf, gf);
  long long* a = fine + 3 * (size_t)(cy * gf + cx);
  atomicAdd((unsigned long long*)&a[0], (unsigned long long)to_fixed(p.x, fx));
  atomicAdd((unsigned long long*)&a[1], (unsigned long long)to_fixed(p.y, fx));
  atomicAdd((unsigned long long*)&a[2], 1ull);
}

// Level l's records; below the finest level the sums come from the children.
__global__ void k_na_level(long long* acc, uint32_t off_l, uint32_t off_child, int G, bool finest, FixedScale fx,
                           float4* __restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (uint32_t)(G * G)) return;
  long long* a = acc + 3 * (size_t)(off_l + c);
  if (!finest) {
    const int x = (int)(c % (uint32_t)G), y = (int)(c / (uint32_t)G), Gc = 2 * G;
    long long sx = 0, sy = 0, sn = 0;
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const long long* ch = acc + 3 * (size_t)(off_child + (2 * y + dy) * Gc + 2 * x + dx);
        sx += ch[0]; sy += ch[1]; sn += ch[2];
      }
    a[0] = sx; a[1] = sy; a[2] = sn;
  }
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if (a[2] > 0) {
    const float cf = (float)a[2];
    r.x = __fdiv_rn(from_fixed(a[0], fx), cf);
    r.y = __fdiv_rn(from_fixed(a[1], fx), cf);
    r.z = cf;
  }
  out[off_l + c] = r;
}

cgl_status na_fail(char* err, size_t len, cgl_status st, const char* fmt, ...) {
  if (err && len) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, len, fmt, ap);
    va_end(ap);
  }
  return st;
}

}  // namespace
}  // namespace cgl

using namespace cgl;

extern "C" cgl_status cgl_levels_noalloc(const float* d_xy, uint64_t n_points, double space_size, float* d_cells,
                                         uint64_t cells_capacity_floats, void* cuda_stream, char* err,
                                         size_t err_len) {
  if (err && err_len) err[0] = '\0';
  if (n_points == 0) return na_fail(err, err_len, CGL_INVALID_ARG, "no points");
  if (n_points > kNaPointsMax)
    return na_fail(err, err_len, CGL_INVALID_ARG, "%llu points exceed the maximum of %llu (2^24)",
                   (unsigned long long)n_points, (unsigned long long)kNaPointsMax);
  if (!d_xy || !d_cells) return na_fail(err, err_len, CGL_INVALID_ARG, "null device pointer");
  if (!(space_size >= 2) || !std::isfinite(space_size))
    return na_fail(err, err_len, CGL_INVALID_ARG, "space size %g must be a finite number >= 2", space_size);
  // grid sizes as the engine's (ForceManyBody.createLevels, ForceManyBody/index.ts:646-667)
  const ingest::Grid grid = ingest::grid_for(n_points);
  const int gf = grid.gf;
  const int L = grid.levels;
  uint32_t off[kNaLevelsMax + 1];
  off[0] = 0;
  for (int l = 0; l < L; ++l) off[l + 1] = off[l] + (uint32_t)((4 << l) * (4 << l));
  const uint32_t cells = off[L];
  if (L > kNaLevelsMax || cells > kNaCellsMax)
    return na_fail(err, err_len, CGL_INVALID_ARG, "pyramid of %u cells exceeds the scratch of %u cells", cells,
                   kNaCellsMax);
  if (cells_capacity_floats < 4ull * cells)
    return na_fail(err, err_len, CGL_INVALID_ARG, "output holds %llu floats, %u levels need %llu",
                   (unsigned long long)cells_capacity_floats, L, 4ull * cells);
  // exact-sum scale as the engine's
  const FixedScale fx = ingest::fixed_for(n_points, space_size, nullptr);

  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return na_fail(err, err_len, CGL_CUDA_ERROR, "cudaGetDevice: %s", cudaGetErrorString(ce));
  if (dev < 0 || dev >= kNaMaxDevices) return na_fail(err, err_len, CGL_INVALID_ARG, "device %d not supported", dev);
  long long* acc = nullptr;
  {
    // One-time set-up per device, with that device current: the device
    // address of the scratch array (its host-side name is not a device address).
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      ce = cudaGetSymbolAddress(&p, g_levels_scratch);
      if (ce != cudaSuccess)
        return na_fail(err, err_len, CGL_CUDA_ERROR, "cudaGetSymbolAddress: %s", cudaGetErrorString(ce));
      g_scratch_addr[dev] = p;
    }
    acc = (long long*)g_scratch_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)cuda_stream;
  const uint32_t fine_words = 3u * (uint32_t)(gf * gf);
  long long* fine = acc + 3 * (size_t)off[L - 1];
  k_na_clear<<<(fine_words + kNaBlock - 1) / kNaBlock, kNaBlock, 0, st>>>(fine, fine_words);
  const uint32_t n = (uint32_t)n_points;
  k_na_bin<<<(n + kNaBlock - 1) / kNaBlock, kNaBlock, 0, st>>>((const float2*)d_xy, n,
                                                                (float)(space_size / gf), gf, fx, fine);
  for (int l = L - 1; l >= 0; --l) {
    const int G = 4 << l;
    const uint32_t nc = (uint32_t)(G * G);
    k_na_level<<<(nc + kNaBlock - 1) / kNaBlock, kNaBlock, 0, st>>>(acc, off[l], l + 1 < L ? off[l + 1] : 0, G,
                                                                    l == L - 1, fx, (float4*)d_cells);
  }
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return na_fail(err, err_len, CGL_CUDA_ERROR, "launch: %s", cudaGetErrorString(ce));
  return CGL_OK;
}
