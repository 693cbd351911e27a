// The warp-cell slot selection (graph_gb300/csrc/warp_cells.cuh) against the
// per-lane top-8 lists it replaced, on cells built to reach every path:
// cells of up to 128 points (keys in registers), heavier cells whose
// candidates under the hash threshold give the slots, and heavier cells where
// they cannot (fewer than 8 distinct hashes under the threshold, or more
// candidates than the buffer holds), which fall back to the lists.  Cells mix
// in points whose peel hashes tie.  Both variants run on copies of the same
// segments; the moved segments, sums and slot counts must be equal bit for bit.
// Prints "cells=<n> ties=<t> fallbacks=<f> mismatches=<m>" per key offset; exit status
// 0 when it ran.
#include <algorithm>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "../../graph_gb300/csrc/warp_cells.cuh"

struct View {
  uint32_t* sorted_idx;
  float2* sorted_pos;
  uint32_t* cell_start;
  long long* big_sx;
  long long* big_sy;
  uint32_t* big_ns;
  uint32_t* inv = nullptr;   // no sorted-position map here
};

constexpr uint32_t kSeed = 0x2545F491u;

__global__ void hash_all(uint32_t* out, uint32_t m) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = __float_as_uint(cgl::peel_hash(i, kSeed));
}

__global__ void run_new(View v, cgl::FixedScale fx, uint32_t koff) {
  __shared__ uint32_t buf[3][cgl::kCandidates];
  cgl::warp_cell(v, fx, kSeed, koff, blockIdx.x, buf);
}

__global__ void run_lists(View v, cgl::FixedScale fx, uint32_t koff) {
  cgl::warp_cell_lists(v, fx, kSeed, koff, blockIdx.x, v.cell_start[blockIdx.x], v.cell_start[blockIdx.x + 1]);
}

static float hash_of(const std::vector<uint32_t>& h, uint32_t i) {
  float f;
  std::memcpy(&f, &h[i], 4);
  return f;
}

int main() {
  const uint32_t M = 1u << 22;
  uint32_t* dh;
  if (cudaMalloc(&dh, M * 4) != cudaSuccess) return 1;
  hash_all<<<M / 256, 256>>>(dh, M);
  std::vector<uint32_t> h(M);
  if (cudaMemcpy(h.data(), dh, M * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  cudaFree(dh);

  // groups of indices sharing one hash
  std::map<uint32_t, std::vector<uint32_t>> by_hash;
  for (uint32_t i = 0; i < M; ++i) by_hash[h[i]].push_back(i);
  std::vector<std::vector<uint32_t>> ties2, ties4;
  for (auto& kv : by_hash) {
    if (kv.second.size() >= 4) ties4.push_back(kv.second);
    else if (kv.second.size() >= 2) ties2.push_back(kv.second);
  }
  std::mt19937_64 rng(7);
  std::shuffle(ties2.begin(), ties2.end(), rng);
  std::shuffle(ties4.begin(), ties4.end(), rng);
  std::vector<char> used(M, 0);
  auto take = [&](std::vector<uint32_t>& cell, uint32_t i) {
    if (!used[i]) { used[i] = 1; cell.push_back(i); return true; }
    return false;
  };
  // random unused indices whose hash lies in [lo, hi)
  auto fill = [&](std::vector<uint32_t>& cell, size_t count, float lo, float hi) {
    size_t got = 0;
    while (got < count) {
      const uint32_t i = (uint32_t)(rng() % M);
      const float f = hash_of(h, i);
      if (f >= lo && f < hi && take(cell, i)) ++got;
    }
  };
  // a tie group whose hash lies in [lo, hi), all members
  size_t t2 = 0, t4 = 0;
  int groups = 0;   // tie groups placed
  auto tie = [&](std::vector<uint32_t>& cell, bool four, float lo, float hi) {
    auto& src = four ? ties4 : ties2;
    size_t& at = four ? t4 : t2;
    for (; at < src.size(); ++at) {
      const float f = hash_of(h, src[at][0]);
      bool free_all = true;
      for (uint32_t i : src[at]) free_all = free_all && !used[i];
      if (f >= lo && f < hi && free_all) {
        for (uint32_t i : src[at]) take(cell, i);
        ++at;
        ++groups;
        return;
      }
    }
  };
  auto below = [](size_t n) { return 48.0f / (float)n; };

  std::vector<std::vector<uint32_t>> cells;
  int fallbacks = 0;
  for (size_t n : {17, 31, 64, 100, 128}) {   // keys in registers
    std::vector<uint32_t> c;
    fill(c, n, 0.f, 1.f);
    cells.push_back(c);
  }
  {   // ties, few distinct hashes: 6 groups of at least 4 (6 slots)
    std::vector<uint32_t> c;
    for (int g = 0; g < 6; ++g) tie(c, true, 0.f, 1.f);
    cells.push_back(c);
  }
  {   // ties among a small cell's smallest hashes
    std::vector<uint32_t> c;
    for (int g = 0; g < 10; ++g) tie(c, false, 0.f, 0.05f);
    fill(c, 100 - c.size(), 0.f, 1.f);
    cells.push_back(c);
  }
  for (size_t n : {129, 300, 1000, 2048}) {   // candidates under the threshold
    std::vector<uint32_t> c;
    fill(c, n, 0.f, 1.f);
    cells.push_back(c);
  }
  {   // ties under the threshold
    std::vector<uint32_t> c;
    for (int g = 0; g < 12; ++g) tie(c, false, 0.f, below(600));
    fill(c, 600 - c.size(), 0.f, 1.f);
    cells.push_back(c);
  }
  {   // exactly 8 distinct hashes under the threshold, three of them tied
    std::vector<uint32_t> c;
    for (int g = 0; g < 3; ++g) tie(c, false, 0.f, below(500));
    fill(c, 5, 0.f, below(500));
    fill(c, 500 - c.size(), below(500), 1.f);
    cells.push_back(c);
  }
  {   // 7 distinct under the threshold: falls back
    std::vector<uint32_t> c;
    for (int g = 0; g < 2; ++g) tie(c, false, 0.f, below(500));
    fill(c, 5, 0.f, below(500));
    fill(c, 500 - c.size(), below(500), 1.f);
    cells.push_back(c);
    ++fallbacks;
  }
  {   // 5 under the threshold in a 300-point cell: falls back
    std::vector<uint32_t> c;
    fill(c, 5, 0.f, below(300));
    fill(c, 295, below(300), 1.f);
    cells.push_back(c);
    ++fallbacks;
  }
  {   // 150 candidates for a buffer of 128: falls back
    std::vector<uint32_t> c;
    fill(c, 150, 0.f, below(200));
    fill(c, 50, below(200), 1.f);
    cells.push_back(c);
    ++fallbacks;
  }

  // segments: each cell's indices shuffled, random positions
  std::vector<uint32_t> start(1, 0), idx;
  std::vector<float2> pos;
  std::uniform_real_distribution<float> coord(0.f, 8192.f);
  for (auto& c : cells) {
    std::shuffle(c.begin(), c.end(), rng);
    for (uint32_t i : c) { idx.push_back(i); pos.push_back(make_float2(coord(rng), coord(rng))); }
    start.push_back((uint32_t)idx.size());
  }
  const uint32_t nc = (uint32_t)cells.size(), np = (uint32_t)idx.size();
  const cgl::FixedScale fx{1048576.f, 65536.f, 1.f / 65536.f};
  for (uint32_t koff : {0u, 12345u}) {
    std::vector<uint32_t> sidx(idx);
    for (auto& i : sidx) i += koff;
    View v[2];
    for (int k = 0; k < 2; ++k) {
      if (cudaMalloc(&v[k].sorted_idx, np * 4) || cudaMalloc(&v[k].sorted_pos, np * 8) ||
          cudaMalloc(&v[k].cell_start, (nc + 1) * 4) || cudaMalloc(&v[k].big_sx, nc * 8) ||
          cudaMalloc(&v[k].big_sy, nc * 8) || cudaMalloc(&v[k].big_ns, nc * 4))
        return 1;
      cudaMemcpy(v[k].sorted_idx, sidx.data(), np * 4, cudaMemcpyHostToDevice);
      cudaMemcpy(v[k].sorted_pos, pos.data(), np * 8, cudaMemcpyHostToDevice);
      cudaMemcpy(v[k].cell_start, start.data(), (nc + 1) * 4, cudaMemcpyHostToDevice);
    }
    run_new<<<nc, 32>>>(v[0], fx, koff);
    run_lists<<<nc, 32>>>(v[1], fx, koff);
    if (cudaDeviceSynchronize() != cudaSuccess) return 1;
    int bad = 0;
    std::vector<uint32_t> i0(np), i1(np), n0(nc), n1(nc);
    std::vector<float2> p0(np), p1(np);
    std::vector<long long> x0(nc), x1(nc), y0(nc), y1(nc);
    cudaMemcpy(i0.data(), v[0].sorted_idx, np * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(i1.data(), v[1].sorted_idx, np * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(p0.data(), v[0].sorted_pos, np * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(p1.data(), v[1].sorted_pos, np * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(n0.data(), v[0].big_ns, nc * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(n1.data(), v[1].big_ns, nc * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(x0.data(), v[0].big_sx, nc * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(x1.data(), v[1].big_sx, nc * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(y0.data(), v[0].big_sy, nc * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(y1.data(), v[1].big_sy, nc * 8, cudaMemcpyDeviceToHost);
    for (uint32_t c = 0; c < nc; ++c) {
      bool ok = n0[c] == n1[c] && x0[c] == x1[c] && y0[c] == y1[c];
      // the slots (head of the segment) in order; the rest as a multiset
      for (uint32_t q = 0; ok && q < n0[c]; ++q) {
        const uint32_t j = start[c] + q;
        ok = i0[j] == i1[j] && std::memcmp(&p0[j], &p1[j], 8) == 0;
      }
      std::vector<uint32_t> r0(i0.begin() + start[c], i0.begin() + start[c + 1]);
      std::vector<uint32_t> r1(i1.begin() + start[c], i1.begin() + start[c + 1]);
      std::sort(r0.begin(), r0.end());
      std::sort(r1.begin(), r1.end());
      ok = ok && r0 == r1;
      for (uint32_t j = start[c]; ok && j < start[c + 1]; ++j)   // each point keeps its position
        ok = std::memcmp(&p0[j], &pos[std::find(sidx.begin(), sidx.end(), i0[j]) - sidx.begin()], 8) == 0;
      if (!ok) ++bad;
    }
    printf("koff=%u cells=%u ties=%d fallbacks=%d mismatches=%d\n", koff, nc, groups, fallbacks, bad);
    for (int k = 0; k < 2; ++k) {
      cudaFree(v[k].sorted_idx); cudaFree(v[k].sorted_pos); cudaFree(v[k].cell_start);
      cudaFree(v[k].big_sx); cudaFree(v[k].big_sy); cudaFree(v[k].big_ns);
    }
  }
  return 0;
}
