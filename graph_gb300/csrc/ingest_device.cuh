// ingest_device.cuh — building blocks of the device-side link ingest
// (ingest_device.cu); the engine strings them together.  All run on one
// stream; sizes are 32-bit (points <= 2^24, links < 2^32).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace cgl {
namespace dingest {

// In-place exclusive scan of n words; tmp holds scan_temp_words(n) words.
size_t scan_temp_words(uint64_t n);
void scan_exclusive(uint32_t* d, uint32_t n, uint32_t* tmp, cudaStream_t st);

// Stable LSD radix sort of (keys, vals) by the low `bits` key bits, 8 per
// pass; tmp holds sort_temp_words(n) words.  key_bits(m) = bits of m.
size_t sort_temp_words(uint64_t n);
int key_bits(uint64_t max_key);
void sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int bits, uint32_t* tmp, cudaStream_t st);

// valid[i] = link i has two point indices; len_in[s]++, len_out[t]++ for those
// (valid, len_in and len_out zeroed by the caller).
void count_links(const float2* links, uint32_t E, uint32_t N, uint32_t* valid, uint32_t* len_in, uint32_t* len_out,
                 cudaStream_t st);
// pos = exclusive scan of valid (E + 1 words, trailing 0): the valid links in
// index order -> (source, link) and (target, link) pairs at pos[i].
void compact_links(const float2* links, uint32_t E, const uint32_t* pos, uint32_t* key_in, uint32_t* key_out,
                   uint32_t* val_in, uint32_t* val_out, cudaStream_t st);
// Entries of one direction from its row-sorted (row, link) pairs; entry `at`
// takes draws[at] (device memory, drawn on the host) or, when draws is null,
// counter draw draw_base + at of `seed`; neighbours are written as
// point_off + index (flags indexed by the graph's own point index).
void fill_csr(const uint32_t* rows, const uint32_t* lidx, uint32_t M, const float2* links, bool incoming,
              const uint32_t* len_in, const uint32_t* len_out, const float* strength, const uint8_t* flags,
              const float* draws, uint64_t seed, uint64_t draw_base, uint32_t point_off, uint4* ent, cudaStream_t st);
// stats[0] = longest list, stats[1] = lists longer than kHeavyDegree (stats zeroed by the caller)
void len_stats(const uint32_t* len, uint32_t N, uint32_t* stats, cudaStream_t st);
// key[p] = stats[0] - len[p], val[p] = p: sorted stably, the points by list length, longest first
void len_keys(const uint32_t* len, uint32_t N, const uint32_t* stats, uint32_t* key, uint32_t* val, cudaStream_t st);
// The many-body jitter of points [0, n) from the counter stream: draws base + 2t, base + 2t + 1.
void jitter(uint64_t seed, uint64_t base, uint32_t n, float2* out, cudaStream_t st);
// b[i] = a[i] + add
void copy_u32(const uint32_t* a, uint32_t* b, uint32_t n, cudaStream_t st, uint32_t add = 0);

}  // namespace dingest
}  // namespace cgl
