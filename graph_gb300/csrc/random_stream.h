// random_stream.h — the reference's random stream, on the host.
//
// cosmos.gl draws every random number through Store.getRandomFloat
// (Store/index.ts:196-202): `random.float(min, max)` of a `Random` that
// Store.addRandomSeed replaced by `random.clone(randomSeed)` (src/index.ts:452).
// Those come from two npm packages that the reference pins but does not vendor
// (package-lock.json:8264-8274, 8687-8690):
//  * random@4.1.0: clone(seed) wraps seedrandom seeded with the seed's string
//    form (`seed + ''`), and float(min, max) is `next() * (max - min) + min`
//    in double precision, next() being one seedrandom output;
//  * seedrandom@3.0.5 (its default generator, ARC4): the seed string's UTF-16
//    code units are mixed into a key of at most 256 bytes (mixkey: key[j & 255]
//    = 255 & ((smear ^= key[j & 255] * 19) + code[j]), smear starting at 0 and
//    an unset key byte counting as 0); RC4's key schedule runs on that key (an
//    empty key is [0]) and the first 256 output bytes are dropped (RC4-drop[256]);
//    each output double takes 6 bytes as a 48-bit numerator n over 2^48, then
//    appends bytes (n = (n + x) * 256, x the next byte) while n < 2^52, shifts
//    n, the denominator and x right until n < 2^53, and returns (n + x) / d.
// Both are restated here from their published algorithms; the restatement
// reproduces seedrandom's README known answers (seed 'hello.': 0.9282578795792454,
// 0.3752569768646784, then quick() 0.7316977467853576 and int32() 1966374204).
//
// The stream is sequential (each byte permutes the generator's state), so the
// engines draw on the host and upload what the kernels need.  The bulk fills
// below keep the generator's state in locals.  seedrandom's double is, exactly,
// the integer M of the first 6 + k bytes (k >= 1 the fewest with M >= 2^52)
// cut to its top 53 bits and scaled by 2^-(48 + 8k): its loop appends bytes to
// n and shifts n, x and d right together, so (n + x) / d is M with the bits
// below the top 53 dropped; that is computed here with one count of leading
// zeros, in exact integer and power-of-two arithmetic.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace cgl {

class RandomStream {
 public:
  // seedrandom(text): text as UTF-16 code units (String.prototype.charCodeAt).
  void seed_units(const uint16_t* units, size_t n) {
    uint8_t key[256];
    bool set[256] = {};
    uint32_t smear = 0;
    for (size_t j = 0; j < n; ++j) {
      const size_t k = j & 255;
      smear ^= set[k] ? (uint32_t)key[k] * 19u : 0u;
      key[k] = (uint8_t)(smear + units[j]);
      set[k] = true;
    }
    size_t keylen = n < 256 ? n : 256;
    if (keylen == 0) { key[0] = 0; keylen = 1; }
    for (int i = 0; i < 256; ++i) S_[i] = (uint32_t)i;
    uint32_t j = 0;
    for (int i = 0; i < 256; ++i) {
      const uint32_t t = S_[i];
      j = (j + key[i % keylen] + t) & 255u;
      S_[i] = S_[j];
      S_[j] = t;
    }
    i_ = 0;
    j_ = 0;
    for (int k = 0; k < 256; ++k) (void)byte();   // RC4-drop[256]
    draws_ = 0;
  }

  // seedrandom(text) for UTF-8 text (converted to UTF-16 code units; invalid
  // sequences become U+FFFD as in a JavaScript string built from them).
  void seed_utf8(const char* s) {
    std::vector<uint16_t> u;
    const unsigned char* p = (const unsigned char*)s;
    while (p && *p) {
      uint32_t c = *p, need = 0;
      if (c < 0x80) { ++p; u.push_back((uint16_t)c); continue; }
      if ((c & 0xE0) == 0xC0) { need = 1; c &= 0x1F; }
      else if ((c & 0xF0) == 0xE0) { need = 2; c &= 0x0F; }
      else if ((c & 0xF8) == 0xF0) { need = 3; c &= 0x07; }
      else { ++p; u.push_back(0xFFFD); continue; }
      ++p;
      bool ok = true;
      for (uint32_t k = 0; k < need; ++k) {
        if ((*p & 0xC0) != 0x80) { ok = false; break; }
        c = (c << 6) | (*p & 0x3F);
        ++p;
      }
      if (!ok || c > 0x10FFFF || (c >= 0xD800 && c < 0xE000)) { u.push_back(0xFFFD); continue; }
      if (c >= 0x10000) {
        c -= 0x10000;
        u.push_back((uint16_t)(0xD800 + (c >> 10)));
        u.push_back((uint16_t)(0xDC00 + (c & 0x3FF)));
      } else {
        u.push_back((uint16_t)c);
      }
    }
    seed_units(u.data(), u.size());
  }

  // seedrandom's double in [0, 1) (its prng()).
  double next() {
    uint32_t i = i_, j = j_;
    const double u = unit(S_, i, j);
    i_ = i;
    j_ = j;
    ++draws_;
    return u;
  }
  // random's float(min, max).
  double uniform(double mn, double mx) { return next() * (mx - mn) + mn; }

  // out[k] = f32(float(0, 1)) for k < n (ForceLink/index.ts:76).
  void fill_unit_f32(float* out, uint64_t n) {
    uint32_t i = i_, j = j_;
    for (uint64_t k = 0; k < n; ++k) out[k] = (float)unit(S_, i, j);
    i_ = i;
    j_ = j;
    draws_ += n;
  }
  // The many-body jitter (ForceManyBody/index.ts:133-138): two draws per texel
  // of `texels`, f32(float(-1, 1) * 0.00001); the first `keep` texels are
  // written as (x, y) pairs.
  void fill_jitter(float* out_xy, uint64_t keep, uint64_t texels) {
    uint32_t i = i_, j = j_;
    for (uint64_t t = 0; t < texels; ++t) {
      const double ux = unit(S_, i, j);
      const double uy = unit(S_, i, j);
      if (t < keep) {
        out_xy[2 * t] = (float)((ux * 2.0 + -1.0) * 0.00001);
        out_xy[2 * t + 1] = (float)((uy * 2.0 + -1.0) * 0.00001);
      }
    }
    i_ = i;
    j_ = j;
    draws_ += 2 * texels;
  }

  uint64_t draws() const { return draws_; }

 private:
  uint8_t byte() {
    uint32_t i = i_, j = j_;
    const uint8_t b = (uint8_t)step(S_, i, j);
    i_ = i;
    j_ = j;
    return b;
  }
  // RC4's output step; the state is kept in 32-bit words (faster here than bytes).
  static inline uint32_t step(uint32_t* __restrict S, uint32_t& i, uint32_t& j) {
    i = (i + 1) & 255u;
    const uint32_t t = S[i];
    j = (j + t) & 255u;
    const uint32_t sj = S[j];
    S[i] = sj;
    S[j] = t;
    return S[(sj + t) & 255u];
  }
  static inline double unit(uint32_t* S, uint32_t& i, uint32_t& j) {
    uint64_t m = 0;
    for (int k = 0; k < 7; ++k) m = (m << 8) | step(S, i, j);
    int e = 56;   // the value is m / 2^e before the cut to 53 bits
    while ((m >> 8) < (1ull << 44)) {   // seedrandom's loop runs again: one more byte
      m = (m << 8) | step(S, i, j);
      e += 8;
    }
    // here 2^52 <= m < 2^60: keep the top 53 bits (exact in a double)
    const int h = 11 - __builtin_clzll(m);   // bit length - 53
    double v = (double)(m >> h);
    e -= h;
    while (e > 60) { v *= 0x1.0p-60; e -= 60; }
    return v * (1.0 / (double)(1ull << e));
  }

  uint32_t S_[256] = {};
  uint32_t i_ = 0, j_ = 0;
  uint64_t draws_ = 0;
};

// JavaScript's String(n) for an integer-valued seed below 2^53 (decimal digits).
inline std::string seed_decimal(uint64_t v) { return std::to_string(v); }

}  // namespace cgl
