// Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), restated for the CPU oracle.
//
// TEST INFRASTRUCTURE: this file belongs to the CPU oracle.  The CUDA library has its own,
// independent implementation; both are pinned to the published known-answer vectors by
// tests/test_oracle_kat.py so that a shared mistake cannot hide.
//
// The reference draws from rand 0.8.8 StdRng (ChaCha12, Cargo.lock:589/914).  That stream
// cannot be reproduced here (no Rust toolchain), so the oracle and the device both draw from
// Philox keyed by (seed, stream) with a counter that names the draw.  Uniforms carry 24 bits so
// that the very same value is exactly representable in float and double.
#pragma once
#include <cstdint>

namespace fgo {

struct Philox4 {
  uint32_t v[4];
};

inline void philox_mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = static_cast<uint64_t>(a) * static_cast<uint64_t>(b);
  hi = static_cast<uint32_t>(p >> 32);
  lo = static_cast<uint32_t>(p);
}

// Ten rounds of the Philox-4x32 bijection; key schedule bumps by the Weyl constants.
inline Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                             uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3;
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(M0, x0, hi0, lo0);
    philox_mulhilo(M1, x2, hi1, lo1);
    const uint32_t n0 = hi1 ^ x1 ^ k0;
    const uint32_t n1 = lo1;
    const uint32_t n2 = hi0 ^ x3 ^ k1;
    const uint32_t n3 = lo0;
    x0 = n0; x1 = n1; x2 = n2; x3 = n3;
    k0 += W0;
    k1 += W1;
  }
  return Philox4{{x0, x1, x2, x3}};
}

// 24-bit uniform in [0, 1): exactly representable in float and double.
inline double u24(uint32_t x) { return static_cast<double>(x >> 8) * (1.0 / 16777216.0); }

// Stream tags: the fourth counter word names which part of the path a draw belongs to.
enum : uint32_t {
  TAG_SYNTH = 0x53594E00u,   // sequential Bridson stream (oracle synthesis)
  TAG_EMIT = 0x454D0000u,    // photon emission
  TAG_BOUNCE = 0x424F0000u,  // free path, Henyey-Greenstein, roulette
  TAG_AH = 0x41480000u,      // anti-halation reflection
  TAG_HIT = 0x48490000u,     // per-hit Bernoulli rounding
  TAG_SCAN = 0x53430000u,    // scanner sub-pixel jitter
};

// Sequential stream over a Philox key: draws counters (n, 0, 0, tag) in order and hands out
// the four words of each block one at a time.
struct PhiloxStream {
  uint32_t k0, k1, tag;
  uint64_t block = 0;
  Philox4 cur{};
  int used = 4;
  PhiloxStream(uint64_t seed, uint32_t tag_)
      : k0(static_cast<uint32_t>(seed)), k1(static_cast<uint32_t>(seed >> 32)), tag(tag_) {}
  uint32_t next_u32() {
    if (used == 4) {
      cur = philox4x32_10(static_cast<uint32_t>(block), static_cast<uint32_t>(block >> 32), 0u,
                          tag, k0, k1);
      ++block;
      used = 0;
    }
    return cur.v[used++];
  }
  double uniform() { return u24(next_u32()); }
  // Integer in [0, n): high word of a 32x32 multiply (Lemire's map without rejection).
  uint64_t below(uint64_t n) { return (static_cast<uint64_t>(next_u32()) * n) >> 32; }
};

}  // namespace fgo
