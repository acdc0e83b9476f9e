// fe_rng.cuh -- counter-based random numbers for device-side Monte Carlo and
// replica-exchange decisions.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): a 128-bit counter and a 64-bit key give four
// 32-bit words after ten rounds of two 32x32->64 multiplies, with a Weyl
// increment of the key between rounds.  Being a pure function of
// (counter, key), the same draw is reproduced on the host, so every
// acceptance decision can be checked against a CPU restatement.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define FE_HD __host__ __device__ __forceinline__
#else
#define FE_HD static inline
#endif

namespace fe {

struct Philox4 {
  uint32_t v[4];
};

FE_HD void philox_mulhilo(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

// Philox4x32 with 10 rounds.  Multipliers and Weyl constants as published.
FE_HD Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(0xD2511F53u, c.v[0], &hi0, &lo0);
    philox_mulhilo(0xCD9E8D57u, c.v[2], &hi1, &lo1);
    Philox4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
  }
  return c;
}

// Uniform double in [0, 1) with 53 random bits from words 0 and 1.
FE_HD double philox_uniform(Philox4 r) {
  uint64_t w = ((uint64_t)r.v[0] << 32) | r.v[1];
  return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

// The draw for (stream tag, event, lane) under a 64-bit seed.
FE_HD double fe_uniform(uint64_t seed, uint32_t tag, uint64_t event, uint32_t lane) {
  Philox4 c;
  c.v[0] = lane;
  c.v[1] = (uint32_t)event;
  c.v[2] = (uint32_t)(event >> 32);
  c.v[3] = tag;
  return philox_uniform(philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32)));
}

// Stream tags keep the draws of different decisions independent.
enum : uint32_t { kRngTagExchange = 0x52455831u /* "REX1" */, kRngTagMC = 0x4D433031u };

}  // namespace fe
