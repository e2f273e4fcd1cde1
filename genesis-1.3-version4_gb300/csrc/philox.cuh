// Counter-based random numbers for the incoherent-radiation energy spread: Philox-4x32-10
// (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011),
// ten rounds of two 32x32->64-bit products with the published multipliers and Weyl key
// increments. A draw is a pure function of (seed, step counter, slice, beamlet), so every
// particle of a beamlet gets the same number without any state or ordering between
// threads.
#pragma once

#include <cstdint>

namespace g4 {

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) {
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    const unsigned lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const unsigned lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

// uniform in (0, 1): the first 32 bits of the draw of (step, slice, beamlet)
__device__ __forceinline__ double isr_uniform(unsigned seed, unsigned long long step, int is, int beamlet) {
  const uint4 r = philox4x32_10(make_uint4((unsigned)beamlet, (unsigned)is, (unsigned)step, (unsigned)(step >> 32)),
                                make_uint2(seed, 0x5EEDu));
  return ((double)r.x + 0.5) * (1.0 / 4294967296.0);
}

}  // namespace g4
