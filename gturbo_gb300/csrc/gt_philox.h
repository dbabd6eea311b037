// gt_philox.h -- Philox4x64-10 counter-based generator (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), host and device.
//
// Each round multiplies counter words 0 and 2 by M0, M1 (128-bit products), swaps and mixes
// them with words 1, 3 and the key; the key advances by the Weyl constants W0, W1 between
// rounds. Ten rounds. This is the generator numpy exposes as numpy.random.Philox.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define GT_HD __host__ __device__ __forceinline__
#else
#define GT_HD inline
#endif

namespace gt {

struct Philox4 {
  uint64_t v[4];
};

GT_HD uint64_t mulhilo64(uint64_t a, uint64_t b, uint64_t* hi) {
#ifdef __CUDA_ARCH__
  *hi = __umul64hi(a, b);
  return a * b;
#else
  const unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
  *hi = (uint64_t)(p >> 64);
  return (uint64_t)p;
#endif
}

GT_HD Philox4 philox4x64_10(Philox4 ctr, uint64_t k0, uint64_t k1) {
  const uint64_t M0 = 0xD2E7470EE14C6C93ull, M1 = 0xCA5A826395121157ull;
  const uint64_t W0 = 0x9E3779B97F4A7C15ull, W1 = 0xBB67AE8584CAA73Bull;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += W0;
      k1 += W1;
    }
    uint64_t hi0, hi1;
    const uint64_t lo0 = mulhilo64(M0, ctr.v[0], &hi0);
    const uint64_t lo1 = mulhilo64(M1, ctr.v[2], &hi1);
    Philox4 o;
    o.v[0] = hi1 ^ ctr.v[1] ^ k0;
    o.v[1] = lo1;
    o.v[2] = hi0 ^ ctr.v[3] ^ k1;
    o.v[3] = lo0;
    ctr = o;
  }
  return ctr;
}

// Uniform double in [0, 1) from the top 53 bits of a 64-bit draw.
GT_HD double u01_53(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

// Phase of forced mode `mode` at step `step` of the stream `key`: counter (step, mode, 0, 0).
GT_HD double philox_phase(uint64_t key, uint64_t step, uint64_t mode) {
  Philox4 c;
  c.v[0] = step;
  c.v[1] = mode;
  c.v[2] = 0;
  c.v[3] = 0;
  const Philox4 o = philox4x64_10(c, key, 0);
  return 2.0 * 3.14159265358979323846 * u01_53(o.v[0]);
}

}  // namespace gt
