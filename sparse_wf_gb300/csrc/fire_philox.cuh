// fire_philox.cuh -- Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3", SC'11): the
// counter-based generator of the Metropolis proposals and of the pseudopotential quadrature rotations.
#pragma once
#include <cstdint>

namespace fire {

struct Philox {
  uint32_t c[4];
};

__device__ __forceinline__ void philox_round(uint32_t (&ctr)[4], uint32_t (&key)[2]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t hi0 = __umulhi(M0, ctr[0]), lo0 = M0 * ctr[0];
  const uint32_t hi1 = __umulhi(M1, ctr[2]), lo1 = M1 * ctr[2];
  const uint32_t n0 = hi1 ^ ctr[1] ^ key[0], n1 = lo1, n2 = hi0 ^ ctr[3] ^ key[1], n3 = lo0;
  ctr[0] = n0; ctr[1] = n1; ctr[2] = n2; ctr[3] = n3;
}

__device__ __forceinline__ void philox10(uint32_t (&ctr)[4], uint64_t seed) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(ctr, key);
    key[0] += 0x9E3779B9u;
    key[1] += 0xBB67AE85u;
  }
}

__device__ __forceinline__ double u01(uint32_t x) { return ((double)(x >> 8) + 0.5) * (1.0 / 16777216.0); }

}  // namespace fire
