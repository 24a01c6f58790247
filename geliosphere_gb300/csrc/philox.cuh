// Counter-based random numbers held in registers.
//
// Philox4x32-10 as defined by Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3" (SC'11): a 4x32-bit counter and a 2x32-bit key,
// ten rounds of two 32x32->64 multiplies, the key bumped by the Weyl constants
// between rounds.  Each trajectory owns the counter space
// (step, stream, particle_lo, particle_hi) under the key (seed, seed_hi ^ sim),
// so a particle's random numbers do not depend on which lane, warp or launch
// integrates it.  This replaces the 48-byte cuRAND XORWOW state that the
// reference keeps in global and shared memory (CosmicUtils.cu:47-51,
// GeliosphereModel.cu:78-80,391).
#pragma once
#include <cstdint>

namespace gelio {

struct Philox4 {
  uint32_t x, y, z, w;
};

// One widening multiply gives both halves (a single mul.wide.u32 instead of
// a mul.lo and a mul.hi).
__host__ __device__ __forceinline__ void philox_mulhilo(uint32_t a, uint32_t b,
                                                        uint32_t &hi, uint32_t &lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
}

__host__ __device__ __forceinline__ Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
  constexpr uint32_t kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;
  constexpr uint32_t kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(kM0, c.x, hi0, lo0);
    philox_mulhilo(kM1, c.z, hi1, lo1);
    Philox4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += kW0;
    k1 += kW1;
  }
  return c;
}

// 23-bit uniform in (0, 1): (x >> 9) * 2^-23 + 2^-24 = (2 (x >> 9) + 1) 2^-24,
// an odd multiple of 2^-24 below 1, so exactly representable in FP32 (and
// identical in the FP64 oracle); never 0, so log() is finite.  Built from the
// bits: 1 + m 2^-23 (exponent of 1, mantissa m) minus (1 - 2^-24); the
// difference is exact (Sterbenz), so no conversion instruction is needed.
__device__ __forceinline__ float u32_to_unit(uint32_t x) {
  return __uint_as_float(0x3f800000u | (x >> 9)) - 0.99999994f;
}

// Box-Muller: z0 = sqrt(-2 ln u1) cos(2 pi u2), z1 = sqrt(-2 ln u1) sin(2 pi u2).
__device__ __forceinline__ void box_muller(float u1, float u2, float &z0, float &z1) {
  const float rad = sqrtf(-2.0f * __logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  z0 = rad * c;
  z1 = rad * s;
}

__device__ __forceinline__ void box_muller(double u1, double u2, double &z0, double &z1) {
  const double rad = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  z0 = rad * c;
  z1 = rad * s;
}

// Four standard normals for (key, step counter) of one trajectory:
// pair A from (x, y), pair B from (z, w).
template <class R>
__device__ __forceinline__ void normals4(uint32_t k0, uint32_t k1, uint32_t step,
                                         uint32_t stream, uint64_t particle, R z[4]) {
  Philox4 c;
  c.x = step;
  c.y = stream;
  c.z = (uint32_t)particle;
  c.w = (uint32_t)(particle >> 32);
  const Philox4 o = philox4x32_10(c, k0, k1);
  box_muller((R)u32_to_unit(o.x), (R)u32_to_unit(o.y), z[0], z[1]);
  box_muller((R)u32_to_unit(o.z), (R)u32_to_unit(o.w), z[2], z[3]);
}

// Stream ids of the counter's second word.
constexpr uint32_t kStreamSde = 0u;
constexpr uint32_t kStreamInjection = 1u;

}  // namespace gelio
