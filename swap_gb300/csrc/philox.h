// philox.h -- Philox4x32-10 counter-based generator (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), usable on the
// host and the device.  A particle load is a pure function of
// (seed, stream, particle id, draw), so any thread can make any particle.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define SWAP_HD __host__ __device__ __forceinline__
#else
#define SWAP_HD inline
#endif

namespace swapk {

struct u32x4 {
  uint32_t v[4];
};

SWAP_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

// Ten rounds of the Philox-4x32 S-box with the paper's multipliers and Weyl
// key increments.
SWAP_HD u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, ctr.v[0], hi0, lo0);
    mulhilo32(M1, ctr.v[2], hi1, lo1);
    u32x4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Uniform double in the open interval (0,1) from one 32-bit word; exact.
SWAP_HD double u01_open(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

// Twelve uniforms for particle `id`: three Philox blocks at draw counters
// 0, 1, 2.  Key = (seed_lo ^ stream, seed_hi).
SWAP_HD void particle_uniforms(uint64_t seed, uint32_t stream, uint64_t id, uint32_t block0, double u[12]) {
  const uint32_t k0 = (uint32_t)seed ^ stream, k1 = (uint32_t)(seed >> 32);
  for (uint32_t b = 0; b < 3; ++b) {
    u32x4 c;
    c.v[0] = (uint32_t)id;
    c.v[1] = (uint32_t)(id >> 32);
    c.v[2] = block0 + b;
    c.v[3] = 0x53574150u;  // "SWAP"
    const u32x4 r = philox4x32_10(c, k0, k1);
    for (int q = 0; q < 4; ++q) u[4 * b + q] = u01_open(r.v[q]);
  }
}

// Four uniforms for a particle source or sink: stream (which rule), step
// (ion step number), slot a (new particle / cell / particle index) and draw
// block b.
SWAP_HD void source_uniforms(uint64_t seed, uint32_t stream, int64_t step, int64_t a, uint32_t b, double u[4]) {
  u32x4 c;
  c.v[0] = (uint32_t)step;
  c.v[1] = (uint32_t)a;
  c.v[2] = (uint32_t)((uint64_t)a >> 32);
  c.v[3] = b;
  const u32x4 r = philox4x32_10(c, (uint32_t)seed ^ (stream * 0x9E3779B9u), (uint32_t)(seed >> 32));
  for (int q = 0; q < 4; ++q) u[q] = u01_open(r.v[q]);
}

// One uniform in (0,1) as a float, from the first word of the same block
// (draw block 0): 24 bits, centred in its interval.
SWAP_HD float source_uniform_f32(uint64_t seed, uint32_t stream, int64_t step, int64_t a) {
  u32x4 c;
  c.v[0] = (uint32_t)step;
  c.v[1] = (uint32_t)a;
  c.v[2] = (uint32_t)((uint64_t)a >> 32);
  c.v[3] = 0u;
  const u32x4 r = philox4x32_10(c, (uint32_t)seed ^ (stream * 0x9E3779B9u), (uint32_t)(seed >> 32));
  return ((float)(r.v[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

enum : uint32_t { RNG_IONIZE = 1, RNG_INFLOW = 2, RNG_CLOUD = 3, RNG_CHEX = 4 };

}  // namespace swapk
