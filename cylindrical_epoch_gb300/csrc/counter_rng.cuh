// counter_rng.cuh -- the counter-based random stream of device loading and
// device window injection.
//
// The reference draws every random number of the loader and of
// insert_particles from one global KISS generator (random_generator.f90),
// in a fixed serial order.  The host loader and host injector of this
// package replay that stream exactly.  The counter mode replaces it with a
// stream in which each number is a pure function of (seed, what it is for):
// Philox4x32-10 (J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), a 10-round Feistel-like bijection of
// a 128-bit counter under a 64-bit key.  Every particle can then be made by
// its own thread, in any order, and the host can recompute any number it
// needs (injection counts) without generating the particles.
//
// Key: the 64-bit seed.  Counter words (c0, c1, c2, c3):
//   loader position   (p, p >> 32, species, TAG_LOAD_POS)
//   loader momentum   (p, p >> 32, species, TAG_LOAD_MOM)
//   injection count   (row, shift, species, TAG_INJ_COUNT)
//   injection place   (j, shift, species, TAG_INJ_POS)
//   injection momentum(j, shift, species, TAG_INJ_MOM)
//   ionisation trial  (id, id >> 32, step, TAG_IONISE + 16 species)
// p is the particle's index in the species' load, j its index in the
// injected column of one species at one window shift, shift the global
// index of that shift (0 for the first shift of the run).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define CYL_HD __host__ __device__ __forceinline__
#else
#define CYL_HD inline
#endif

namespace cyl {

constexpr uint32_t TAG_LOAD_POS = 1, TAG_LOAD_MOM = 2, TAG_INJ_COUNT = 3, TAG_INJ_POS = 4, TAG_INJ_MOM = 5;
// field ionisation trial: (id, id >> 32, step, TAG_IONISE + 16 charge-state species)
constexpr uint32_t TAG_IONISE = 6;

struct U4 {
  uint32_t v[4];
};

CYL_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

// Philox4x32 with 10 rounds: multipliers 0xD2511F53, 0xCD9E8D57 and key
// increments 0x9E3779B9, 0xBB67AE85 (the golden ratio and sqrt(3) - 1 in
// 32-bit fixed point), as the paper specifies.
CYL_HD U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t key) {
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return U4{{c0, c1, c2, c3}};
}

// A 32-bit word as a double in (0, 1): (r + 1/2) 2^-32.
CYL_HD double u01(uint32_t r) { return ((double)r + 0.5) * 2.3283064365386963e-10; }

}  // namespace cyl
