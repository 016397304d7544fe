// Residues mod d (d = 5 or 7) in 4-bit lanes: 8 residues per 32-bit word.
//
// A sum of two residues is at most 2 d - 2 <= 12, so it never carries into
// the next lane; adding 8 - d to every lane then sets bit 3 of exactly the
// lanes that reached d, and subtracting d there reduces them.  Addition,
// negation and scalar multiples are a few word operations for 8 residues;
// products of two residue words and per-lane maps go lane by lane.  Host and
// device code, checked exhaustively on the host.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define N4_FN __host__ __device__ __forceinline__
#else
#define N4_FN inline
#endif

namespace sdim {

template <int D>
struct N4 {
  static_assert(D == 5 || D == 7, "nibble residues serve d = 5 and 7");
  static constexpr uint32_t kOnes = 0x11111111u;   // 1 in every lane
  static constexpr uint32_t kD = D * kOnes;        // d in every lane
  static constexpr uint32_t kLift = (8 - D) * kOnes;

  // lanes of s in [0, 2d - 2] reduced mod d
  static N4_FN uint32_t reduce(uint32_t s) { return s - (((s + kLift) >> 3) & kOnes) * D; }
  static N4_FN uint32_t add(uint32_t a, uint32_t b) { return reduce(a + b); }
  static N4_FN uint32_t neg(uint32_t a) { return reduce(kD - a); }
  static N4_FN uint32_t sub(uint32_t a, uint32_t b) { return reduce(a + kD - b); }
  // a * c for a scalar c in [0, d)
  static N4_FN uint32_t mulc(uint32_t a, int c) {
    const uint32_t a2 = add(a, a);
    switch (c) {
      case 0: return 0u;
      case 1: return a;
      case 2: return a2;
      case 3: return add(a2, a);
      case 4: return add(a2, a2);
      case 5: return add(add(a2, a2), a);
      default: return add(add(a2, a2), a2);  // 6
    }
  }
  static N4_FN int get(uint32_t a, int j) { return (int)((a >> (4 * j)) & 15u); }
  static N4_FN uint32_t set(uint32_t a, int j, int v) {
    return (a & ~(15u << (4 * j))) | ((uint32_t)v << (4 * j));
  }
  // bit 4 j set where lane j is not zero
  static N4_FN uint32_t nz(uint32_t a) { return (a | (a >> 1) | (a >> 2) | (a >> 3)) & kOnes; }
  // lane-wise product mod d
  static N4_FN uint32_t mul(uint32_t a, uint32_t b) {
    uint32_t r = 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) r |= (uint32_t)((get(a, j) * get(b, j)) % D) << (4 * j);
    return r;
  }
  // lane-wise x (x - 1) / 2 mod d
  static N4_FN uint32_t half(uint32_t a) {
    uint32_t r = 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int x = get(a, j);
      r |= (uint32_t)(((x * (x - 1)) >> 1) % D) << (4 * j);
    }
    return r;
  }
  // sum of the 8 residues (not reduced)
  static N4_FN int rsum(uint32_t a) {
    const uint32_t b = (a & 0x0F0F0F0Fu) + ((a >> 4) & 0x0F0F0F0Fu);
    return (int)((b * 0x01010101u) >> 24);
  }
};

}  // namespace sdim
