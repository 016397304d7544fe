// Residues mod 3 in two bit planes: 32 residues per pair of 32-bit words.
//
// Residue r of lane j (bit j of both words): r = 1 sets bit j of p0, r = 2
// sets bit j of p1, r = 0 sets neither; both set never occurs.  With this
// encoding negation swaps the planes, multiplication is four ANDs and two
// ORs, and addition is two three-term sums of products, each a couple of
// LOP3 instructions, so a gate, a rank-1 row update or a column dot costs a
// few logic operations per 32 residues.  The functions are host and device
// code, so the host tests check them exhaustively against integer
// arithmetic.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define P3_FN __host__ __device__ __forceinline__
#else
#define P3_FN inline
#endif

namespace sdim {

struct P3 {
  uint32_t p0, p1;
};

P3_FN P3 p3(uint32_t a, uint32_t b) {
  P3 r;
  r.p0 = a;
  r.p1 = b;
  return r;
}
P3_FN P3 p3_zero() { return p3(0u, 0u); }
P3_FN uint32_t p3_nz(P3 a) { return a.p0 | a.p1; }
// -a mod 3
P3_FN P3 p3_neg(P3 a) { return p3(a.p1, a.p0); }
// a + b mod 3: the sum is 1 for (0, 1), (1, 0), (2, 2) and 2 for (0, 2), (2, 0), (1, 1)
P3_FN P3 p3_add(P3 a, P3 b) {
  const uint32_t za = ~(a.p0 | a.p1), zb = ~(b.p0 | b.p1);
  return p3((za & b.p0) | (zb & a.p0) | (a.p1 & b.p1), (za & b.p1) | (zb & a.p1) | (a.p0 & b.p0));
}
P3_FN P3 p3_sub(P3 a, P3 b) { return p3_add(a, p3_neg(b)); }
// a * b mod 3: 1 when equal and non-zero, 2 when different and non-zero
P3_FN P3 p3_mul(P3 a, P3 b) { return p3((a.p0 & b.p0) | (a.p1 & b.p1), (a.p0 & b.p1) | (a.p1 & b.p0)); }
// a * c mod 3 for a scalar c in [0, 3)
P3_FN P3 p3_mulc(P3 a, int c) { return c == 0 ? p3_zero() : c == 1 ? a : p3_neg(a); }
// a (a - 1) / 2 mod 3: 0, 0, 1 for a = 0, 1, 2
P3_FN P3 p3_half(P3 a) { return p3(a.p1, 0u); }
// every lane set to the scalar v in [0, 3)
P3_FN P3 p3_splat(int v) { return p3(v == 1 ? 0xffffffffu : 0u, v == 2 ? 0xffffffffu : 0u); }
// lanes moved up by s (lane j takes lane j - s; the lowest s lanes get 0)
P3_FN P3 p3_shl(P3 a, int s) { return p3(a.p0 << s, a.p1 << s); }
// lanes outside mask set to 0
P3_FN P3 p3_and(P3 a, uint32_t mask) { return p3(a.p0 & mask, a.p1 & mask); }

#ifdef __CUDACC__
P3_FN int p3_popc(uint32_t v) {
#ifdef __CUDA_ARCH__
  return __popc(v);
#else
  return __builtin_popcount(v);
#endif
}
#else
P3_FN int p3_popc(uint32_t v) { return __builtin_popcount(v); }
#endif

// sum of the 32 residues as an integer (not reduced)
P3_FN int p3_rsum(P3 a) { return p3_popc(a.p0) + 2 * p3_popc(a.p1); }
// residue of lane j
P3_FN int p3_get(P3 a, int j) { return (int)((a.p0 >> j) & 1u) | (int)(((a.p1 >> j) & 1u) << 1); }
// lane j set to v in [0, 3)
P3_FN P3 p3_set(P3 a, int j, int v) {
  const uint32_t m = 1u << j;
  return p3((a.p0 & ~m) | (v == 1 ? m : 0u), (a.p1 & ~m) | (v == 2 ? m : 0u));
}
// exclusive prefix sums mod 3 along the lanes: lane j gets sum_{i < j} a_i
P3_FN P3 p3_prefix(P3 a) {
  P3 e = p3_shl(a, 1);
  e = p3_add(e, p3_shl(e, 1));
  e = p3_add(e, p3_shl(e, 2));
  e = p3_add(e, p3_shl(e, 4));
  e = p3_add(e, p3_shl(e, 8));
  e = p3_add(e, p3_shl(e, 16));
  return e;
}

// Contribution of one word of one row to the deterministic outcome phase:
// with a = f z and b = f x over the word's lanes and carry = sum of a over
// the row's earlier lanes (mod 3), adds sum_j b_j (carry + sum_{i<j} a_i) to
// t and sum_j h_j x_j z_j to dd (h = f (f - 1) / 2), and returns the new
// carry.  Over the whole row this gives the cross term
// sum_{i<j} f_i z_i f_j x_j and the term sum_i h_i x_i z_i of
// sdim/tableau/tableau_prime.py:336-363.
P3_FN int p3_det_word(P3 f, P3 h, P3 x, P3 z, int carry, int& t, int& dd) {
  const P3 a = p3_mul(f, z), b = p3_mul(f, x);
  const P3 e = p3_add(p3_prefix(a), p3_splat(carry));
  t += p3_rsum(p3_mul(b, e));
  dd += p3_rsum(p3_mul(h, p3_mul(x, z)));
  return (carry + p3_rsum(a)) % 3;
}

}  // namespace sdim
