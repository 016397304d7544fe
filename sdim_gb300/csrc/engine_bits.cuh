// Bit-plane engine for d = 2, one warp per tableau.
//
// Slot layout (32-bit words; bit b of word w = generator 32 w + b):
//   X[n][RS], Z[n][RS]  row k = qudit k; words [0, Wn) hold the n
//                       stabilizers, words [Wn, 2 Wn) the n destabilizers
//                       (destabilizer i at word Wn + i/32, bit i%32);
//   P0[RS], P1[RS]      phase mod 4 = P0 + 2 P1 per generator;
// Wn = ceil(n/32), W2 = 2 Wn, RS = W2 rounded up to an odd number of words so
// 32 lanes reading one word from 32 consecutive rows hit 32 banks.  Bits past
// n in each half are zero and stay zero under every update.
//
// Residue arithmetic mod 2 / phase arithmetic mod 4 of the reference's
// ExtendedTableau (sdim/tableau/tableau_optimized.py:5-118,
// sdim/tableau/tableau_prime.py:262-380) becomes word-wide boolean algebra:
//   H, H_INV : swap x/z rows, ph += 2 x z            -> P1 ^= x & z
//   P        : ph += x, z ^= x                       -> 2-bit add of x
//   P_INV    : ph -= x, z ^= x                       -> 2-bit subtract of x
//   CNOT(c,t): x_t ^= x_c, z_c ^= z_t
//   X, Z     : ph -= 2 z_q / ph += 2 x_q             -> P1 ^= z_q / x_q
// Lane l owns words w = l, l + 32, ... for gates.
#pragma once
#include "common.cuh"

namespace sdim {

struct SlotBits {
  __host__ __device__ static int wn(int n) { return (n + 31) >> 5; }
  __host__ __device__ static int rs(int n) { return (2 * wn(n)) | 1; }
  __host__ __device__ static size_t bytes(int n) { return (size_t)4 * (2 * (size_t)n + 2) * rs(n); }
};

struct EngineBits {
  static constexpr int kBackend = 1;
  uint32_t* X;
  uint32_t* Z;
  uint32_t* P0;
  uint32_t* P1;
  int n, Wn, W2, RS;

  __device__ EngineBits(uint8_t* slot, int n_, int /*d*/) : n(n_) {
    Wn = SlotBits::wn(n_);
    W2 = 2 * Wn;
    RS = SlotBits::rs(n_);
    X = reinterpret_cast<uint32_t*>(slot);
    Z = X + (size_t)n * RS;
    P0 = Z + (size_t)n * RS;
    P1 = P0 + RS;
  }

  static __host__ __device__ size_t slot_bytes(int n) { return SlotBits::bytes(n); }

  __device__ void init(int lane) {
    const size_t words = (2 * (size_t)n + 2) * RS;
    for (size_t i = lane; i < words; i += 32) X[i] = 0u;
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
      Z[(size_t)k * RS + (k >> 5)] |= 1u << (k & 31);
      X[(size_t)k * RS + Wn + (k >> 5)] |= 1u << (k & 31);
    }
    __syncwarp();
  }

  __device__ __forceinline__ void h(int lane, int q) {
    uint32_t* xr = X + (size_t)q * RS;
    uint32_t* zr = Z + (size_t)q * RS;
    for (int w = lane; w < W2; w += 32) {
      const uint32_t x = xr[w], z = zr[w];
      P1[w] ^= x & z;
      xr[w] = z;
      zr[w] = x;
    }
  }
  __device__ __forceinline__ void h_inv(int lane, int q) { h(lane, q); }

  __device__ __forceinline__ void p(int lane, int q, bool inverse) {
    const uint32_t* xr = X + (size_t)q * RS;
    uint32_t* zr = Z + (size_t)q * RS;
    for (int w = lane; w < W2; w += 32) {
      const uint32_t x = xr[w];
      const uint32_t lo = P0[w];
      const uint32_t c = inverse ? (~lo & x) : (lo & x);  // carry / borrow into bit 1
      P0[w] = lo ^ x;
      P1[w] ^= c;
      zr[w] ^= x;
    }
  }

  __device__ __forceinline__ void cnot(int lane, int c, int t, bool /*inverse*/) {
    uint32_t* xc = X + (size_t)c * RS;
    uint32_t* xt = X + (size_t)t * RS;
    uint32_t* zc = Z + (size_t)c * RS;
    uint32_t* zt = Z + (size_t)t * RS;
    for (int w = lane; w < W2; w += 32) {
      const uint32_t a = xc[w], b = xt[w], e = zc[w], f = zt[w];
      xt[w] = a ^ b;
      zc[w] = e ^ f;
    }
  }

  // ph += 2 (cz z_q + cx x_q): only the parity of each coefficient matters.
  __device__ __forceinline__ void pauli(int lane, int q, int cz, int cx) {
    const uint32_t* xr = X + (size_t)q * RS;
    const uint32_t* zr = Z + (size_t)q * RS;
    const uint32_t mz = (cz & 1) ? 0xffffffffu : 0u, mx = (cx & 1) ? 0xffffffffu : 0u;
    for (int w = lane; w < W2; w += 32) P1[w] ^= (zr[w] & mz) ^ (xr[w] & mx);
  }

  // ---------------- Z measurement, in reusable pieces ----------------
  // Lowest stabilizer with a set x bit in row q, or >= n (tableau_prime.py:273-283).
  __device__ __forceinline__ int pivot(int lane, int q) const {
    const uint32_t* xq = X + (size_t)q * RS;
    int mine = 0x7fffffff;
    for (int w = lane; w < Wn; w += 32) {
      const uint32_t v = xq[w];
      if (v) { mine = (w << 5) + __ffs(v) - 1; break; }
    }
    return __reduce_min_sync(0xffffffffu, mine);
  }
  __device__ __forceinline__ int phase_of(int g) const {
    const int w = g >> 5, b = g & 31;
    return (int)((P0[w] >> b) & 1u) | (int)(((P1[w] >> b) & 1u) << 1);
  }

  // Rowsum of a random measurement (tableau_prime.py:308-322): every
  // generator g != stabilizer p with x_q[g] = 1 absorbs the pivot column:
  // x_g ^= x_p, z_g ^= z_p, ph_g += php + 2 (z_g . x_p).  Word w of the
  // factor row F (the x_q row without bit p) is left in fw[w] when fw != 0.
  __device__ void rowsum(int lane, int q, int p, int php, uint32_t* fw) {
    const uint32_t* xq = X + (size_t)q * RS;
    const int wp = p >> 5, bp = p & 31;
    const uint32_t pbit = 1u << bp;
    const uint32_t lo_m = (php & 1) ? 0xffffffffu : 0u;
    const uint32_t hi_m = (php & 2) ? 0xffffffffu : 0u;
    if (W2 <= 32) {
      // rows split over R = 32 / W2p lane groups, W2p = pow2 >= W2
      int W2p = 1;
      while (W2p < W2) W2p <<= 1;
      const int R = 32 / W2p;
      const int w = lane & (W2p - 1), r = lane / W2p;
      const bool act = w < W2;
      uint32_t F = act ? xq[w] : 0u;
      if (w == wp) F &= ~pbit;
      if (fw && act && r == 0) fw[w] = F;
      uint32_t C = 0u;
      __syncwarp();
      if (act) {
        for (int k = r; k < n; k += R) {
          uint32_t* xr = X + (size_t)k * RS;
          uint32_t* zr = Z + (size_t)k * RS;
          const uint32_t xpk = (xr[wp] >> bp) & 1u, zpk = (zr[wp] >> bp) & 1u;
          const uint32_t zk = zr[w];
          C ^= zk & (0u - xpk);
          xr[w] ^= F & (0u - xpk);
          zr[w] = zk ^ (F & (0u - zpk));
        }
      }
      for (int off = W2p; off < 32; off <<= 1) C ^= __shfl_xor_sync(0xffffffffu, C, off);
      if (act && r == 0) {
        const uint32_t lo = P0[w];
        const uint32_t a_lo = F & lo_m;
        const uint32_t carry = lo & a_lo;
        P0[w] = lo ^ a_lo;
        P1[w] ^= (F & (hi_m ^ C)) ^ carry;
      }
    } else {
      for (int w = lane; w < W2; w += 32) {
        uint32_t F = xq[w];
        if (w == wp) F &= ~pbit;
        if (fw) fw[w] = F;
        uint32_t C = 0u;
        for (int k = 0; k < n; ++k) {
          uint32_t* xr = X + (size_t)k * RS;
          uint32_t* zr = Z + (size_t)k * RS;
          const uint32_t xpk = (xr[wp] >> bp) & 1u, zpk = (zr[wp] >> bp) & 1u;
          const uint32_t zk = zr[w];
          C ^= zk & (0u - xpk);
          xr[w] ^= F & (0u - xpk);
          zr[w] = zk ^ (F & (0u - zpk));
        }
        const uint32_t lo = P0[w];
        const uint32_t a_lo = F & lo_m;
        const uint32_t carry = lo & a_lo;
        P0[w] = lo ^ a_lo;
        P1[w] ^= (F & (hi_m ^ C)) ^ carry;
      }
    }
  }

  // destabilizer p <- stabilizer p (phase php); stabilizer p <- Z_q with
  // phase -2m (tableau_prime.py:324-333)
  __device__ void pivot_columns(int lane, int q, int p, int php, int m) {
    const int wp = p >> 5, bp = p & 31;
    const uint32_t pbit = 1u << bp;
    const int wd = Wn + wp;
    for (int k = lane; k < n; k += 32) {
      uint32_t* xr = X + (size_t)k * RS;
      uint32_t* zr = Z + (size_t)k * RS;
      const uint32_t xs = xr[wp], zs = zr[wp];
      const uint32_t xpk = (xs >> bp) & 1u, zpk = (zs >> bp) & 1u;
      xr[wd] = (xr[wd] & ~pbit) | (xpk << bp);
      zr[wd] = (zr[wd] & ~pbit) | (zpk << bp);
      xr[wp] = xs & ~pbit;
      zr[wp] = (zs & ~pbit) | ((k == q) ? pbit : 0u);
    }
    if (lane == 0) {
      P0[wd] = (P0[wd] & ~pbit) | ((uint32_t)(php & 1) << bp);
      P1[wd] = (P1[wd] & ~pbit) | ((uint32_t)(php >> 1) << bp);
      P0[wp] &= ~pbit;                                  // ph_p = -2m mod 4 = 2m
      P1[wp] = (P1[wp] & ~pbit) | ((uint32_t)(m & 1) << bp);
    }
  }

  // Deterministic outcome phase (tableau_prime.py:348-361), f = destab_x row q:
  //   aph = sum_{i in f} ph_i + 2 sum_k parity(a_k & exclusive_prefix_xor(b_k))
  // with a_k = x_k & f, b_k = z_k & f over the stabilizer words; mod 4.
  __device__ int det_phase(int lane, int q) const {
    const uint32_t* fq = X + (size_t)q * RS + Wn;
    int pl = 0;
    for (int w = lane; w < Wn; w += 32) {
      const uint32_t f = fq[w];
      pl += __popc(f & P0[w]) + 2 * __popc(f & P1[w]);
    }
    uint32_t tpar = 0u;
    for (int k = lane; k < n; k += 32) {
      const uint32_t* xr = X + (size_t)k * RS;
      const uint32_t* zr = Z + (size_t)k * RS;
      uint32_t carry = 0u;  // parity of b bits below the current word
      for (int w = 0; w < Wn; ++w) {
        const uint32_t f = fq[w];
        if (!f) continue;
        const uint32_t a = xr[w] & f, b = zr[w] & f;
        uint32_t v = b;
        v ^= v << 1;
        v ^= v << 2;
        v ^= v << 4;
        v ^= v << 8;
        v ^= v << 16;                      // inclusive prefix xor
        const uint32_t excl = (v ^ b) ^ (0u - carry);
        tpar ^= (uint32_t)__popc(a & excl) & 1u;
        carry ^= (uint32_t)__popc(b) & 1u;
      }
    }
    const int P = __reduce_add_sync(0xffffffffu, pl) & 3;
    const uint32_t T = __reduce_xor_sync(0xffffffffu, tpar) & 1u;
    return (P + 2 * (int)T) & 3;
  }

  __device__ int measure(int lane, int q, unsigned long long seed, long long shot,
                         uint32_t ordinal, int* det) {
    __syncwarp();
    const int p = pivot(lane, q);
    if (p < n) {
      const int php = phase_of(p);
      __syncwarp();
      rowsum(lane, q, p, php, nullptr);
      __syncwarp();
      const int m = mulshift(stream_block(seed, shot, ordinal, 0u).x, 2u);
      pivot_columns(lane, q, p, php, m);
      __syncwarp();
      *det = 0;
      return m;
    }
    const int aph = det_phase(lane, q);
    __syncwarp();
    *det = 1;
    return ((aph + 1) >> 1) & 1;  // floor(-aph / 2) mod 2
  }

  __device__ __forceinline__ void reset_fix(int lane, int q, int m) {
    if (m & 1) pauli(lane, q, 1, 0);
    __syncwarp();
  }

  __device__ void export_tableau(int lane, int8_t* dst) {
    __syncwarp();
    const size_t nn = (size_t)n * n;
    for (size_t e = lane; e < nn; e += 32) {
      const int k = (int)(e / n), i = (int)(e % n);
      const uint32_t* xr = X + (size_t)k * RS;
      const uint32_t* zr = Z + (size_t)k * RS;
      dst[e] = (int8_t)((xr[i >> 5] >> (i & 31)) & 1u);
      dst[nn + e] = (int8_t)((zr[i >> 5] >> (i & 31)) & 1u);
      dst[2 * nn + n + e] = (int8_t)((xr[Wn + (i >> 5)] >> (i & 31)) & 1u);
      dst[3 * nn + n + e] = (int8_t)((zr[Wn + (i >> 5)] >> (i & 31)) & 1u);
    }
    for (int i = lane; i < n; i += 32) {
      const int w = i >> 5, b = i & 31;
      dst[2 * nn + i] = (int8_t)(((P0[w] >> b) & 1u) | (((P1[w] >> b) & 1u) << 1));
      const int wdst = Wn + w;
      dst[4 * nn + n + i] = (int8_t)(((P0[wdst] >> b) & 1u) | (((P1[wdst] >> b) & 1u) << 1));
    }
    __syncwarp();
  }
};

}  // namespace sdim
