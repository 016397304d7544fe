// Shot-group engine for d = 2: up to 32 shots of one program per warp.
//
// Every shot's tableau is (x, z, ph_s).  The x / z blocks do not depend on
// measurement outcomes or noise: pivots, factors and the x / z rowsum of
// sdim's measure (sdim/tableau/tableau_prime.py:262-334) read only x / z, and
// RESET corrections and Paulis touch phases only (sdim/program.py:335-339,
// sdim/tableau/tableau_gates.py:27-137).  So all shots of one program share
// x / z after every instruction, and each phase vector splits as
//     ph_s = c + delta_s   (mod 4, per generator)
// where c follows the shared updates (Clifford phase terms, the rowsum phase
// terms, outcome 0, no RESET correction) and delta_s is linear in the shot's
// own outcomes and noise:
//   gates            : delta unchanged
//   rowsum (g in F)  : delta_g += delta_p
//   pivot columns    : delta_{n+p} = delta_p, delta_p = 2 m_s
//   deterministic M  : aph_s = aph_c + sum_{i in f} delta_i
//   RESET, noise     : delta += 2 (b x_q - a z_q) (only parity matters)
// Shot s's full tableau is available at any instruction as (x, z, c + delta_s).
//
// Slot: the EngineBits region (X, Z, C0 = P0, C1 = P1), then FW[RS] (factor
// words), then D0[32][RS], D1[32][RS] (delta planes; RS odd, so lane s reading
// word w of its own row hits bank (s RS + w) mod 32: conflict-free).
#pragma once
#include "engine_bits.cuh"

namespace sdim {

struct SlotGroupBits {
  static constexpr int kShots = 32;
  __host__ __device__ static size_t bytes(int n) {
    const int rs = SlotBits::rs(n);
    return (size_t)4 * rs * ((2 * (size_t)n + 2) + 1 + 2 * kShots);
  }
};

struct GroupBits {
  EngineBits sh;
  uint32_t* FW;
  uint32_t* D0;
  uint32_t* D1;
  int n, Wn, W2, RS;

  __device__ GroupBits(uint8_t* slot, int n_, int d) : sh(slot, n_, d) {
    n = n_;
    Wn = sh.Wn;
    W2 = sh.W2;
    RS = sh.RS;
    FW = sh.P1 + RS;
    D0 = FW + RS;
    D1 = D0 + SlotGroupBits::kShots * RS;
  }
  static __host__ __device__ size_t slot_bytes(int n) { return SlotGroupBits::bytes(n); }

  __device__ void init(int lane) {
    sh.init(lane);
    for (int i = lane; i < 2 * SlotGroupBits::kShots * RS; i += 32) D0[i] = 0u;
    __syncwarp();
  }

  // shared gates
  __device__ __forceinline__ void h(int lane, int q) { sh.h(lane, q); }
  __device__ __forceinline__ void h_inv(int lane, int q) { sh.h(lane, q); }
  __device__ __forceinline__ void p(int lane, int q, bool inv) { sh.p(lane, q, inv); }
  __device__ __forceinline__ void cnot(int lane, int c, int t, bool inv) { sh.cnot(lane, c, t, inv); }
  __device__ __forceinline__ void pauli(int lane, int q, int cz, int cx) { sh.pauli(lane, q, cz, cx); }

  // per-shot Pauli: delta_s += 2 (cz z_q + cx x_q) for the lanes with on = true
  __device__ void shot_pauli(int lane, bool on, int q, int cz, int cx) {
    __syncwarp();
    if (on && ((cz | cx) & 1)) {
      const uint32_t* xr = sh.X + (size_t)q * RS;
      const uint32_t* zr = sh.Z + (size_t)q * RS;
      const uint32_t mz = (cz & 1) ? 0xffffffffu : 0u, mx = (cx & 1) ? 0xffffffffu : 0u;
      uint32_t* d1 = D1 + (size_t)lane * RS;
      for (int w = 0; w < W2; ++w) d1[w] ^= (zr[w] & mz) ^ (xr[w] & mx);
    }
    __syncwarp();
  }

  // Z measurement of qudit q for every shot of the group; returns lane s's
  // outcome, *det the (shared) deterministic flag.
  __device__ int measure(int lane, bool active, int q, unsigned long long seed, long long shot,
                         uint32_t ordinal, int* det) {
    __syncwarp();
    const int p = sh.pivot(lane, q);
    uint32_t* d0 = D0 + (size_t)lane * RS;
    uint32_t* d1 = D1 + (size_t)lane * RS;
    if (p < n) {
      const int wp = p >> 5, bp = p & 31;
      const uint32_t pbit = 1u << bp;
      const int wd = Wn + wp;
      const int phc = sh.phase_of(p);
      const uint32_t dp0 = (d0[wp] >> bp) & 1u, dp1 = (d1[wp] >> bp) & 1u;
      __syncwarp();
      sh.rowsum(lane, q, p, phc, FW);
      __syncwarp();
      if (active && (dp0 | dp1)) {
        // delta_g += delta_p for g in F
        const uint32_t m0 = 0u - dp0, m1 = 0u - dp1;
        for (int w = 0; w < W2; ++w) {
          const uint32_t F = FW[w];
          const uint32_t lo = d0[w];
          const uint32_t a = F & m0;
          d0[w] = lo ^ a;
          d1[w] ^= (F & m1) ^ (lo & a);
        }
      }
      sh.pivot_columns(lane, q, p, phc, 0);
      int m = 0;
      if (active) {
        m = mulshift(stream_block(seed, shot, ordinal, 0u).x, 2u);
        d0[wd] = (d0[wd] & ~pbit) | (dp0 << bp);
        d1[wd] = (d1[wd] & ~pbit) | (dp1 << bp);
        d0[wp] &= ~pbit;
        d1[wp] = (d1[wp] & ~pbit) | ((uint32_t)m << bp);
      }
      __syncwarp();
      *det = 0;
      return m;
    }
    const int aphc = sh.det_phase(lane, q);
    int m = 0;
    if (active) {
      const uint32_t* fq = sh.X + (size_t)q * RS + Wn;
      int s = aphc;
      for (int w = 0; w < Wn; ++w) {
        const uint32_t f = fq[w];
        s += __popc(f & d0[w]) + 2 * __popc(f & d1[w]);
      }
      m = (((s & 3) + 1) >> 1) & 1;
    }
    __syncwarp();
    *det = 1;
    return m;
  }

  // RESET correction per shot: X applied m times: delta -= 2 m z_q
  __device__ void reset_fix(int lane, bool active, int q, int m) { shot_pauli(lane, active && (m & 1), q, 1, 0); }

  // shot (lane src) tableau in the reference's int8 block order
  __device__ void export_shot(int lane, int src, int8_t* dst) {
    __syncwarp();
    const size_t nn = (size_t)n * n;
    const uint32_t* X = sh.X;
    const uint32_t* Z = sh.Z;
    for (size_t e = lane; e < nn; e += 32) {
      const int k = (int)(e / n), i = (int)(e % n);
      const uint32_t* xr = X + (size_t)k * RS;
      const uint32_t* zr = Z + (size_t)k * RS;
      dst[e] = (int8_t)((xr[i >> 5] >> (i & 31)) & 1u);
      dst[nn + e] = (int8_t)((zr[i >> 5] >> (i & 31)) & 1u);
      dst[2 * nn + n + e] = (int8_t)((xr[Wn + (i >> 5)] >> (i & 31)) & 1u);
      dst[3 * nn + n + e] = (int8_t)((zr[Wn + (i >> 5)] >> (i & 31)) & 1u);
    }
    const uint32_t* e0 = D0 + (size_t)src * RS;
    const uint32_t* e1 = D1 + (size_t)src * RS;
    for (int i = lane; i < n; i += 32) {
      for (int half = 0; half < 2; ++half) {
        const int w = half * Wn + (i >> 5), b = i & 31;
        const int c = (int)((sh.P0[w] >> b) & 1u) | (int)(((sh.P1[w] >> b) & 1u) << 1);
        const int dl = (int)((e0[w] >> b) & 1u) | (int)(((e1[w] >> b) & 1u) << 1);
        dst[half ? 4 * nn + n + i : 2 * nn + i] = (int8_t)((c + dl) & 3);
      }
    }
    __syncwarp();
  }
};

}  // namespace sdim
