// Shot-group engine for d = 2 (bit planes), any team size.
//
// Every shot's tableau is (x, z, ph_s).  The x / z blocks do not depend on
// measurement outcomes or noise: pivots, factors and the x / z rowsum of
// sdim's measure (sdim/tableau/tableau_prime.py:262-334) read only x / z, and
// RESET corrections and Paulis touch phases only (sdim/program.py:335-339,
// sdim/tableau/tableau_gates.py:27-137).  So the 32 shots of a group share
// X / Z after every instruction, and each phase vector splits as
//     ph_s = c + delta_s   (mod 4, per generator)
// where c (planes C0, C1) follows the shared updates (Clifford phase terms,
// the rowsum phase terms, outcome 0, no RESET correction) and delta_s
// (planes D0[s], D1[s]) is linear in the shot's own outcomes and noise:
//   gates            : delta unchanged
//   rowsum (g in F)  : delta_g += delta_p
//   pivot columns    : delta_{n+p} = delta_p, delta_p = 2 m_s
//   deterministic M  : aph_s = aph_c + sum_{i in f} delta_i
//   RESET, noise     : delta += 2 (b x_q - a z_q) (only parity matters)
// Shot s's full tableau is (X, Z, c + delta_s) at any instruction.  The
// arithmetic per generator is that of engine_bits.cuh.
//
// Two regions per group.  The x / z region X[n][RS], Z[n][RS] (32-bit
// words) lives in shared memory when it fits, else in global memory; the hot
// region always lives in shared memory: C0[RS], C1[RS], FW[RS] (factor words
// of the last random measurement), CW[RS] (commute parities of CTA teams),
// D0[32][RS], D1[32][RS], then ints shot_m[32], shot_dp[32], shot_acc[32],
// shot_ab[32].  RS odd (see engine_bits.cuh), so thread s reading word w of
// its own delta row hits bank (s RS + w) mod 32.  Per-shot work is spread
// over (shot, chunk) pairs: thread t serves shot t % 32 and word chunk t / 32.
#pragma once
#include "engine_bits.cuh"
#include "team.cuh"

namespace sdim {

struct SlotGroupBits2 {
  static constexpr int kShots = 32;
  __host__ __device__ static size_t xz_bytes(int n) { return (size_t)4 * 2 * n * SlotBits::rs(n); }
  __host__ __device__ static size_t hot_bytes(int n) {
    return (size_t)4 * SlotBits::rs(n) * (4 + 2 * kShots) + 4 * 4 * kShots;
  }
};

template <class Team>
struct TGroupBits {
  static constexpr int kWarpBlockMax = 1024;  // threads of a block of warp teams
  Team tm;
  uint32_t *X, *Z, *C0, *C1, *FW, *CW, *D0, *D1;
  int *shot_m, *shot_dp, *shot_acc, *shot_ab;
  int n, Wn, W2, RS;
  int nact;

  __device__ TGroupBits(uint8_t* xz, uint8_t* hot, int n_, int /*d*/, Team team) : tm(team), n(n_) {
    Wn = SlotBits::wn(n_);
    W2 = 2 * Wn;
    RS = SlotBits::rs(n_);
    X = reinterpret_cast<uint32_t*>(xz);
    Z = X + (size_t)n * RS;
    C0 = reinterpret_cast<uint32_t*>(hot);
    C1 = C0 + RS;
    FW = C1 + RS;
    CW = FW + RS;
    D0 = CW + RS;
    D1 = D0 + (size_t)SlotGroupBits2::kShots * RS;
    int* ints = reinterpret_cast<int*>(D1 + (size_t)SlotGroupBits2::kShots * RS);
    shot_m = ints;
    shot_dp = ints + 32;
    shot_acc = ints + 64;
    shot_ab = ints + 96;
    nact = 0;
  }
  static __host__ __device__ size_t xz_bytes(int n) { return SlotGroupBits2::xz_bytes(n); }
  static __host__ __device__ size_t hot_bytes(int n) { return SlotGroupBits2::hot_bytes(n); }

  __device__ __forceinline__ int shot_of() const { return tm.t & 31; }
  __device__ __forceinline__ int chunk_of() const { return tm.t >> 5; }
  __device__ __forceinline__ int nchunks() const { return tm.size() >> 5; }

  __device__ void init(int active_shots) {
    nact = active_shots;
    for (size_t i = tm.t; i < 2 * (size_t)n * RS; i += tm.size()) X[i] = 0u;
    for (size_t i = tm.t; i < (size_t)RS * (4 + 2 * SlotGroupBits2::kShots); i += tm.size()) C0[i] = 0u;
    tm.sync();
    for (int k = tm.t; k < n; k += tm.size()) {
      Z[(size_t)k * RS + (k >> 5)] |= 1u << (k & 31);
      X[(size_t)k * RS + Wn + (k >> 5)] |= 1u << (k & 31);
    }
    tm.sync();
  }

  // ---------------- shared gates (owned words w = t mod size) ----------------
  __device__ __forceinline__ void h(int q) {
    uint32_t* xr = X + (size_t)q * RS;
    uint32_t* zr = Z + (size_t)q * RS;
    for (int w = tm.t; w < W2; w += tm.size()) {
      const uint32_t x = xr[w], z = zr[w];
      C1[w] ^= x & z;
      xr[w] = z;
      zr[w] = x;
    }
  }
  __device__ __forceinline__ void h_inv(int q) { h(q); }
  __device__ __forceinline__ void p(int q, bool inverse) {
    const uint32_t* xr = X + (size_t)q * RS;
    uint32_t* zr = Z + (size_t)q * RS;
    for (int w = tm.t; w < W2; w += tm.size()) {
      const uint32_t x = xr[w];
      const uint32_t lo = C0[w];
      const uint32_t c = inverse ? (~lo & x) : (lo & x);
      C0[w] = lo ^ x;
      C1[w] ^= c;
      zr[w] ^= x;
    }
  }
  __device__ __forceinline__ void cnot(int c, int t, bool) {
    uint32_t* xc = X + (size_t)c * RS;
    uint32_t* xt = X + (size_t)t * RS;
    uint32_t* zc = Z + (size_t)c * RS;
    uint32_t* zt = Z + (size_t)t * RS;
    for (int w = tm.t; w < W2; w += tm.size()) {
      const uint32_t a = xc[w], b = xt[w], e = zc[w], f = zt[w];
      xt[w] = a ^ b;
      zc[w] = e ^ f;
    }
  }
  __device__ __forceinline__ void pauli(int q, int cz, int cx) {
    const uint32_t* xr = X + (size_t)q * RS;
    const uint32_t* zr = Z + (size_t)q * RS;
    const uint32_t mz = (cz & 1) ? 0xffffffffu : 0u, mx = (cx & 1) ? 0xffffffffu : 0u;
    for (int w = tm.t; w < W2; w += tm.size()) C1[w] ^= (zr[w] & mz) ^ (xr[w] & mx);
  }

  // per-shot Pauli from shot_ab[s] = cz | cx << 8 (parities only)
  __device__ void shot_pauli(int q) {
    tm.sync();
    const int s = shot_of();
    const int ab = shot_ab[s];
    const uint32_t mz = (ab & 1) ? 0xffffffffu : 0u, mx = ((ab >> 8) & 1) ? 0xffffffffu : 0u;
    if (s < nact && (mz | mx)) {
      const uint32_t* xr = X + (size_t)q * RS;
      const uint32_t* zr = Z + (size_t)q * RS;
      uint32_t* d1 = D1 + (size_t)s * RS;
      for (int w = chunk_of(); w < W2; w += nchunks()) d1[w] ^= (zr[w] & mz) ^ (xr[w] & mx);
    }
    tm.sync();
  }
  __device__ __forceinline__ void set_shot_ab(int s, int cz, int cx) { shot_ab[s] = cz | (cx << 8); }

  // shared rowsum of a random measurement; leaves the factor words in FW
  __device__ void rowsum(int q, int p, int phc) {
    const int size = tm.size(), t = tm.t;
    const uint32_t* xq = X + (size_t)q * RS;
    const int wp = p >> 5, bp = p & 31;
    const uint32_t pbit = 1u << bp;
    const uint32_t lo_m = (phc & 1) ? 0xffffffffu : 0u;
    const uint32_t hi_m = (phc & 2) ? 0xffffffffu : 0u;
    if (W2 <= size) {
      int W2p = 1;
      while (W2p < W2) W2p <<= 1;
      const int R = size / W2p;
      const int w = t & (W2p - 1), r = t / W2p;
      const bool act = w < W2 && r < R;
      uint32_t F = act ? xq[w] : 0u;
      if (w == wp) F &= ~pbit;
      if (act && r == 0) {
        FW[w] = F;
        CW[w] = 0u;
      }
      tm.sync();
      uint32_t Cp = 0u;
      if (act) {
        for (int k = r; k < n; k += R) {
          uint32_t* xr = X + (size_t)k * RS;
          uint32_t* zr = Z + (size_t)k * RS;
          const uint32_t xpk = (xr[wp] >> bp) & 1u, zpk = (zr[wp] >> bp) & 1u;
          const uint32_t zk = zr[w];
          Cp ^= zk & (0u - xpk);
          xr[w] ^= F & (0u - xpk);
          zr[w] = zk ^ (F & (0u - zpk));
        }
      }
      // combine the row groups: shuffles inside a warp, shared atomics across warps
      if (W2p < 32)
        for (int off = W2p; off < 32; off <<= 1) Cp ^= __shfl_xor_sync(0xffffffffu, Cp, off);
      if (size > 32) {
        if (act && (W2p >= 32 || (t & 31) < W2p) && Cp) atomicXor(&CW[w], Cp);
        tm.sync();
        if (act && r == 0) Cp = CW[w];
      }
      if (act && r == 0) {
        const uint32_t lo = C0[w];
        const uint32_t a_lo = F & lo_m;
        C0[w] = lo ^ a_lo;
        C1[w] ^= (F & (hi_m ^ Cp)) ^ (lo & a_lo);
      }
    } else {
      for (int w = t; w < W2; w += size) {
        uint32_t F = xq[w];
        if (w == wp) F &= ~pbit;
        FW[w] = F;
        uint32_t Cp = 0u;
        for (int k = 0; k < n; ++k) {
          uint32_t* xr = X + (size_t)k * RS;
          uint32_t* zr = Z + (size_t)k * RS;
          const uint32_t xpk = (xr[wp] >> bp) & 1u, zpk = (zr[wp] >> bp) & 1u;
          const uint32_t zk = zr[w];
          Cp ^= zk & (0u - xpk);
          xr[w] ^= F & (0u - xpk);
          zr[w] = zk ^ (F & (0u - zpk));
        }
        const uint32_t lo = C0[w];
        const uint32_t a_lo = F & lo_m;
        C0[w] = lo ^ a_lo;
        C1[w] ^= (F & (hi_m ^ Cp)) ^ (lo & a_lo);
      }
    }
  }

  // Outcome of shot s left in shot_m[s]; returns the deterministic flag.
  __device__ int measure(int q, unsigned long long seed, long long group_shot0, uint32_t ordinal) {
    tm.sync();
    const int size = tm.size(), t = tm.t;
    const uint32_t* xq = X + (size_t)q * RS;
    int mine = INT_MAX;
    for (int w = t; w < Wn; w += size) {
      const uint32_t v = xq[w];
      if (v) { mine = (w << 5) + __ffs(v) - 1; break; }
    }
    const int p = tm.min(mine);
    const int s = shot_of(), ch = chunk_of(), nch = nchunks();
    const bool live = s < nact;
    uint32_t* d0 = D0 + (size_t)s * RS;
    uint32_t* d1 = D1 + (size_t)s * RS;
    if (p < n) {
      const int wp = p >> 5, bp = p & 31;
      const uint32_t pbit = 1u << bp;
      const int wd = Wn + wp;
      const int phc = (int)((C0[wp] >> bp) & 1u) | (int)(((C1[wp] >> bp) & 1u) << 1);
      if (ch == 0)
        shot_dp[s] = live ? (int)((d0[wp] >> bp) & 1u) | (int)(((d1[wp] >> bp) & 1u) << 1) : 0;
      tm.sync();
      rowsum(q, p, phc);
      tm.sync();
      const int dp = live ? shot_dp[s] : 0;
      if (dp) {
        const uint32_t m0 = (dp & 1) ? 0xffffffffu : 0u, m1 = (dp & 2) ? 0xffffffffu : 0u;
        for (int w = ch; w < W2; w += nch) {
          const uint32_t F = FW[w];
          const uint32_t lo = d0[w];
          const uint32_t a = F & m0;
          d0[w] = lo ^ a;
          d1[w] ^= (F & m1) ^ (lo & a);
        }
      }
      // shared pivot columns
      for (int k = t; k < n; k += size) {
        uint32_t* xr = X + (size_t)k * RS;
        uint32_t* zr = Z + (size_t)k * RS;
        const uint32_t xs = xr[wp], zs = zr[wp];
        xr[wd] = (xr[wd] & ~pbit) | (xs & pbit);
        zr[wd] = (zr[wd] & ~pbit) | (zs & pbit);
        xr[wp] = xs & ~pbit;
        zr[wp] = (zs & ~pbit) | ((k == q) ? pbit : 0u);
      }
      tm.sync();
      if (ch == 0) {
        int m = 0;
        if (live) {
          m = mulshift(stream_block(seed, group_shot0 + s, ordinal, 0u).x, 2u);
          d0[wd] = (d0[wd] & ~pbit) | ((uint32_t)(dp & 1) << bp);
          d1[wd] = (d1[wd] & ~pbit) | ((uint32_t)(dp >> 1) << bp);
          d0[wp] &= ~pbit;
          d1[wp] = (d1[wp] & ~pbit) | ((uint32_t)m << bp);
        }
        shot_m[s] = m;
      }
      if (tm.leader()) {
        C0[wd] = (C0[wd] & ~pbit) | ((uint32_t)(phc & 1) << bp);
        C1[wd] = (C1[wd] & ~pbit) | ((uint32_t)(phc >> 1) << bp);
        C0[wp] &= ~pbit;
        C1[wp] &= ~pbit;
      }
      tm.sync();
      return 0;
    }
    // deterministic: shared part aph_c, then per shot sum_{i in f} delta_i
    const uint32_t* fq = xq + Wn;
    if (ch == 0) shot_acc[s] = 0;
    int pl = 0;
    for (int w = t; w < Wn; w += size) {
      const uint32_t f = fq[w];
      pl += __popc(f & C0[w]) + 2 * __popc(f & C1[w]);
    }
    uint32_t tpar = 0u;
    for (int k = t; k < n; k += size) {
      const uint32_t* xr = X + (size_t)k * RS;
      const uint32_t* zr = Z + (size_t)k * RS;
      uint32_t carry = 0u;
      for (int w = 0; w < Wn; ++w) {
        const uint32_t f = fq[w];
        if (!f) continue;
        const uint32_t a = xr[w] & f, b = zr[w] & f;
        uint32_t v = b;
        v ^= v << 1;
        v ^= v << 2;
        v ^= v << 4;
        v ^= v << 8;
        v ^= v << 16;
        const uint32_t excl = (v ^ b) ^ (0u - carry);
        tpar ^= (uint32_t)__popc(a & excl) & 1u;
        carry ^= (uint32_t)__popc(b) & 1u;
      }
    }
    int sacc = 0;
    if (live) {
      for (int w = ch; w < Wn; w += nch) {
        const uint32_t f = fq[w];
        sacc += __popc(f & d0[w]) + 2 * __popc(f & d1[w]);
      }
    }
    const int P = tm.add(pl) & 3;
    const uint32_t T = tm.bxor(tpar) & 1u;
    const int aphc = (P + 2 * (int)T) & 3;
    if (nch > 1) {
      if (live && sacc) atomicAdd(&shot_acc[s], sacc);
      tm.sync();
      sacc = shot_acc[s];
    }
    if (ch == 0) shot_m[s] = live ? ((((aphc + sacc) & 3) + 1) >> 1) & 1 : 0;
    tm.sync();
    return 1;
  }

  // RESET correction per shot: X applied m_s times, delta -= 2 m_s z_q
  __device__ void reset_fix(int q) {
    const int s = shot_of();
    const bool on = (s < nact) && (shot_m[s] & 1);
    if (tm.any(on)) {
      if (on) {
        const uint32_t* zr = Z + (size_t)q * RS;
        uint32_t* d1 = D1 + (size_t)s * RS;
        for (int w = chunk_of(); w < W2; w += nchunks()) d1[w] ^= zr[w];
      }
      tm.sync();
    }
  }

  __device__ void export_shot(int src, int8_t* dst) {
    tm.sync();
    const size_t nn = (size_t)n * n;
    for (size_t e = tm.t; e < nn; e += tm.size()) {
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
    for (int i = tm.t; i < n; i += tm.size()) {
      for (int half = 0; half < 2; ++half) {
        const int w = half * Wn + (i >> 5), b = i & 31;
        const int c = (int)((C0[w] >> b) & 1u) | (int)(((C1[w] >> b) & 1u) << 1);
        const int dl = (int)((e0[w] >> b) & 1u) | (int)(((e1[w] >> b) & 1u) << 1);
        dst[half ? 4 * nn + n + i : 2 * nn + i] = (int8_t)((c + dl) & 3);
      }
    }
    tm.sync();
  }
};

}  // namespace sdim
