// Shot-group engine for odd prime d (residue bytes), any team size.
//
// Same decomposition as the d = 2 group engine (group_bits.cuh): the 32
// shots of a group share the x / z blocks and a common phase vector c; shot
// s keeps delta_s with ph_s = c + delta_s (mod d).  Every update of the
// reference's ExtendedTableau (sdim/tableau/tableau_prime.py:262-380) is
// affine in the phases with coefficients that depend only on x / z:
//   gates                    : delta unchanged (the phase terms go to c)
//   exponentiate(p, e)       : delta_p *= e
//   rowsum (factor f_g)      : delta_g += f_g delta_p
//   pivot columns            : delta_{n+p} = delta_p, delta_p = -m_s
//   deterministic outcome    : aph_s = aph_c + sum_i f_i delta_i
//   RESET (k = -m_s), noise  : delta += (cx x_q + cz z_q)
//
// Two regions per group.  The x / z region X[n][S], Z[n][S] (bytes; row k =
// qudit k, column g = generator g) lives in shared memory when it fits, else
// in global memory; the hot region always lives in shared memory:
// C[S], FW[S] (factors), CX[NP], CZ[NP] (pivot column), D[32][S] (deltas),
// DOT[S] ints (column dot products), then ints shot_m[32], shot_dp[32],
// shot_acc[32], shot_ab[32].  S is a multiple of 4 with S / 4 odd, so 32
// threads reading the same generator of 32 delta rows hit 32 banks.
//
// The rowsum of a random measurement is a rank-1 update of X and Z plus the
// column dots Z^T x_p: threads own 32-bit words (4 generators) of a set of
// rows and keep rows in flight (16 for the trace engine's x / z pass and 8
// for a CTA team, whose x / z region may stream from global memory; four for
// a warp team), so the region is read and written at full width.  Per-shot work is spread over (shot,
// chunk) thread pairs: thread t serves shot t % 32 and chunk t / 32.
#pragma once
#include <type_traits>

#include "engine_u8.cuh"
#include "team.cuh"

namespace sdim {

// Four residues of a 32-bit word, each in [0, d^2 - d], reduced mod d at
// once for d in {3, 5, 7}: even and odd bytes go through 16-bit lanes, where
// floor(v / d) = (v m) >> 8 with m = 86, 52, 37 is exact over that range.
template <int DD>
__device__ __forceinline__ uint32_t packed_mod(uint32_t v) {
  constexpr uint32_t m = DD == 3 ? 86u : DD == 5 ? 52u : 37u;
  const uint32_t lo = v & 0x00FF00FFu, hi = (v >> 8) & 0x00FF00FFu;
  const uint32_t qlo = ((lo * m) >> 8) & 0x00FF00FFu, qhi = ((hi * m) >> 8) & 0x00FF00FFu;
  return (lo - qlo * (uint32_t)DD) | ((hi - qhi * (uint32_t)DD) << 8);
}

struct SlotGroupU8 {
  static constexpr int kShots = 32;
  __host__ __device__ static size_t xz_bytes(int n) { return 2 * (size_t)n * SlotU8::stride(n); }
  __host__ __device__ static size_t hot_bytes(int n) {
    const size_t s = (size_t)SlotU8::stride(n);
    const size_t b = (2 + kShots) * s + 2 * (size_t)SlotU8::npad(n) + 4 * s;
    return ((b + 15) & ~(size_t)15) + 4 * 4 * kShots;
  }
};

template <int DD, class Team>
struct TGroupU8 {
  static constexpr int kWarpBlockMax = 512;  // threads of a block of warp teams
  Team tm;
  ModU8<DD> M;
  uint8_t *X, *Z, *C, *FW, *CX, *CZ, *D;
  int* DOT;
  int *shot_m, *shot_dp, *shot_acc, *shot_ab;
  int n, S;
  int nact;  // shots of this group that exist

  __device__ TGroupU8(uint8_t* xz, uint8_t* hot, int n_, int d, Team team) : tm(team), M(d), n(n_) {
    S = SlotU8::stride(n_);
    const int np = SlotU8::npad(n_);
    X = xz;
    Z = X + (size_t)n * S;
    C = hot;
    FW = C + S;
    D = FW + S;
    CX = D + (size_t)SlotGroupU8::kShots * S;
    CZ = CX + np;
    DOT = reinterpret_cast<int*>(CZ + np);
    const size_t b = (2 + SlotGroupU8::kShots) * (size_t)S + 2 * (size_t)np + 4 * (size_t)S;
    int* ints = reinterpret_cast<int*>(hot + ((b + 15) & ~(size_t)15));
    shot_m = ints;
    shot_dp = ints + 32;
    shot_acc = ints + 64;
    shot_ab = ints + 96;
    nact = 0;
  }
  static __host__ __device__ size_t xz_bytes(int n) { return SlotGroupU8::xz_bytes(n); }
  static __host__ __device__ size_t hot_bytes(int n) { return SlotGroupU8::hot_bytes(n); }

  __device__ void init(int active_shots) {
    nact = active_shots;
    uint32_t* xw = reinterpret_cast<uint32_t*>(X);
    for (size_t i = tm.t; i < ((2 * (size_t)n * S) >> 2); i += tm.size()) xw[i] = 0u;
    uint32_t* hw = reinterpret_cast<uint32_t*>(C);
    for (size_t i = tm.t; i < (((2 + (size_t)SlotGroupU8::kShots) * S) >> 2); i += tm.size()) hw[i] = 0u;
    tm.sync();
    for (int k = tm.t; k < n; k += tm.size()) {
      Z[(size_t)k * S + k] = 1;
      X[(size_t)k * S + n + k] = 1;
    }
    tm.sync();
  }

  __device__ __forceinline__ int shot_of() const { return tm.t & 31; }
  __device__ __forceinline__ int chunk_of() const { return tm.t >> 5; }
  __device__ __forceinline__ int nchunks() const { return tm.size() >> 5; }

  // ---------------- shared Clifford gates (owned columns g = t mod size) ----------------
  __device__ __forceinline__ void h(int q) {
    uint8_t* xr = X + (size_t)q * S;
    uint8_t* zr = Z + (size_t)q * S;
    for (int g = tm.t; g < 2 * n; g += tm.size()) {
      const int x = xr[g], z = zr[g];
      const int nx = M.neg(z);
      C[g] = (uint8_t)M.mo(C[g] + M.phi * nx * x);
      xr[g] = (uint8_t)nx;
      zr[g] = (uint8_t)x;
    }
  }
  __device__ __forceinline__ void h_inv(int q) {
    uint8_t* xr = X + (size_t)q * S;
    uint8_t* zr = Z + (size_t)q * S;
    for (int g = tm.t; g < 2 * n; g += tm.size()) {
      const int x = xr[g], z = zr[g];
      const int nz = M.neg(x);
      C[g] = (uint8_t)M.mo(C[g] + M.phi * z * nz);
      xr[g] = (uint8_t)z;
      zr[g] = (uint8_t)nz;
    }
  }
  __device__ __forceinline__ void p(int q, bool inverse) {
    const uint8_t* xr = X + (size_t)q * S;
    uint8_t* zr = Z + (size_t)q * S;
    for (int g = tm.t; g < 2 * n; g += tm.size()) {
      const int x = xr[g];
      const int t = M.mo((x * (x - 1)) >> 1);
      if (!inverse) {
        C[g] = (uint8_t)M.mo(C[g] + t);
        zr[g] = (uint8_t)M.md(zr[g] + x);
      } else {
        C[g] = (uint8_t)M.mo(C[g] + M.ord - t);
        zr[g] = (uint8_t)M.md(zr[g] + M.d - x);
      }
    }
  }
  __device__ __forceinline__ void cnot(int c, int t, bool inverse) {
    uint8_t* xc = X + (size_t)c * S;
    uint8_t* xt = X + (size_t)t * S;
    uint8_t* zc = Z + (size_t)c * S;
    uint8_t* zt = Z + (size_t)t * S;
    for (int g = tm.t; g < 2 * n; g += tm.size()) {
      const int a = xc[g], b = xt[g], e = zc[g], f = zt[g];
      if (!inverse) {
        xt[g] = (uint8_t)M.md(b + a);
        zc[g] = (uint8_t)M.md(e + M.d - f);
      } else {
        xt[g] = (uint8_t)M.md(b + M.d - a);
        zc[g] = (uint8_t)M.md(e + f);
      }
    }
  }
  __device__ __forceinline__ void pauli(int q, int cz, int cx) {
    const uint8_t* xr = X + (size_t)q * S;
    const uint8_t* zr = Z + (size_t)q * S;
    for (int g = tm.t; g < 2 * n; g += tm.size()) C[g] = (uint8_t)M.mo(C[g] + M.phi * (cz * zr[g] + cx * xr[g]));
  }

  // ---------------- per-shot Pauli from shot_ab[s] = cz | cx << 8 ----------------
  __device__ void shot_pauli(int q) {
    tm.sync();
    const int s = shot_of();
    const int ab = shot_ab[s];
    const int cz = ab & 0xff, cx = ab >> 8;
    if (s < nact && (cz | cx)) {
      const uint8_t* xr = X + (size_t)q * S;
      const uint8_t* zr = Z + (size_t)q * S;
      uint8_t* ds = D + (size_t)s * S;
      for (int g = chunk_of(); g < 2 * n; g += nchunks())
        ds[g] = (uint8_t)M.mo(ds[g] + M.phi * (cz * zr[g] + cx * xr[g]));
    }
    tm.sync();
  }
  __device__ __forceinline__ void set_shot_ab(int s, int cz, int cx) { shot_ab[s] = cz | (cx << 8); }

  // One 32-bit word of 4 residues of a row absorbs the pivot entries (a, b):
  // x_j += f_j a, z_j += f_j b; dots_j += z_j a (old z).
  __device__ __forceinline__ void word_update(uint32_t& xw, uint32_t& zw, uint32_t fw, int a, int b, int* dots) const {
    uint32_t xo = 0u, zo = 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int f = (fw >> (8 * j)) & 0xff;
      const int x = (xw >> (8 * j)) & 0xff, z = (zw >> (8 * j)) & 0xff;
      dots[j] += z * a;
      xo |= (uint32_t)M.md(x + f * a) << (8 * j);
      zo |= (uint32_t)M.md(z + f * b) << (8 * j);
    }
    xw = xo;
    zw = zo;
  }

  // Shared rowsum (tableau_prime.py:308-322) as a rank-1 update of X and Z
  // over the words with a nonzero factor, with the dots Z^T x_p in DOT.
  // Needs FW (all 2n factors) and CX / CZ; leaves DOT[g] for every generator.
  __device__ void rank1(int p) {
    const int size = tm.size(), t = tm.t;
    const int words = (2 * n + 3) >> 2;  // 32-bit words per row holding generators
    for (int g = t; g < 2 * n; g += size) DOT[g] = 0;
    tm.sync();
    const int R = size >= words ? size / words : 1;     // row groups
    const int act_threads = size >= words ? R * words : size;
    if (t < act_threads) {
      const int w0 = size >= words ? t % words : t;
      const int r = size >= words ? t / words : 0;
      const uint32_t* fws = reinterpret_cast<const uint32_t*>(FW);
      for (int w = w0; w < words; w += (size >= words ? words : size)) {
        const uint32_t fw = fws[w];
        if (fw == 0u) continue;
        int dots[4] = {0, 0, 0, 0};
        uint32_t* xcol = reinterpret_cast<uint32_t*>(X) + w;
        uint32_t* zcol = reinterpret_cast<uint32_t*>(Z) + w;
        const int S4 = S >> 2;
        int k = r;
        if constexpr (DD == 3 || DD == 5 || DD == 7) {
          // four residues per operation (packed_mod): f a <= (d-1)^2 and
          // x + f a <= d^2 - d stay inside a byte; dots add up in 16-bit lanes
          uint32_t dlo = 0u, dhi = 0u;
          int rows = 0;
          // RF rows in flight: their loads are issued before any store, which
          // is what hides the latency when a large tableau streams from global
          // memory (16 for the trace engine's x / z pass, 8 for the CTA-team
          // group engine within its registers; a warp team's tableau is in
          // shared memory)
          constexpr int RF = std::is_same<Team, StreamCtaTeam>::value ? 16
                             : std::is_same<Team, CtaTeam>::value     ? 8
                                                                      : 4;
          for (; k + (RF - 1) * R < n; k += RF * R) {
            uint32_t xw[RF], zw[RF];
#pragma unroll
            for (int i = 0; i < RF; ++i) {
              xw[i] = xcol[(size_t)(k + i * R) * S4];
              zw[i] = zcol[(size_t)(k + i * R) * S4];
            }
#pragma unroll
            for (int i = 0; i < RF; ++i) {
              const uint32_t a = CX[k + i * R], b = CZ[k + i * R];
              dlo += (zw[i] & 0x00FF00FFu) * a;
              dhi += ((zw[i] >> 8) & 0x00FF00FFu) * a;
              xcol[(size_t)(k + i * R) * S4] = packed_mod<DD>(xw[i] + fw * a);
              zcol[(size_t)(k + i * R) * S4] = packed_mod<DD>(zw[i] + fw * b);
            }
            if ((rows += RF) >= 1024) {  // 1024 (d-1)^2 < 2^16
              dots[0] += (int)(dlo & 0xffffu);
              dots[2] += (int)(dlo >> 16);
              dots[1] += (int)(dhi & 0xffffu);
              dots[3] += (int)(dhi >> 16);
              dlo = dhi = 0u;
              rows = 0;
            }
          }
          for (; k < n; k += R) {
            const uint32_t xw = xcol[(size_t)k * S4], zw = zcol[(size_t)k * S4];
            const uint32_t a = CX[k], b = CZ[k];
            dlo += (zw & 0x00FF00FFu) * a;
            dhi += ((zw >> 8) & 0x00FF00FFu) * a;
            xcol[(size_t)k * S4] = packed_mod<DD>(xw + fw * a);
            zcol[(size_t)k * S4] = packed_mod<DD>(zw + fw * b);
          }
          dots[0] += (int)(dlo & 0xffffu);
          dots[2] += (int)(dlo >> 16);
          dots[1] += (int)(dhi & 0xffffu);
          dots[3] += (int)(dhi >> 16);
        }
        for (; k + 3 * R < n; k += 4 * R) {
          uint32_t x0 = xcol[(size_t)k * S4], x1 = xcol[(size_t)(k + R) * S4];
          uint32_t x2 = xcol[(size_t)(k + 2 * R) * S4], x3 = xcol[(size_t)(k + 3 * R) * S4];
          uint32_t z0 = zcol[(size_t)k * S4], z1 = zcol[(size_t)(k + R) * S4];
          uint32_t z2 = zcol[(size_t)(k + 2 * R) * S4], z3 = zcol[(size_t)(k + 3 * R) * S4];
          word_update(x0, z0, fw, CX[k], CZ[k], dots);
          word_update(x1, z1, fw, CX[k + R], CZ[k + R], dots);
          word_update(x2, z2, fw, CX[k + 2 * R], CZ[k + 2 * R], dots);
          word_update(x3, z3, fw, CX[k + 3 * R], CZ[k + 3 * R], dots);
          xcol[(size_t)k * S4] = x0;
          xcol[(size_t)(k + R) * S4] = x1;
          xcol[(size_t)(k + 2 * R) * S4] = x2;
          xcol[(size_t)(k + 3 * R) * S4] = x3;
          zcol[(size_t)k * S4] = z0;
          zcol[(size_t)(k + R) * S4] = z1;
          zcol[(size_t)(k + 2 * R) * S4] = z2;
          zcol[(size_t)(k + 3 * R) * S4] = z3;
          // keep the dot sums small: reduce every block of four rows
#pragma unroll
          for (int j = 0; j < 4; ++j) dots[j] = M.md(dots[j]);
        }
        for (; k < n; k += R) {
          uint32_t x0 = xcol[(size_t)k * S4], z0 = zcol[(size_t)k * S4];
          word_update(x0, z0, fw, CX[k], CZ[k], dots);
          xcol[(size_t)k * S4] = x0;
          zcol[(size_t)k * S4] = z0;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int g = 4 * w + j;
          if (g < 2 * n && ((fw >> (8 * j)) & 0xff)) {
            if (R > 1)
              atomicAdd(&DOT[g], M.md(dots[j]));
            else
              DOT[g] = M.md(dots[j]);
          }
        }
      }
    }
    tm.sync();
  }

  // ---------------- Z measurement of every shot of the group ----------------
  // Outcome of shot s left in shot_m[s]; returns the (shared) deterministic flag.
  __device__ int measure(int q, unsigned long long seed, long long group_shot0, uint32_t ordinal) {
    tm.sync();
    const int size = tm.size(), t = tm.t;
    const uint8_t* xq = X + (size_t)q * S;
    int mine = INT_MAX;
    for (int g = t; g < n; g += size) {
      if (xq[g]) { mine = g; break; }
    }
    const int p = tm.min(mine);
    const int s = shot_of(), ch = chunk_of(), nch = nchunks();
    const bool live = s < nact;
    uint8_t* ds = D + (size_t)s * S;
    if (p < n) {
      const int xv = xq[p];
      if (xv != 1) {
        const int e = M.inv(xv);
        int sl = 0;
        for (int k = t; k < n; k += size) sl += X[(size_t)k * S + p] * Z[(size_t)k * S + p];
        const int s0 = M.md(tm.add(sl));
        tm.sync();
        if (tm.leader()) C[p] = (uint8_t)M.mo(C[p] * e + M.md(s0 * M.md((e * (e - 1)) >> 1)) * M.phi);
        for (int k = t; k < n; k += size) {
          X[(size_t)k * S + p] = (uint8_t)M.md(X[(size_t)k * S + p] * e);
          Z[(size_t)k * S + p] = (uint8_t)M.md(Z[(size_t)k * S + p] * e);
        }
        if (ch == 0 && live) ds[p] = (uint8_t)M.mo(ds[p] * e);
        tm.sync();
      }
      int sl = 0;
      for (int k = t; k < n; k += size) {
        const int a = X[(size_t)k * S + p], b = Z[(size_t)k * S + p];
        CX[k] = (uint8_t)a;
        CZ[k] = (uint8_t)b;
        sl += a * b;
      }
      // factors of every generator; stabilizer p and the padding stay 0
      for (int g = t; g < S; g += size) FW[g] = (g < 2 * n && g != p) ? (uint8_t)M.neg(xq[g]) : (uint8_t)0;
      const int s1 = M.md(tm.add(sl));
      const int phc = C[p];
      if (ch == 0) shot_dp[s] = live ? ds[p] : 0;
      tm.sync();
      rank1(p);
      // common phases of the absorbing generators
      for (int g = t; g < 2 * n; g += size) {
        const int f = FW[g];
        if (f == 0) continue;
        const int half = M.md(s1 * ((f * (f - 1)) >> 1));
        C[g] = (uint8_t)M.mo(C[g] + phc * f + M.phi * M.md(f * DOT[g]) + M.phi * M.phi * half);
      }
      // per shot: delta_g += f_g delta_p
      const int dp = live ? shot_dp[s] : 0;
      if (dp) {
        for (int g = ch; g < 2 * n; g += nch) {
          const int f = FW[g];
          if (f) ds[g] = (uint8_t)M.mo(ds[g] + f * dp);
        }
      }
      tm.sync();
      // shared pivot columns: destabilizer p <- stabilizer p, stabilizer p <- Z_q
      for (int k = t; k < n; k += size) {
        X[(size_t)k * S + n + p] = CX[k];
        Z[(size_t)k * S + n + p] = CZ[k];
        X[(size_t)k * S + p] = 0;
        Z[(size_t)k * S + p] = (uint8_t)(k == q);
      }
      if (ch == 0) {
        int m = 0;
        if (live) {
          m = mulshift(stream_block(seed, group_shot0 + s, ordinal, 0u).x, (uint32_t)M.d);
          ds[n + p] = (uint8_t)dp;
          ds[p] = (uint8_t)M.mo(M.ord - M.mo(m * M.phi));
        }
        shot_m[s] = m;
      }
      if (tm.leader()) {
        C[n + p] = (uint8_t)phc;
        C[p] = 0;
      }
      tm.sync();
      return 0;
    }
    // deterministic (tableau_prime.py:336-363), f_i = destab_x[q][i]; the
    // factor row is read back as 32-bit words, so its padding is zeroed
    for (int i = t; i < SlotU8::npad(n); i += size) CX[i] = i < n ? xq[n + i] : (uint8_t)0;
    if (ch == 0) shot_acc[s] = 0;
    tm.sync();
    // sum_i f_i c_i here; the f_i (f_i - 1) / 2 (x_i . z_i) term is summed
    // row by row in the cross-term pass below (one pass over the tableau)
    int pl = 0, dl = 0;
    for (int i = t; i < n; i += size) {
      const int f = CX[i];
      if (f) pl += f * C[i];
    }
    // cross term: rows over threads, each row read as 32-bit words
    int tl = 0;
    const int nw = (n + 3) >> 2;
    const uint32_t* fq = reinterpret_cast<const uint32_t*>(CX);
    for (int k = t; k < n; k += size) {
      const uint32_t* xr = reinterpret_cast<const uint32_t*>(X + (size_t)k * S);
      const uint32_t* zr = reinterpret_cast<const uint32_t*>(Z + (size_t)k * S);
      int pre = 0, acc = 0, dd = 0;
      for (int w = 0; w < nw; ++w) {
        const uint32_t fw = fq[w];
        if (!fw) continue;
        const uint32_t xw = xr[w], zw = zr[w];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int f = (fw >> (8 * j)) & 0xff;
          if (f) {
            const int xv = (int)((xw >> (8 * j)) & 0xff), zv = (int)((zw >> (8 * j)) & 0xff);
            acc = M.md(acc + f * xv * pre);
            pre = M.md(pre + f * zv);
            dd = M.half_xz(dd, f, xv, zv);
          }
        }
      }
      tl += acc;
      dl += M.md(dd);
    }
    // per shot: sum_i f_i delta_i over this thread's chunk
    int sacc = 0;
    if (live) {
      for (int i = ch; i < n; i += nch) {
        const int f = CX[i];
        if (f) sacc += f * ds[i];
      }
    }
    tm.add3(pl, tl, dl);
    const int P = M.mo(pl);
    const int T = M.md(tl);
    const int Dd = M.md(dl);
    const int aphc = M.mo(P + M.phi * T + M.phi * M.phi * Dd);
    if (nch > 1) {
      if (live && sacc) atomicAdd(&shot_acc[s], sacc);
      tm.sync();
      sacc = shot_acc[s];
    }
    if (ch == 0) {
      const int aph = M.mo(aphc + M.mo(sacc));
      shot_m[s] = live ? M.md(M.d - aph) : 0;
    }
    tm.sync();
    return 1;
  }

  // RESET correction per shot: X applied k_s = -m_s mod d times
  __device__ void reset_fix(int q) {
    const int s = shot_of();
    const int k = (s < nact) ? M.md(M.d - shot_m[s]) : 0;
    if (tm.any(k != 0)) {
      if (k) {
        const uint8_t* zr = Z + (size_t)q * S;
        uint8_t* ds = D + (size_t)s * S;
        const int neg = M.d - k;
        for (int g = chunk_of(); g < 2 * n; g += nchunks()) ds[g] = (uint8_t)M.mo(ds[g] + M.phi * neg * zr[g]);
      }
      tm.sync();
    }
  }

  __device__ void export_shot(int src, int8_t* dst) {
    tm.sync();
    const size_t nn = (size_t)n * n;
    for (size_t e = tm.t; e < nn; e += tm.size()) {
      const int k = (int)(e / n), i = (int)(e % n);
      dst[e] = (int8_t)X[(size_t)k * S + i];
      dst[nn + e] = (int8_t)Z[(size_t)k * S + i];
      dst[2 * nn + n + e] = (int8_t)X[(size_t)k * S + n + i];
      dst[3 * nn + n + e] = (int8_t)Z[(size_t)k * S + n + i];
    }
    const uint8_t* ds = D + (size_t)src * S;
    for (int i = tm.t; i < n; i += tm.size()) {
      dst[2 * nn + i] = (int8_t)M.mo(C[i] + ds[i]);
      dst[4 * nn + n + i] = (int8_t)M.mo(C[n + i] + ds[n + i]);
    }
    tm.sync();
  }
};

}  // namespace sdim
