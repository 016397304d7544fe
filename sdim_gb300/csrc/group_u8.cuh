// Shot-group engine for odd prime d (residue bytes), any team size.
//
// Same decomposition as the d = 2 group engine (engine_group.cuh): the 32
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
// Slot layout (bytes): X[n][S], Z[n][S], C[S], FW[S] (factors f_g), CX[NP],
// CZ[NP], D[32][S] (deltas), then ints: shot_m[32], shot_dp[32], shot_acc[32],
// shot_ab[32], red[40].  S as in engine_u8.cuh (S / 4 odd: 32 threads reading
// the same generator of 32 different delta rows hit 32 banks).
//
// Per-shot work is spread over (shot, chunk) thread pairs: thread t serves
// shot t % 32 and generator chunk t / 32 (one chunk in a warp team).
#pragma once
#include "engine_u8.cuh"
#include "team.cuh"

namespace sdim {

struct SlotGroupU8 {
  static constexpr int kShots = 32;
  __host__ __device__ static size_t int_offset(int n) {
    const size_t s = (size_t)SlotU8::stride(n);
    const size_t b = (2 * (size_t)n + 2 + kShots) * s + 2 * (size_t)SlotU8::npad(n);
    return (b + 15) & ~(size_t)15;
  }
  __host__ __device__ static size_t bytes(int n) { return int_offset(n) + 4 * (4 * kShots + 40); }
};

template <int DD, class Team>
struct TGroupU8 {
  Team tm;
  ModU8<DD> M;
  uint8_t *X, *Z, *C, *FW, *CX, *CZ, *D;
  int *shot_m, *shot_dp, *shot_acc, *shot_ab;
  int n, S;
  int nact;  // shots of this group that exist

  __device__ TGroupU8(uint8_t* slot, int n_, int d, Team team) : tm(team), M(d), n(n_) {
    S = SlotU8::stride(n_);
    const int np = SlotU8::npad(n_);
    X = slot;
    Z = X + (size_t)n * S;
    C = Z + (size_t)n * S;
    FW = C + S;
    D = FW + S;
    CX = D + (size_t)SlotGroupU8::kShots * S;
    CZ = CX + np;
    int* ints = reinterpret_cast<int*>(slot + SlotGroupU8::int_offset(n_));
    shot_m = ints;
    shot_dp = ints + 32;
    shot_acc = ints + 64;
    shot_ab = ints + 96;
    nact = 0;
  }
  static __host__ __device__ size_t slot_bytes(int n) { return SlotGroupU8::bytes(n); }
  static __device__ int* red_of(uint8_t* slot, int n) {
    return reinterpret_cast<int*>(slot + SlotGroupU8::int_offset(n)) + 128;
  }

  __device__ void init(int active_shots) {
    nact = active_shots;
    const size_t words = ((2 * (size_t)n + 2) * S) >> 2;  // X, Z, C, FW
    uint32_t* w = reinterpret_cast<uint32_t*>(X);
    for (size_t i = tm.t; i < words; i += tm.size()) w[i] = 0u;
    uint32_t* dw = reinterpret_cast<uint32_t*>(D);
    for (size_t i = tm.t; i < ((size_t)SlotGroupU8::kShots * S) >> 2; i += tm.size()) dw[i] = 0u;
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
      const int s1 = M.md(tm.add(sl));
      const int phc = C[p];
      if (ch == 0) shot_dp[s] = live ? ds[p] : 0;
      tm.sync();
      // shared rowsum over owned columns (tableau_prime.py:308-322)
      for (int g = t; g < 2 * n; g += size) {
        const int f = (g == p) ? 0 : M.neg(xq[g]);
        FW[g] = (uint8_t)f;
        if (f == 0) continue;
        int dot = 0;
        uint8_t* xc = X + g;
        uint8_t* zc = Z + g;
        for (int k = 0; k < n; ++k) {
          const int x = xc[(size_t)k * S], z = zc[(size_t)k * S];
          const int a = CX[k], b = CZ[k];
          dot += z * a;
          xc[(size_t)k * S] = (uint8_t)M.md(x + f * a);
          zc[(size_t)k * S] = (uint8_t)M.md(z + f * b);
        }
        const int half = M.md(s1 * ((f * (f - 1)) >> 1));
        C[g] = (uint8_t)M.mo(C[g] + phc * f + M.phi * M.md(f * M.md(dot)) + M.phi * M.phi * half);
      }
      tm.sync();
      // per shot: delta_g += f_g delta_p
      const int dp = live ? shot_dp[s] : 0;
      if (dp) {
        for (int g = ch; g < 2 * n; g += nch) {
          const int f = FW[g];
          if (f) ds[g] = (uint8_t)M.mo(ds[g] + f * dp);
        }
      }
      // shared pivot columns: destabilizer p <- stabilizer p, stabilizer p <- Z_q
      for (int k = t; k < n; k += size) {
        X[(size_t)k * S + n + p] = CX[k];
        Z[(size_t)k * S + n + p] = CZ[k];
        X[(size_t)k * S + p] = 0;
        Z[(size_t)k * S + p] = (uint8_t)(k == q);
      }
      tm.sync();
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
    // deterministic (tableau_prime.py:336-363), f_i = destab_x[q][i]
    for (int i = t; i < n; i += size) CX[i] = xq[n + i];
    if (ch == 0) shot_acc[s] = 0;
    tm.sync();
    int pl = 0, dl = 0;
    for (int i = t; i < n; i += size) {
      const int f = CX[i];
      if (!f) continue;
      pl += f * C[i];
      int cd = 0;
      for (int k = 0; k < n; ++k) cd += X[(size_t)k * S + i] * Z[(size_t)k * S + i];
      dl += M.md(M.md(cd) * ((f * (f - 1)) >> 1));
    }
    int tl = 0;
    for (int k = t; k < n; k += size) {
      const uint8_t* xr = X + (size_t)k * S;
      const uint8_t* zr = Z + (size_t)k * S;
      int pre = 0, acc = 0;
      for (int i = 0; i < n; ++i) {
        const int f = CX[i];
        if (f) {
          acc = M.md(acc + f * xr[i] * pre);
          pre = M.md(pre + f * zr[i]);
        }
      }
      tl += acc;
    }
    // per shot: sum_i f_i delta_i over this thread's chunk
    int sacc = 0;
    if (live) {
      for (int i = ch; i < n; i += nch) {
        const int f = CX[i];
        if (f) sacc += f * ds[i];
      }
    }
    const int P = M.mo(tm.add(pl));
    const int T = M.md(tm.add(tl));
    const int Dd = M.md(tm.add(dl));
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
