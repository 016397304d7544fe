// Residue engine: one byte per residue, any prime d < 128, one warp per tableau.
//
// Layout of a tableau slot (shared or global memory):
//   X[n][S], Z[n][S]   row k = qudit k, byte g = generator g
//                      (g < n: stabilizer g, n <= g < 2n: destabilizer g - n),
//                      i.e. the reference's x_block[k][g] and
//                      destab_x_block[k][g - n] side by side
//                      (sdim/tableau/dataclasses.py:30-39,
//                       sdim/tableau/tableau_prime.py:76-86);
//   PH[S]              phases of the 2n generators, mod 2d (d = 2) or d;
//   CX[NP], CZ[NP]     scratch: pivot column / factor row.
// S is the row stride in bytes: 2n rounded up to a multiple of 4 with S/4 odd,
// so 32 lanes reading one word each from 32 consecutive rows hit 32 banks.
//
// Every residue is kept fully reduced.  The reference reduces lazily (every
// 64 instructions, sdim/program.py:317-318, and inside measure,
// sdim/tableau/tableau_prime.py:284-289); all of its updates are polynomials
// in the residues that are well defined modulo d (phases modulo 2d / d), so
// the reduced state after every instruction is the reference's state reduced.
//
// Lane l owns generator columns g = l, l + 32, ...  Clifford gates and the
// rowsum of a random measurement only touch owned columns, so consecutive
// gates need no synchronisation; the pivot search, the pivot-column copy and
// the deterministic-outcome scan read other lanes' columns and are fenced
// with __syncwarp.
#pragma once
#include "common.cuh"

namespace sdim {

// Arithmetic modulo d and the phase order; DD > 0 fixes d at compile time.
template <int DD>
struct ModU8 {
  int d, ord, phi;
  uint32_t mu_d, mu_ord;
  __device__ explicit ModU8(int dim) {
    d = DD ? DD : dim;
    ord = (d == 2) ? 4 : d;     // dataclasses.py:88-96
    phi = (d == 2) ? 2 : 1;     // dataclasses.py:98-106
    mu_d = 0xffffffffu / (uint32_t)d + 1u;
    mu_ord = 0xffffffffu / (uint32_t)ord + 1u;
  }
  // x in [0, 2^24)
  __device__ __forceinline__ int md(int x) const {
    if constexpr (DD > 0) return x % DD;
    else return x - (int)__umulhi((uint32_t)x, mu_d) * d;
  }
  __device__ __forceinline__ int mo(int x) const {
    if constexpr (DD > 0) return x % (DD == 2 ? 4 : DD);
    else return x - (int)__umulhi((uint32_t)x, mu_ord) * ord;
  }
  __device__ __forceinline__ int neg(int x) const { return x ? d - x : 0; }
  // dd + f (f - 1) / 2 x z, the term of one generator in the deterministic
  // outcome's sum_i f_i (f_i - 1) / 2 (x_i . z_i): plain sums for d <= 7
  // (at most 15 * 36 per term, so rows of thousands of terms stay far inside
  // an int), reduced mod d otherwise
  __device__ __forceinline__ int half_xz(int dd, int f, int x, int z) const {
    const int h = (f * (f - 1)) >> 1;
    if constexpr (DD > 0 && DD <= 7) return dd + h * x * z;
    else return md(dd + md(h) * x * z);
  }
  __device__ __forceinline__ int inv(int x) const {  // d prime, 0 < x < d
    int r = 1, b = x, e = d - 2;
    while (e > 0) {
      if (e & 1) r = md(r * b);
      b = md(b * b);
      e >>= 1;
    }
    return r;
  }
};

struct SlotU8 {
  int n, S, NP;
  __host__ __device__ static int stride(int n) {
    int s = (2 * n + 3) & ~3;
    if (((s >> 2) & 1) == 0) s += 4;
    return s;
  }
  __host__ __device__ static int npad(int n) { return (n + 15) & ~15; }
  __host__ __device__ static size_t bytes(int n) {
    const int s = stride(n);
    return (size_t)(2 * n + 1) * s + 2 * (size_t)npad(n);
  }
};

template <int DD>
struct EngineU8 {
  static constexpr int kBackend = 0;
  uint8_t* X;
  uint8_t* Z;
  uint8_t* PH;
  uint8_t* CX;
  uint8_t* CZ;
  int n, S;
  ModU8<DD> M;

  __device__ EngineU8(uint8_t* slot, int n_, int d) : n(n_), M(d) {
    S = SlotU8::stride(n_);
    X = slot;
    Z = X + (size_t)n * S;
    PH = Z + (size_t)n * S;
    CX = PH + S;
    CZ = CX + SlotU8::npad(n_);
  }

  static __host__ __device__ size_t slot_bytes(int n) { return SlotU8::bytes(n); }

  // z = I, x = 0, destab_x = I, destab_z = 0, phases 0
  __device__ void init(int lane) {
    uint32_t* w = reinterpret_cast<uint32_t*>(X);
    const int words = ((2 * n + 1) * S) >> 2;
    for (int i = lane; i < words; i += 32) w[i] = 0u;
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
      Z[(size_t)k * S + k] = 1;
      X[(size_t)k * S + n + k] = 1;
    }
    __syncwarp();
  }

  // ---------------- Clifford gates (owned columns only) ----------------
  // H: x' = -z, z' = x, ph += phi x' z'   (tableau_optimized.py:5-30)
  __device__ __forceinline__ void h(int lane, int q) {
    uint8_t* xr = X + (size_t)q * S;
    uint8_t* zr = Z + (size_t)q * S;
    for (int g = lane; g < 2 * n; g += 32) {
      const int x = xr[g], z = zr[g];
      const int nx = M.neg(z);
      PH[g] = (uint8_t)M.mo(PH[g] + M.phi * nx * x);
      xr[g] = (uint8_t)nx;
      zr[g] = (uint8_t)x;
    }
  }
  // H_INV: x' = z, z' = -x   (tableau_optimized.py:33-58)
  __device__ __forceinline__ void h_inv(int lane, int q) {
    uint8_t* xr = X + (size_t)q * S;
    uint8_t* zr = Z + (size_t)q * S;
    for (int g = lane; g < 2 * n; g += 32) {
      const int x = xr[g], z = zr[g];
      const int nz = M.neg(x);
      PH[g] = (uint8_t)M.mo(PH[g] + M.phi * z * nz);
      xr[g] = (uint8_t)z;
      zr[g] = (uint8_t)nz;
    }
  }
  // P: ph += x^2 (even d) or x(x-1)/2 (odd d); z += x; P_INV subtracts
  // (tableau_optimized.py:62-96)
  __device__ __forceinline__ void p(int lane, int q, bool inverse) {
    const uint8_t* xr = X + (size_t)q * S;
    uint8_t* zr = Z + (size_t)q * S;
    for (int g = lane; g < 2 * n; g += 32) {
      const int x = xr[g];
      const int t = M.mo((M.d == 2) ? x * x : (x * (x - 1)) >> 1);
      if (!inverse) {
        PH[g] = (uint8_t)M.mo(PH[g] + t);
        zr[g] = (uint8_t)M.md(zr[g] + x);
      } else {
        PH[g] = (uint8_t)M.mo(PH[g] + M.ord - t);
        zr[g] = (uint8_t)M.md(zr[g] + M.d - x);
      }
    }
  }
  // CNOT: x_t += x_c, z_c += (d-1) z_t; no phase (tableau_optimized.py:99-118).
  // All four inputs are read before either store, so c == t behaves as the
  // reference's in-place loop does (x doubled, z cleared).
  __device__ __forceinline__ void cnot(int lane, int c, int t, bool inverse) {
    uint8_t* xc = X + (size_t)c * S;
    uint8_t* xt = X + (size_t)t * S;
    uint8_t* zc = Z + (size_t)c * S;
    uint8_t* zt = Z + (size_t)t * S;
    for (int g = lane; g < 2 * n; g += 32) {
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
  // Phase-only Paulis: ph += phi * (cz * z_q + cx * x_q) with coefficients in
  // [0, d).  X = (-1, 0), X_INV = (1, 0), Z = (0, 1), Z_INV = (0, -1): the
  // closed forms of the reference's H/P compositions
  // (sdim/tableau/tableau_gates.py:27-137).
  __device__ __forceinline__ void pauli(int lane, int q, int cz, int cx) {
    const uint8_t* xr = X + (size_t)q * S;
    const uint8_t* zr = Z + (size_t)q * S;
    for (int g = lane; g < 2 * n; g += 32) {
      PH[g] = (uint8_t)M.mo(PH[g] + M.phi * (cz * zr[g] + cx * xr[g]));
    }
  }

  // ---------------- Z measurement (tableau_prime.py:262-363) ----------------
  // Returns the outcome; *det receives the deterministic flag.
  __device__ int measure(int lane, int q, unsigned long long seed, long long shot,
                         uint32_t ordinal, int* det) {
    __syncwarp();
    const uint8_t* xq = X + (size_t)q * S;
    // pivot: lowest stabilizer with x_q != 0
    int mine = 0x7fffffff;
    for (int g = lane; g < n; g += 32) {
      if (xq[g]) { mine = g; break; }
    }
    const int p = __reduce_min_sync(0xffffffffu, mine);
    if (p < n) {
      const int xv = xq[p];
      if (xv != 1) {
        // exponentiate(p, xv^-1) (tableau_prime.py:365-380)
        const int e = M.inv(xv);
        int sl = 0;
        for (int k = lane; k < n; k += 32) sl += X[(size_t)k * S + p] * Z[(size_t)k * S + p];
        const int s = M.md(__reduce_add_sync(0xffffffffu, sl));
        __syncwarp();
        if (lane == (p & 31)) {
          const int half = M.md(s * M.md((e * (e - 1)) >> 1));
          PH[p] = (uint8_t)M.mo(PH[p] * e + half * M.phi);
        }
        for (int k = lane; k < n; k += 32) {
          X[(size_t)k * S + p] = (uint8_t)M.md(X[(size_t)k * S + p] * e);
          Z[(size_t)k * S + p] = (uint8_t)M.md(Z[(size_t)k * S + p] * e);
        }
        __syncwarp();
      }
      // pivot column -> scratch
      int sl = 0;
      for (int k = lane; k < n; k += 32) {
        const int a = X[(size_t)k * S + p], b = Z[(size_t)k * S + p];
        CX[k] = (uint8_t)a;
        CZ[k] = (uint8_t)b;
        sl += a * b;
      }
      const int s = M.md(__reduce_add_sync(0xffffffffu, sl));
      const int php = PH[p];
      __syncwarp();
      // column-parallel rowsum: every generator g != stab p with x_q[g] != 0
      // absorbs f = -x_q[g] copies of the pivot (tableau_prime.py:308-322)
      for (int g = lane; g < 2 * n; g += 32) {
        const int f = (g == p) ? 0 : M.neg(xq[g]);
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
        const int half = M.md(s * ((f * (f - 1)) >> 1));
        const int cp = M.phi * M.md(f * M.md(dot)) + M.phi * M.phi * half;
        PH[g] = (uint8_t)M.mo(PH[g] + php * f + cp);
      }
      __syncwarp();
      // destabilizer p <- stabilizer p; stabilizer p <- Z_q with phase -m phi
      const uint4 w = stream_block(seed, shot, ordinal, 0u);
      const int m = mulshift(w.x, (uint32_t)M.d);
      for (int k = lane; k < n; k += 32) {
        X[(size_t)k * S + n + p] = CX[k];
        Z[(size_t)k * S + n + p] = CZ[k];
        X[(size_t)k * S + p] = 0;
        Z[(size_t)k * S + p] = (uint8_t)(k == q);
      }
      if (lane == 0) {
        PH[n + p] = (uint8_t)php;
        PH[p] = (uint8_t)M.mo(M.ord - M.mo(m * M.phi));
      }
      __syncwarp();
      *det = 0;
      return m;
    }
    // deterministic: ancilla accumulation (tableau_prime.py:336-363)
    //   aph = sum_i f_i ph_i + phi * sum_k sum_i f_i x_i[k] (sum_{j<i} f_j z_j[k])
    //         + phi^2 * sum_i (x_i . z_i) f_i (f_i - 1) / 2,   f_i = destab_x[q][i]
    for (int i = lane; i < n; i += 32) CX[i] = xq[n + i];
    __syncwarp();
    // sum_i f_i ph_i here; the f_i (f_i - 1) / 2 (x_i . z_i) term is summed
    // row by row in the cross-term pass below (one pass over the tableau)
    int pl = 0, dl = 0;
    for (int i = lane; i < n; i += 32) {
      const int f = CX[i];
      if (f) pl += f * PH[i];
    }
    int tl = 0;
    for (int k = lane; k < n; k += 32) {
      const uint8_t* xr = X + (size_t)k * S;
      const uint8_t* zr = Z + (size_t)k * S;
      int pre = 0, acc = 0, dd = 0;
      for (int i = 0; i < n; ++i) {
        const int f = CX[i];
        if (f) {
          const int xv = xr[i], zv = zr[i];
          acc = M.md(acc + f * xv * pre);
          pre = M.md(pre + f * zv);
          dd = M.half_xz(dd, f, xv, zv);
        }
      }
      tl += acc;
      dl += M.md(dd);
    }
    const int P = M.mo(__reduce_add_sync(0xffffffffu, pl));
    const int T = M.md(__reduce_add_sync(0xffffffffu, tl));
    const int D = M.md(__reduce_add_sync(0xffffffffu, dl));
    const int aph = M.mo(P + M.phi * T + M.phi * M.phi * D);
    __syncwarp();
    *det = 1;
    if (M.phi == 1) return M.md(M.d - aph);
    return ((aph + 1) >> 1) & 1;  // floor(-aph / 2) mod 2 for d = 2
  }

  // RESET correction: X applied k = -m mod d times, ph -= k phi z_q
  __device__ __forceinline__ void reset_fix(int lane, int q, int m) {
    const int k = M.md(M.d - m);
    if (k) pauli(lane, q, M.d - k, 0);
    __syncwarp();
  }

  // ---------------- export in the reference's int8 block order ----------------
  // x[n][n], z[n][n], ph[n], dx[n][n], dz[n][n], dph[n]
  __device__ void export_tableau(int lane, int8_t* dst) {
    __syncwarp();
    const size_t nn = (size_t)n * n;
    for (size_t e = lane; e < nn; e += 32) {
      const int k = (int)(e / n), i = (int)(e % n);
      dst[e] = (int8_t)X[(size_t)k * S + i];
      dst[nn + e] = (int8_t)Z[(size_t)k * S + i];
      dst[2 * nn + n + e] = (int8_t)X[(size_t)k * S + n + i];
      dst[3 * nn + n + e] = (int8_t)Z[(size_t)k * S + n + i];
    }
    for (int i = lane; i < n; i += 32) {
      dst[2 * nn + i] = (int8_t)PH[i];
      dst[4 * nn + n + i] = (int8_t)PH[n + i];
    }
    __syncwarp();
  }
};

}  // namespace sdim
