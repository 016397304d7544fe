// x / z pass of the trace engine for d = 3 with the tableau in two bit
// planes (planes3.cuh): 32 generators per pair of words, a quarter of the
// bytes of one residue per byte, so one CTA holds n <= 448 in shared memory
// and a streamed tableau moves a quarter of the traffic.
//
// Layout.  Row k of X (of Z) is W = 2 Wh plane pairs, Wh = ceil(n / 32):
// stabilizer g < n in word g / 32, lane g % 32; destabilizer n + i in word
// Wh + i / 32, lane i % 32; lanes past n in each half stay 0.  Rows are RS =
// W | 1 pairs apart (an odd stride keeps a warp that walks 32 rows at the
// same word on distinct banks).  The common phase C has the same word layout.
//
// The pass computes exactly what the byte-residue pass (trace_u8.cuh)
// computes -- the reference's ExtendedTableau updates mod 3
// (sdim/tableau/tableau_prime.py:97-380) with phi = 1 -- and writes the same
// trace (mhdr, byte rows mrow / nrow, nhdr), so the phase pass of the odd-d
// trace engine replays it unchanged.
//
// Work split.  Gates and N1 rows: thread w owns word w of every row, so a run
// of gates needs no barrier.  Rank-1 update of a random measurement: threads
// are (word w, row group r) pairs; each adds a multiple of the factor row to
// its rows and sums its share of the column dots Z^T x_p, which the row
// groups then add up.  Deterministic outcome: one thread per row walks its
// stabilizer words with prefix sums inside each word (p3_det_word).
#pragma once
#include <climits>

#include "planes3.cuh"
#include "team.cuh"
#include "trace.cuh"
#include "trace_u8.cuh"

namespace sdim {

// Threads of a CTA of the pass: up to 512 in batches (two CTAs per SM), 1024
// for a lone program (its rank-1 update spread over more row groups).
constexpr int kP3Threads = 512;
constexpr int kP3WideThreads = 1024;

struct P3Layout {
  int n, Wh, W, RS, np;
  __host__ __device__ explicit P3Layout(int n_) : n(n_) {
    Wh = (n_ + 31) >> 5;
    W = 2 * Wh;
    RS = W | 1;
    np = (n_ + 15) & ~15;
  }
  // bytes of X and Z
  __host__ __device__ size_t xz_bytes() const { return (size_t)2 * n * RS * sizeof(P3); }
  // bytes of C, FW, DOT (W pairs each), F, H (Wh each), the row-group partial
  // dots (one pair per thread of a CTA of `threads`), CX and CZ (np bytes each)
  __host__ __device__ size_t hot_bytes(int threads) const {
    return (size_t)(3 * W + 2 * Wh + threads) * sizeof(P3) + 2 * (size_t)np;
  }
};

struct TabP3 {
  CtaTeam tm;
  P3Layout L;
  P3 *X, *Z, *C, *FW, *DOT, *F, *H, *part;
  uint8_t *CX, *CZ;
  int pcap;  // row-group partial dots: the CTA's threads

  __device__ TabP3(uint8_t* xz, uint8_t* hot, int n, CtaTeam team, int threads)
      : tm(team), L(n), pcap(threads) {
    X = reinterpret_cast<P3*>(xz);
    Z = X + (size_t)n * L.RS;
    C = reinterpret_cast<P3*>(hot);
    FW = C + L.W;
    DOT = FW + L.W;
    F = DOT + L.W;
    H = F + L.Wh;
    part = H + L.Wh;
    CX = reinterpret_cast<uint8_t*>(part + pcap);
    CZ = CX + L.np;
  }

  // word and lane of generator g
  __device__ __forceinline__ int word_of(int g) const { return g < L.n ? g >> 5 : L.Wh + ((g - L.n) >> 5); }
  __device__ __forceinline__ int lane_of(int g) const { return g < L.n ? g & 31 : (g - L.n) & 31; }
  // generator of lane j of word w, or -1 for a padding lane
  __device__ __forceinline__ int gen_of(int w, int j) const {
    const int i = (w < L.Wh ? w : w - L.Wh) * 32 + j;
    return i < L.n ? (w < L.Wh ? i : L.n + i) : -1;
  }

  __device__ void init() {
    const int t = tm.t, size = tm.size();
    for (size_t i = t; i < (size_t)2 * L.n * L.RS; i += size) X[i] = p3_zero();
    for (int w = t; w < L.W; w += size) C[w] = p3_zero();
    tm.sync();
    for (int k = t; k < L.n; k += size) {
      P3* z = Z + (size_t)k * L.RS + (k >> 5);
      *z = p3_set(*z, k & 31, 1);                     // stabilizer k = Z_k
      P3* x = X + (size_t)k * L.RS + L.Wh + (k >> 5);
      *x = p3_set(*x, k & 31, 1);                     // destabilizer k = X_k
    }
    tm.sync();
  }

  // ---------------- gates: thread w owns word w of every row ----------------
  __device__ __forceinline__ void h(int q, bool inverse) {
    P3* xr = X + (size_t)q * L.RS;
    P3* zr = Z + (size_t)q * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) {
      const P3 x = xr[w], z = zr[w];
      if (!inverse) {  // x' = -z, z' = x, c += x' x
        const P3 nx = p3_neg(z);
        C[w] = p3_add(C[w], p3_mul(nx, x));
        xr[w] = nx;
        zr[w] = x;
      } else {         // x' = z, z' = -x, c += z z'
        const P3 nz = p3_neg(x);
        C[w] = p3_add(C[w], p3_mul(z, nz));
        xr[w] = z;
        zr[w] = nz;
      }
    }
  }
  __device__ __forceinline__ void p(int q, bool inverse) {
    const P3* xr = X + (size_t)q * L.RS;
    P3* zr = Z + (size_t)q * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) {
      const P3 x = xr[w], t = p3_half(x);  // x (x - 1) / 2
      if (!inverse) {
        C[w] = p3_add(C[w], t);
        zr[w] = p3_add(zr[w], x);
      } else {
        C[w] = p3_sub(C[w], t);
        zr[w] = p3_sub(zr[w], x);
      }
    }
  }
  __device__ __forceinline__ void cnot(int c, int tq, bool inverse) {
    P3* xc = X + (size_t)c * L.RS;
    P3* xt = X + (size_t)tq * L.RS;
    P3* zc = Z + (size_t)c * L.RS;
    P3* zt = Z + (size_t)tq * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) {
      const P3 a = xc[w], f = zt[w];
      if (!inverse) {  // x_t += x_c, z_c -= z_t
        xt[w] = p3_add(xt[w], a);
        zc[w] = p3_sub(zc[w], f);
      } else {
        xt[w] = p3_sub(xt[w], a);
        zc[w] = p3_add(zc[w], f);
      }
    }
  }
  // c += cz z_q + cx x_q
  __device__ __forceinline__ void pauli(int q, int cz, int cx) {
    const P3* xr = X + (size_t)q * L.RS;
    const P3* zr = Z + (size_t)q * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size())
      C[w] = p3_add(C[w], p3_add(p3_mulc(zr[w], cz), p3_mulc(xr[w], cx)));
  }

  // Byte residues of a plane row (generators of both halves, limit = 2n, or
  // the stabilizer half only, limit = n, read from words [w0, w0 + Wh)) into
  // dst[0, sw), zero past the limit.  Thread w writes the lanes of word w.
  __device__ void row_bytes(const P3* row, int w0, int limit, uint8_t* dst, int sw) const {
    const int t = tm.t, size = tm.size();
    const int words = limit > L.n ? L.W : L.Wh;
    for (int w = t; w < words; w += size) {
      const P3 v = row[w0 + w];
#pragma unroll 4
      for (int j = 0; j < 32; ++j) {
        const int g = limit > L.n ? gen_of(w, j) : (w * 32 + j < L.n ? w * 32 + j : -1);
        if (g >= 0) dst[g] = (uint8_t)p3_get(v, j);
      }
    }
    for (int g = limit + t; g < sw; g += size) dst[g] = 0;
  }
};

// One Z measurement of qudit q on the planes tableau; writes trace record mord.
__device__ void trace_measure_p3(TabP3& e, const TraceDescU8& td, int q, uint32_t mord, uint32_t nord, bool reset) {
  e.tm.sync();
  const int size = e.tm.size(), t = e.tm.t;
  const P3Layout& L = e.L;
  const int n = L.n, RS = L.RS, sw = td.sw;
  P3* X = e.X;
  P3* Z = e.Z;
  P3* C = e.C;
  const P3* xq = X + (size_t)q * RS;
  uint8_t* row = td.mrow + (size_t)mord * 2 * sw;
  int mine = INT_MAX;
  for (int w = t; w < L.Wh; w += size) {
    const uint32_t nz = p3_nz(xq[w]);
    if (nz) {
      mine = w * 32 + __ffs(nz) - 1;
      break;
    }
  }
  const int p = e.tm.min(mine);
  if (p < n) {
    const int wp = p >> 5, lp = p & 31;
    const int wn = L.Wh + wp;  // destabilizer n + p: same lane, other half
    const int xv = p3_get(xq[wp], lp);
    const int ex = xv == 1 ? 1 : 2;  // x_q[p]^-1 mod 3
    if (ex != 1) {
      // exponentiate (tableau_prime.py:365-380): column p times 2, c_p = 2 c_p + s0
      int sl = 0;
      for (int k = t; k < n; k += size)
        sl += p3_get(X[(size_t)k * RS + wp], lp) * p3_get(Z[(size_t)k * RS + wp], lp);
      const int s0 = e.tm.add(sl) % 3;
      e.tm.sync();
      if (e.tm.leader()) C[wp] = p3_set(C[wp], lp, (2 * p3_get(C[wp], lp) + s0) % 3);
      for (int k = t; k < n; k += size) {
        P3* xk = X + (size_t)k * RS + wp;
        P3* zk = Z + (size_t)k * RS + wp;
        *xk = p3_set(*xk, lp, (2 * p3_get(*xk, lp)) % 3);
        *zk = p3_set(*zk, lp, (2 * p3_get(*zk, lp)) % 3);
      }
      e.tm.sync();
    }
    int sl = 0;
    for (int k = t; k < n; k += size) {
      const int a = p3_get(X[(size_t)k * RS + wp], lp), b = p3_get(Z[(size_t)k * RS + wp], lp);
      e.CX[k] = (uint8_t)a;
      e.CZ[k] = (uint8_t)b;
      sl += a * b;
    }
    for (int w = t; w < L.W; w += size) {
      const P3 f = p3_neg(xq[w]);
      e.FW[w] = w == wp ? p3_and(f, ~(1u << lp)) : f;
    }
    const int s1 = e.tm.add(sl) % 3;
    const int phc = p3_get(C[wp], lp);
    e.tm.sync();
    e.row_bytes(e.FW, 0, 2 * n, row, sw);
    // rank-1 update of X and Z and the column dots, (word, row group) threads;
    // at least four rows per group, so that few partial dots are summed
    const int W = L.W, R = max(1, min(min(size, e.pcap) / W, (n + 3) >> 2));
    if (t < R * W) {
      const int w = t % W, r = t / W;
      const P3 f1 = e.FW[w], f2 = p3_neg(f1);
      P3 acc = p3_zero();
      if (p3_nz(f1)) {
        int k = r;
        for (; k + 3 * R < n; k += 4 * R) {  // four rows in flight
          P3 xw[4], zw[4];
          int a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            xw[i] = X[(size_t)(k + i * R) * RS + w];
            zw[i] = Z[(size_t)(k + i * R) * RS + w];
            a[i] = e.CX[k + i * R];
            b[i] = e.CZ[k + i * R];
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            if (a[i]) {
              X[(size_t)(k + i * R) * RS + w] = p3_add(xw[i], a[i] == 1 ? f1 : f2);
              acc = p3_add(acc, a[i] == 1 ? zw[i] : p3_neg(zw[i]));
            }
            if (b[i]) Z[(size_t)(k + i * R) * RS + w] = p3_add(zw[i], b[i] == 1 ? f1 : f2);
          }
        }
        for (; k < n; k += R) {
          const P3 xw = X[(size_t)k * RS + w], zw = Z[(size_t)k * RS + w];
          const int a = e.CX[k], b = e.CZ[k];
          if (a) {
            X[(size_t)k * RS + w] = p3_add(xw, a == 1 ? f1 : f2);
            acc = p3_add(acc, a == 1 ? zw : p3_neg(zw));
          }
          if (b) Z[(size_t)k * RS + w] = p3_add(zw, b == 1 ? f1 : f2);
        }
      }
      e.part[r * W + w] = acc;
    }
    e.tm.sync();
    // phases of the absorbing generators: c += phc f + f DOT + s1 f (f - 1) / 2
    for (int w = t; w < W; w += size) {
      const P3 f = e.FW[w];
      if (!p3_nz(f)) continue;
      P3 dot = p3_zero();
      for (int r = 0; r < R; ++r) dot = p3_add(dot, e.part[r * W + w]);
      C[w] = p3_add(C[w], p3_add(p3_mulc(f, phc), p3_add(p3_mul(f, dot), p3_mulc(p3_half(f), s1))));
    }
    e.tm.sync();
    // pivot columns: destabilizer p <- stabilizer p, stabilizer p <- Z_q
    for (int k = t; k < n; k += size) {
      P3* xr = X + (size_t)k * RS;
      P3* zr = Z + (size_t)k * RS;
      xr[wn] = p3_set(xr[wn], lp, e.CX[k]);
      zr[wn] = p3_set(zr[wn], lp, e.CZ[k]);
      xr[wp] = p3_set(xr[wp], lp, 0);
      zr[wp] = p3_set(zr[wp], lp, k == q ? 1 : 0);
    }
    if (e.tm.leader()) {
      C[wn] = p3_set(C[wn], lp, phc);
      C[wp] = p3_set(C[wp], lp, 0);
      td.mhdr[mord] = make_uint4((reset ? 2u : 0u) | ((uint32_t)ex << 8), (uint32_t)p, nord, 0u);
    }
    e.tm.sync();
  } else {
    // deterministic (tableau_prime.py:336-363): f_i = destabilizer x_q[n + i]
    for (int w = t; w < L.Wh; w += size) {
      const P3 f = xq[L.Wh + w];
      e.F[w] = f;
      e.H[w] = p3_half(f);
    }
    e.tm.sync();
    int pl = 0;
    for (int w = t; w < L.Wh; w += size) pl += p3_rsum(p3_mul(e.F[w], C[w]));
    int tl = 0, dl = 0;
    for (int k = t; k < n; k += size) {
      const P3* xr = X + (size_t)k * RS;
      const P3* zr = Z + (size_t)k * RS;
      int carry = 0, tk = 0, dk = 0;
      for (int w = 0; w < L.Wh; ++w) carry = p3_det_word(e.F[w], e.H[w], xr[w], zr[w], carry, tk, dk);
      tl += tk % 3;
      dl += dk % 3;
    }
    e.row_bytes(xq, L.Wh, n, row, sw);
    e.tm.add3(pl, tl, dl);
    const int P = pl % 3;
    const int T = tl % 3;
    const int Dd = dl % 3;
    const int aphc = (P + T + Dd) % 3;
    if (e.tm.leader()) td.mhdr[mord] = make_uint4(reset ? 3u : 1u, 0u, nord, (uint32_t)aphc);
    e.tm.sync();
  }
  if (reset) {
    e.row_bytes(Z + (size_t)q * RS, 0, 2 * n, row + sw, sw);
    e.tm.sync();
  }
}

// Runs the shared part of td's program (d = 3) on the planes tableau and
// writes its trace; win: room for kOpWindow instructions in shared memory.
__device__ void trace_program_p3(const TraceDescU8& td, TabP3& e, uint2* win, int* status) {
  const CircuitDesc& c = td.c;
  e.init();
  const int t = e.tm.t, size = e.tm.size();
  const int n = c.n, sw = td.sw;
  uint32_t mord = 0, nord = 0;
  for (int i = 0; i < c.nops; ++i) {
    if ((i & (kOpWindow - 1)) == 0) {  // stage the next window of instructions
      e.tm.sync();
      const int cnt = min(kOpWindow, c.nops - i);
      for (int j = t; j < cnt; j += size) win[j] = __ldg(c.ops + i + j);
      e.tm.sync();
    }
    const uint2 cur = win[i & (kOpWindow - 1)];
    const uint32_t op = cur.x & kOpMask;
    const int q = (int)(cur.x >> 8);
    if (q >= n) {
      if (t == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      return;
    }
    switch (op) {
      case OP_NOP: break;
      case OP_X: e.pauli(q, 2, 0); break;
      case OP_X_INV: e.pauli(q, 1, 0); break;
      case OP_Z: e.pauli(q, 0, 1); break;
      case OP_Z_INV: e.pauli(q, 0, 2); break;
      case OP_H: e.h(q, false); break;
      case OP_H_INV: e.h(q, true); break;
      case OP_P: e.p(q, false); break;
      case OP_P_INV: e.p(q, true); break;
      case OP_CNOT:
      case OP_CNOT_INV: {
        const int tq = (int)cur.y;
        if (tq >= n) {
          if (t == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
          return;
        }
        e.cnot(q, tq, op == OP_CNOT_INV);
        break;
      }
      case OP_M:
      case OP_RESET:
        if ((int)mord >= td.nm) {
          if (t == 0) atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
          return;
        }
        trace_measure_p3(e, td, q, mord, nord, op == OP_RESET);
        ++mord;
        break;
      case OP_N1D:
      case OP_N1F:
      case OP_N1P:
      case OP_N1OFF:
        if ((int)nord >= td.nn1) {
          if (t == 0) atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
          return;
        }
        if (t == 0) td.nhdr[nord] = make_uint2(op == OP_N1OFF ? 0xffffffffu : cur.y, op);
        if (op != OP_N1OFF) {
          // word w of row q was last written by thread w (or before a barrier)
          uint8_t* dst = td.nrow + (size_t)nord * 2 * sw;
          e.row_bytes(e.X + (size_t)q * e.L.RS, 0, 2 * n, dst, sw);
          e.row_bytes(e.Z + (size_t)q * e.L.RS, 0, 2 * n, dst + sw, sw);
        }
        ++nord;
        break;
      default:
        if (t == 0) atomicCAS(status, DEV_OK, DEV_BAD_OPCODE);
        return;
    }
  }
  e.tm.sync();
}

}  // namespace sdim
