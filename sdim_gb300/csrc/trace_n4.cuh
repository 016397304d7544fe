// x / z pass of the trace engine for d = 5 and 7 with the tableau in 4-bit
// residue lanes (nibbles.cuh): 8 generators per 32-bit word, half the bytes
// of one residue per byte, so one CTA holds n <= 320 in shared memory on
// GB300 (the n = 256 workloads fit one SM instead of a CTA cluster) and a
// streamed tableau moves half the traffic.
//
// Layout.  Row k of X (of Z) is W = 2 Wh words, Wh = ceil(n / 8):
// stabilizer g < n in word g / 8, lane g % 8; destabilizer n + i in word
// Wh + i / 8, lane i % 8; lanes past n in each half stay 0.  Rows are RS =
// W | 1 words apart.  The common phase C has the same word layout.
//
// Same algorithm, trace and work split as the d = 3 bit-plane pass
// (trace_p3.cuh): the reference's ExtendedTableau updates mod d
// (sdim/tableau/tableau_prime.py:97-380) with phi = 1, written as the same
// trace the byte-residue passes write.  The rank-1 update adds a precomputed
// multiple c * FW of the factor row to each row, and the column dots
// Z^T x_p are summed as sum_c c (sum of the rows with x_p = c).
#pragma once
#include <climits>

#include "nibbles.cuh"
#include "team.cuh"
#include "trace.cuh"
#include "trace_u8.cuh"

namespace sdim {

// Threads of a CTA of the pass: up to 512 in batches (two CTAs per SM), 1024
// for a lone program (its rank-1 update spread over more row groups).
constexpr int kN4Threads = 512;
constexpr int kN4WideThreads = 1024;

template <int DD>
struct N4Layout {
  int n, Wh, W, RS, np;
  __host__ __device__ explicit N4Layout(int n_) : n(n_) {
    Wh = (n_ + 7) >> 3;
    W = 2 * Wh;
    RS = W | 1;
    np = (n_ + 15) & ~15;
  }
  __host__ __device__ size_t xz_bytes() const { return (size_t)2 * n * RS * 4; }
  // C, FW, DOT (W words each), F, H (Wh each), the multiples c * FW
  // (d - 1 rows of W words), the row-group partial sums ((d - 1) x threads
  // words for a CTA of `threads`), CX and CZ (np bytes each)
  __host__ __device__ size_t hot_bytes(int threads) const {
    return (size_t)(3 * W + 2 * Wh + (DD - 1) * W + (DD - 1) * threads) * 4 + 2 * (size_t)np;
  }
};

template <int DD>
struct TabN4 {
  using M = N4<DD>;
  CtaTeam tm;
  N4Layout<DD> L;
  uint32_t *X, *Z, *C, *FW, *DOT, *F, *H, *FWC, *part;
  uint8_t *CX, *CZ;
  int pcap;  // row-group partial sums per pivot value: the CTA's threads

  __device__ TabN4(uint8_t* xz, uint8_t* hot, int n, CtaTeam team, int threads)
      : tm(team), L(n), pcap(threads) {
    X = reinterpret_cast<uint32_t*>(xz);
    Z = X + (size_t)n * L.RS;
    C = reinterpret_cast<uint32_t*>(hot);
    FW = C + L.W;
    DOT = FW + L.W;
    F = DOT + L.W;
    H = F + L.Wh;
    FWC = H + L.Wh;              // FWC[(c - 1) W + w] = c * FW[w]
    part = FWC + (DD - 1) * L.W;  // part[(c - 1) pcap + r W + w]
    CX = reinterpret_cast<uint8_t*>(part + (DD - 1) * pcap);
    CZ = CX + L.np;
  }

  // generator of lane j of word w, or -1 for a padding lane
  __device__ __forceinline__ int gen_of(int w, int j) const {
    const int i = (w < L.Wh ? w : w - L.Wh) * 8 + j;
    return i < L.n ? (w < L.Wh ? i : L.n + i) : -1;
  }

  __device__ void init() {
    const int t = tm.t, size = tm.size();
    for (size_t i = t; i < (size_t)2 * L.n * L.RS; i += size) X[i] = 0u;
    for (int w = t; w < L.W; w += size) C[w] = 0u;
    tm.sync();
    for (int k = t; k < L.n; k += size) {
      uint32_t* z = Z + (size_t)k * L.RS + (k >> 3);
      *z = M::set(*z, k & 7, 1);                   // stabilizer k = Z_k
      uint32_t* x = X + (size_t)k * L.RS + L.Wh + (k >> 3);
      *x = M::set(*x, k & 7, 1);                   // destabilizer k = X_k
    }
    tm.sync();
  }

  // ---------------- gates: thread w owns word w of every row ----------------
  __device__ __forceinline__ void h(int q, bool inverse) {
    uint32_t* xr = X + (size_t)q * L.RS;
    uint32_t* zr = Z + (size_t)q * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) {
      const uint32_t x = xr[w], z = zr[w];
      if (!inverse) {  // x' = -z, z' = x, c += x' x
        const uint32_t nx = M::neg(z);
        C[w] = M::add(C[w], M::mul(nx, x));
        xr[w] = nx;
        zr[w] = x;
      } else {         // x' = z, z' = -x, c += z z'
        const uint32_t nz = M::neg(x);
        C[w] = M::add(C[w], M::mul(z, nz));
        xr[w] = z;
        zr[w] = nz;
      }
    }
  }
  __device__ __forceinline__ void p(int q, bool inverse) {
    const uint32_t* xr = X + (size_t)q * L.RS;
    uint32_t* zr = Z + (size_t)q * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) {
      const uint32_t x = xr[w], t = M::half(x);
      if (!inverse) {
        C[w] = M::add(C[w], t);
        zr[w] = M::add(zr[w], x);
      } else {
        C[w] = M::sub(C[w], t);
        zr[w] = M::sub(zr[w], x);
      }
    }
  }
  __device__ __forceinline__ void cnot(int c, int tq, bool inverse) {
    uint32_t* xc = X + (size_t)c * L.RS;
    uint32_t* xt = X + (size_t)tq * L.RS;
    uint32_t* zc = Z + (size_t)c * L.RS;
    uint32_t* zt = Z + (size_t)tq * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) {
      const uint32_t a = xc[w], f = zt[w];
      if (!inverse) {  // x_t += x_c, z_c -= z_t
        xt[w] = M::add(xt[w], a);
        zc[w] = M::sub(zc[w], f);
      } else {
        xt[w] = M::sub(xt[w], a);
        zc[w] = M::add(zc[w], f);
      }
    }
  }
  // c += cz z_q + cx x_q
  __device__ __forceinline__ void pauli(int q, int cz, int cx) {
    const uint32_t* xr = X + (size_t)q * L.RS;
    const uint32_t* zr = Z + (size_t)q * L.RS;
    for (int w = tm.t; w < L.W; w += tm.size()) C[w] = M::add(C[w], M::add(M::mulc(zr[w], cz), M::mulc(xr[w], cx)));
  }

  // Byte residues of a row (both halves, limit = 2n, or the stabilizer half
  // read from words [w0, w0 + Wh), limit = n) into dst[0, sw), zero past the
  // limit.  Thread w writes the lanes of word w.
  __device__ void row_bytes(const uint32_t* row, int w0, int limit, uint8_t* dst, int sw) const {
    const int t = tm.t, size = tm.size();
    const int words = limit > L.n ? L.W : L.Wh;
    for (int w = t; w < words; w += size) {
      const uint32_t v = row[w0 + w];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int g = limit > L.n ? gen_of(w, j) : (w * 8 + j < L.n ? w * 8 + j : -1);
        if (g >= 0) dst[g] = (uint8_t)M::get(v, j);
      }
    }
    for (int g = limit + t; g < sw; g += size) dst[g] = 0;
  }
};

// x^-1 mod d for 0 < x < d
template <int DD>
__device__ __forceinline__ int n4_inv(int x) {
  int r = 1;
  for (int k = 0; k < DD - 2; ++k) r = (r * x) % DD;
  return r;
}

// One Z measurement of qudit q on the nibble tableau; writes trace record mord.
template <int DD>
__device__ void trace_measure_n4(TabN4<DD>& e, const TraceDescU8& td, int q, uint32_t mord, uint32_t nord,
                                 bool reset) {
  using M = N4<DD>;
  e.tm.sync();
  const int size = e.tm.size(), t = e.tm.t;
  const N4Layout<DD>& L = e.L;
  const int n = L.n, RS = L.RS, sw = td.sw;
  uint32_t* X = e.X;
  uint32_t* Z = e.Z;
  uint32_t* C = e.C;
  const uint32_t* xq = X + (size_t)q * RS;
  uint8_t* row = td.mrow + (size_t)mord * 2 * sw;
  int mine = INT_MAX;
  for (int w = t; w < L.Wh; w += size) {
    const uint32_t nz = M::nz(xq[w]);
    if (nz) {
      mine = w * 8 + ((__ffs(nz) - 1) >> 2);
      break;
    }
  }
  const int p = e.tm.min(mine);
  if (p < n) {
    const int wp = p >> 3, lp = p & 7;
    const int wn = L.Wh + wp;  // destabilizer n + p: same lane, other half
    const int xv = M::get(xq[wp], lp);
    const int ex = xv == 1 ? 1 : n4_inv<DD>(xv);
    if (ex != 1) {
      // exponentiate (tableau_prime.py:365-380): column p times e,
      // c_p = c_p e + s0 e (e - 1) / 2
      int sl = 0;
      for (int k = t; k < n; k += size) sl += M::get(X[(size_t)k * RS + wp], lp) * M::get(Z[(size_t)k * RS + wp], lp);
      const int s0 = e.tm.add(sl) % DD;
      e.tm.sync();
      if (e.tm.leader())
        C[wp] = M::set(C[wp], lp, (M::get(C[wp], lp) * ex + s0 * (((ex * (ex - 1)) >> 1) % DD)) % DD);
      for (int k = t; k < n; k += size) {
        uint32_t* xk = X + (size_t)k * RS + wp;
        uint32_t* zk = Z + (size_t)k * RS + wp;
        *xk = M::set(*xk, lp, (M::get(*xk, lp) * ex) % DD);
        *zk = M::set(*zk, lp, (M::get(*zk, lp) * ex) % DD);
      }
      e.tm.sync();
    }
    int sl = 0;
    for (int k = t; k < n; k += size) {
      const int a = M::get(X[(size_t)k * RS + wp], lp), b = M::get(Z[(size_t)k * RS + wp], lp);
      e.CX[k] = (uint8_t)a;
      e.CZ[k] = (uint8_t)b;
      sl += a * b;
    }
    for (int w = t; w < L.W; w += size) {
      uint32_t f = M::neg(xq[w]);
      if (w == wp) f = M::set(f, lp, 0);
      e.FW[w] = f;
      const uint32_t f2 = M::add(f, f);
      e.FWC[w] = f;
      e.FWC[L.W + w] = f2;
      uint32_t fc = f2;
#pragma unroll
      for (int c = 3; c < DD; ++c) {
        fc = M::add(fc, f);
        e.FWC[(c - 1) * L.W + w] = fc;
      }
    }
    const int s1 = e.tm.add(sl) % DD;
    const int phc = M::get(C[wp], lp);
    e.tm.sync();
    e.row_bytes(e.FW, 0, 2 * n, row, sw);
    // rank-1 update of X and Z, (word, row group) threads; row-group sums of
    // the old Z rows per pivot value c for the column dots
    const int W = L.W, R = max(1, min(min(size, e.pcap) / W, (n + 3) >> 2));
    if (t < R * W) {
      const int w = t % W, r = t / W;
      uint32_t acc[DD - 1];
#pragma unroll
      for (int c = 0; c < DD - 1; ++c) acc[c] = 0u;
      if (e.FW[w]) {
        int k = r;
        for (; k + 3 * R < n; k += 4 * R) {  // four rows in flight
          uint32_t xw[4], zw[4];
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
              X[(size_t)(k + i * R) * RS + w] = M::add(xw[i], e.FWC[(a[i] - 1) * W + w]);
#pragma unroll
              for (int c = 1; c < DD; ++c)
                if (a[i] == c) acc[c - 1] = M::add(acc[c - 1], zw[i]);
            }
            if (b[i]) Z[(size_t)(k + i * R) * RS + w] = M::add(zw[i], e.FWC[(b[i] - 1) * W + w]);
          }
        }
        for (; k < n; k += R) {
          const uint32_t xw = X[(size_t)k * RS + w], zw = Z[(size_t)k * RS + w];
          const int a = e.CX[k], b = e.CZ[k];
          if (a) {
            X[(size_t)k * RS + w] = M::add(xw, e.FWC[(a - 1) * W + w]);
#pragma unroll
            for (int c = 1; c < DD; ++c)
              if (a == c) acc[c - 1] = M::add(acc[c - 1], zw);
          }
          if (b) Z[(size_t)k * RS + w] = M::add(zw, e.FWC[(b - 1) * W + w]);
        }
      }
#pragma unroll
      for (int c = 0; c < DD - 1; ++c) e.part[c * e.pcap + r * W + w] = acc[c];
    }
    e.tm.sync();
    // phases of the absorbing generators: c += phc f + f DOT + s1 f (f - 1) / 2
    for (int w = t; w < W; w += size) {
      const uint32_t f = e.FW[w];
      if (!f) continue;
      uint32_t dot = 0u;
#pragma unroll
      for (int c = 1; c < DD; ++c) {
        uint32_t sc = 0u;
        for (int r = 0; r < R; ++r) sc = M::add(sc, e.part[(c - 1) * e.pcap + r * W + w]);
        dot = M::add(dot, M::mulc(sc, c));
      }
      C[w] = M::add(C[w], M::add(M::mulc(f, phc), M::add(M::mul(f, dot), M::mulc(M::half(f), s1))));
    }
    e.tm.sync();
    // pivot columns: destabilizer p <- stabilizer p, stabilizer p <- Z_q
    for (int k = t; k < n; k += size) {
      uint32_t* xr = X + (size_t)k * RS;
      uint32_t* zr = Z + (size_t)k * RS;
      xr[wn] = M::set(xr[wn], lp, e.CX[k]);
      zr[wn] = M::set(zr[wn], lp, e.CZ[k]);
      xr[wp] = M::set(xr[wp], lp, 0);
      zr[wp] = M::set(zr[wp], lp, k == q ? 1 : 0);
    }
    if (e.tm.leader()) {
      C[wn] = M::set(C[wn], lp, phc);
      C[wp] = M::set(C[wp], lp, 0);
      td.mhdr[mord] = make_uint4((reset ? 2u : 0u) | ((uint32_t)ex << 8), (uint32_t)p, nord, 0u);
    }
    e.tm.sync();
  } else {
    // deterministic (tableau_prime.py:336-363): f_i = destabilizer x_q[n + i]
    for (int w = t; w < L.Wh; w += size) {
      const uint32_t f = xq[L.Wh + w];
      e.F[w] = f;
      e.H[w] = M::half(f);
    }
    e.tm.sync();
    int pl = 0;
    for (int w = t; w < L.Wh; w += size) pl += M::rsum(M::mul(e.F[w], C[w]));
    int tl = 0, dl = 0;
    for (int k = t; k < n; k += size) {
      const uint32_t* xr = X + (size_t)k * RS;
      const uint32_t* zr = Z + (size_t)k * RS;
      int pre = 0, acc = 0, dd = 0;
      for (int w = 0; w < L.Wh; ++w) {
        const uint32_t fw = e.F[w];
        if (!fw) continue;
        const uint32_t xw = xr[w], zw = zr[w], hw = e.H[w];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int f = M::get(fw, j);
          if (f) {
            const int xv = M::get(xw, j), zv = M::get(zw, j);
            acc = (acc + f * xv * pre) % DD;
            pre = (pre + f * zv) % DD;
            dd += M::get(hw, j) * xv * zv;
          }
        }
      }
      tl += acc;
      dl += dd % DD;
    }
    e.row_bytes(xq, L.Wh, n, row, sw);
    e.tm.add3(pl, tl, dl);
    const int P = pl % DD;
    const int T = tl % DD;
    const int Dd = dl % DD;
    const int aphc = (P + T + Dd) % DD;
    if (e.tm.leader()) td.mhdr[mord] = make_uint4(reset ? 3u : 1u, 0u, nord, (uint32_t)aphc);
    e.tm.sync();
  }
  if (reset) {
    e.row_bytes(Z + (size_t)q * RS, 0, 2 * n, row + sw, sw);
    e.tm.sync();
  }
}

// Runs the shared part of td's program (d = 5 or 7) on the nibble tableau
// and writes its trace; win: room for kOpWindow instructions in shared memory.
template <int DD>
__device__ void trace_program_n4(const TraceDescU8& td, TabN4<DD>& e, uint2* win, int* status) {
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
      case OP_X: e.pauli(q, DD - 1, 0); break;
      case OP_X_INV: e.pauli(q, 1, 0); break;
      case OP_Z: e.pauli(q, 0, 1); break;
      case OP_Z_INV: e.pauli(q, 0, DD - 1); break;
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
        trace_measure_n4(e, td, q, mord, nord, op == OP_RESET);
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
