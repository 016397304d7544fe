// x / z pass of the odd-d trace engine on a cluster of K CTAs (K =
// kTraceClusterCtas = 8): the generalisation of the CTA pair
// (trace_split_u8.cuh) that spreads the rank-1 update of a random
// measurement -- the bulk of the pass -- over K SMs.  Each CTA's columns live in its shared memory where they fit (n up to
// about 600) and otherwise in a slot of global memory; a cluster then streams
// 1 / K of one tableau, so the few programs in flight at a time stay in L2.
//
// Columns.  H = K / 2 CTAs hold the stabilizer columns and H the
// destabilizer columns, C = ceil(n / H) per CTA: CTA r < H holds stabilizers
// [r C, r C + nc), CTA H + c holds destabilizers n + [c C, c C + nc), each as
// X[n][SL], Z[n][SL] with its phases.  Gates act per column, so every CTA
// applies every gate to its own columns; thread j mod size owns column j.
//
// A measurement on qudit q takes one cluster barrier, whatever its outcome:
//   before it: every CTA's column owners store the negated row x_q of their
//     columns (the factors f), and a destabilizer CTA H + c also sends
//     stabilizer CTA c its slice of x_q (the factors of a deterministic
//     outcome).  Stabilizer CTA c finds its lowest column with x_q != 0 (its
//     candidate, one shared atomicMin and a CTA barrier) and sends every CTA
//     the candidate, x_q there, its phase and the whole candidate column
//     (x and z over the n rows) -- speculatively, since only the lowest
//     candidate of the cluster becomes the pivot;
//   after it: every CTA knows the pivot p (the lowest candidate) and holds
//     its column.  A random outcome runs the rank-1 update with the
//     unexponentiated column and the factors scaled by the exponent e
//     (x_k += (e f) cx_k is the update with the exponentiated column e cx),
//     the phases, and the pivot columns.  A deterministic one needs no
//     second cluster barrier (a stabilizer CTA takes a CTA barrier once its
//     rows are read): each stabilizer CTA writes its slice sums to global
//     memory -- P_c = sum f_i c_i, the in-slice cross term A_c and
//     D_c = sum f_i (f_i - 1) / 2 x_i.z_i as per-warp partials, and per row
//     k the slice sums Z_c[k] = sum f_i z_k[i], X_c[k] = sum f_i x_k[i] --
//     and the cluster's deterministic-header pass (k_cluster_det_headers)
//     adds the cross-slice term sum_k sum_{c' < c} Z_c'[k] X_c[k] and the
//     phase into the header after the x / z pass.
// Between measurements every write to X, Z and the phases comes from the
// column's owner or is followed by a CTA barrier, so a measurement starts
// without one.  Exchange buffers alternate by measurement parity: a CTA
// writes the buffer of measurement m + 2 only after the barrier of m + 1,
// which its partners pass only after they finished reading m's.  The
// arithmetic per column is that of group_u8.cuh and the trace written is the
// one of trace_u8.cuh.
#pragma once
#include "trace_split_u8.cuh"

namespace sdim {

__host__ __device__ inline int cluster_cols(int n, int K) { return (n + K / 2 - 1) / (K / 2); }

// Byte offsets inside one exchange buffer: per stabilizer slice c a slot
// (candidate, x_q there, its phase, 0) then its column x[np], z[np]; then the
// factors f[cpad] of this CTA's slice, then per factor word w the four words
// G_j (j = 0..3; byte i < j: f_i f_j, byte j: f_j (f_j - 1) / 2, of the
// word's four factors) with which a row's in-word sums are dot products.
struct ClusterXchg {
  int slot, f, g, total;
  __host__ __device__ ClusterXchg(int n, int K) {
    const int H = K / 2, np = SlotU8::npad(n), cpad = (cluster_cols(n, K) + 15) & ~15;
    slot = 16 + 2 * np;
    f = H * slot;
    g = f + cpad;
    total = g + 4 * cpad;
  }
};

// Shared memory of one CTA besides its columns: phases and factors (SL
// each), the dots (int[SL]), 16 bytes of ints (the candidates of two
// measurements, the pivot column's self-dot) and two exchange buffers.
__host__ __device__ inline size_t cluster_hot_bytes(int n, int K) {
  const size_t sl = (size_t)split_stride(cluster_cols(n, K));
  return round_up(2 * sl, 16) + 4 * sl + 16 + 2 * round_up((size_t)ClusterXchg(n, K).total, 16);
}

// The columns of one CTA: X and Z, n rows of SL bytes each.
__host__ __device__ inline size_t cluster_xz_bytes(int n, int K) {
  return round_up(2 * (size_t)n * (size_t)split_stride(cluster_cols(n, K)), 16);
}

// Global memory of one measurement's deterministic slice sums: per
// stabilizer slice Z_c[np] and X_c[np] (bytes), then (P, A, D) per warp.
__host__ __device__ inline size_t cluster_det_slice(int n) {
  return round_up(2 * (size_t)SlotU8::npad(n) + 12 * (size_t)(kTracePassThreads / 32), 16);
}
__host__ __device__ inline size_t cluster_det_bytes(int n, int K) { return (size_t)(K / 2) * cluster_det_slice(n); }

template <int DD, int K, bool kStream>
struct ClusterU8 {
  static constexpr int H = K / 2;
  CtaTeam tm;
  ModU8<DD> M;
  int r, c, stab;             // cluster rank, slice, 1 for a stabilizer CTA
  int n, nc, C0, g0, SL, np;  // local columns, columns per slice, first generator held
  uint8_t *X, *Z, *Cp, *FW;
  int* DOT;
  int* HS;      // candidates of the two exchange buffers, the pivot column's self-dot
  uint8_t* xb;  // two exchange buffers
  int xbytes;
  ClusterXchg L;

  // hot: this CTA's shared memory; xz: its columns (shared or global memory)
  __device__ ClusterU8(uint8_t* hot, uint8_t* xz, int n_, int d, int* red) : tm(red), M(d), n(n_), L(n_, K) {
    r = (int)cluster_rank();
    stab = r < H ? 1 : 0;
    c = r % H;
    C0 = cluster_cols(n_, K);
    nc = max(0, min(n_, (c + 1) * C0) - c * C0);
    g0 = (stab ? 0 : n_) + c * C0;
    SL = split_stride(C0);
    np = SlotU8::npad(n_);
    X = xz;
    Z = X + (size_t)n * SL;
    Cp = hot;
    FW = Cp + SL;
    DOT = reinterpret_cast<int*>(hot + round_up(2 * (size_t)SL, 16));
    HS = DOT + SL;
    xb = reinterpret_cast<uint8_t*>(HS + 4);
    xbytes = (int)round_up((size_t)L.total, 16);
  }
  __device__ uint8_t* buf(uint32_t mord) const { return xb + (size_t)(mord & 1u) * xbytes; }

  __device__ void init() {
    uint32_t* w = reinterpret_cast<uint32_t*>(X);
    const size_t words = (2 * (size_t)n * SL) >> 2;
    for (size_t i = tm.t; i < words; i += tm.size()) w[i] = 0u;
    for (int j = tm.t; j < 2 * SL; j += tm.size()) Cp[j] = 0;  // phases and factors
    if (tm.t < 2) HS[tm.t] = INT_MAX;
    tm.sync();
    // stabilizer g = Z_g, destabilizer n + g = X_g
    for (int j = tm.t; j < nc; j += tm.size()) (stab ? Z : X)[(size_t)(c * C0 + j) * SL + j] = 1;
    tm.sync();
  }

  // ---- gates on the local columns (column j owned by thread j mod size)
  __device__ __forceinline__ void h(int q) {
    uint8_t* xr = X + (size_t)q * SL;
    uint8_t* zr = Z + (size_t)q * SL;
    for (int j = tm.t; j < nc; j += tm.size()) {
      const int x = xr[j], z = zr[j];
      const int nx = M.neg(z);
      Cp[j] = (uint8_t)M.mo(Cp[j] + M.phi * nx * x);
      xr[j] = (uint8_t)nx;
      zr[j] = (uint8_t)x;
    }
  }
  __device__ __forceinline__ void h_inv(int q) {
    uint8_t* xr = X + (size_t)q * SL;
    uint8_t* zr = Z + (size_t)q * SL;
    for (int j = tm.t; j < nc; j += tm.size()) {
      const int x = xr[j], z = zr[j];
      const int nz = M.neg(x);
      Cp[j] = (uint8_t)M.mo(Cp[j] + M.phi * z * nz);
      xr[j] = (uint8_t)z;
      zr[j] = (uint8_t)nz;
    }
  }
  __device__ __forceinline__ void p(int q, bool inverse) {
    const uint8_t* xr = X + (size_t)q * SL;
    uint8_t* zr = Z + (size_t)q * SL;
    for (int j = tm.t; j < nc; j += tm.size()) {
      const int x = xr[j];
      const int t = M.mo((x * (x - 1)) >> 1);
      if (!inverse) {
        Cp[j] = (uint8_t)M.mo(Cp[j] + t);
        zr[j] = (uint8_t)M.md(zr[j] + x);
      } else {
        Cp[j] = (uint8_t)M.mo(Cp[j] + M.ord - t);
        zr[j] = (uint8_t)M.md(zr[j] + M.d - x);
      }
    }
  }
  __device__ __forceinline__ void cnot(int cq, int tq, bool inverse) {
    uint8_t* xc = X + (size_t)cq * SL;
    uint8_t* xt = X + (size_t)tq * SL;
    uint8_t* zc = Z + (size_t)cq * SL;
    uint8_t* zt = Z + (size_t)tq * SL;
    for (int j = tm.t; j < nc; j += tm.size()) {
      const int a = xc[j], b = xt[j], e = zc[j], f = zt[j];
      if (!inverse) {
        xt[j] = (uint8_t)M.md(b + a);
        zc[j] = (uint8_t)M.md(e + M.d - f);
      } else {
        xt[j] = (uint8_t)M.md(b + M.d - a);
        zc[j] = (uint8_t)M.md(e + f);
      }
    }
  }
  __device__ __forceinline__ void pauli(int q, int cz, int cx) {
    const uint8_t* xr = X + (size_t)q * SL;
    const uint8_t* zr = Z + (size_t)q * SL;
    for (int j = tm.t; j < nc; j += tm.size()) Cp[j] = (uint8_t)M.mo(Cp[j] + M.phi * (cz * zr[j] + cx * xr[j]));
  }

  // Rank-1 update of the local columns with the unexponentiated pivot column
  // (cx, cz) and the factors FW scaled by the exponent ex (word maskw keeps
  // only the bytes in keep: the pivot's own column is left out), with the
  // dots DOT[j] += z_j . cx of the columns before it (DOT zeroed by the
  // column owners) and the column's self-dot cx . cz added into HS[2]: the
  // arithmetic of SplitU8::rank1 over nc columns.  RF rows are in flight
  // per thread (their loads issued before any store): 16 when the columns
  // stream from global memory, 4 in shared memory.
  __device__ void rank1(const uint8_t* cx, const uint8_t* cz, int ex, int maskw, uint32_t keep) {
    const int size = tm.size(), t = tm.t;
    const int words = (nc + 3) >> 2;  // 0 in a CTA whose slice is empty (n < 4 K)
    const int R = words > 0 && size >= words ? size / words : 1;
    const int act = words == 0 ? 0 : size >= words ? R * words : size;
    if (t < act) {
      const int w0 = size >= words ? t % words : t;
      const int rr = size >= words ? t / words : 0;
      if (w0 == 0) {  // every row once among the threads of word 0
        int s = 0;
        for (int k = rr; k < n; k += R) s += cx[k] * cz[k];
        atomicAdd(&HS[2], s);
      }
      const uint32_t* fws = reinterpret_cast<const uint32_t*>(FW);
      const int S4 = SL >> 2;
      for (int w = w0; w < words; w += (size >= words ? words : size)) {
        uint32_t fw = fws[w];
        if (w == maskw) fw &= keep;
        if (fw == 0u) continue;
        if (ex != 1) {
          if constexpr (DD == 3 || DD == 5 || DD == 7) {
            fw = packed_mod<DD>(fw * (uint32_t)ex);  // bytes below d^2 - 2d + 2: no carries
          } else {
            uint32_t o = 0u;
#pragma unroll
            for (int j = 0; j < 4; ++j) o |= (uint32_t)M.md((int)((fw >> (8 * j)) & 0xff) * ex) << (8 * j);
            fw = o;
          }
        }
        int dots[4] = {0, 0, 0, 0};
        uint32_t* xcol = reinterpret_cast<uint32_t*>(X) + w;
        uint32_t* zcol = reinterpret_cast<uint32_t*>(Z) + w;
        if constexpr (DD == 3 || DD == 5 || DD == 7) {
          constexpr int RF = kStream ? 16 : 4;
          int k = rr;
          uint32_t dlo = 0u, dhi = 0u;
          int rows = 0;
          for (; k + (RF - 1) * R < n; k += RF * R) {
            uint32_t xw[RF], zw[RF];
#pragma unroll
            for (int i = 0; i < RF; ++i) {
              xw[i] = xcol[(size_t)(k + i * R) * S4];
              zw[i] = zcol[(size_t)(k + i * R) * S4];
            }
#pragma unroll
            for (int i = 0; i < RF; ++i) {
              const uint32_t a = cx[k + i * R], b = cz[k + i * R];
              dlo += (zw[i] & 0x00FF00FFu) * a;
              dhi += ((zw[i] >> 8) & 0x00FF00FFu) * a;
              xcol[(size_t)(k + i * R) * S4] = packed_mod<DD>(xw[i] + fw * a);
              zcol[(size_t)(k + i * R) * S4] = packed_mod<DD>(zw[i] + fw * b);
            }
            if ((rows += RF) >= 1024) {  // (1024 + RF) (d-1)^2 < 2^16
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
            const uint32_t a = cx[k], b = cz[k];
            dlo += (zw & 0x00FF00FFu) * a;
            dhi += ((zw >> 8) & 0x00FF00FFu) * a;
            xcol[(size_t)k * S4] = packed_mod<DD>(xw + fw * a);
            zcol[(size_t)k * S4] = packed_mod<DD>(zw + fw * b);
          }
          dots[0] += (int)(dlo & 0xffffu);
          dots[2] += (int)(dlo >> 16);
          dots[1] += (int)(dhi & 0xffffu);
          dots[3] += (int)(dhi >> 16);
        } else {
          for (int k = rr; k < n; k += R) {
            const uint32_t xw = xcol[(size_t)k * S4], zw = zcol[(size_t)k * S4];
            const int a = cx[k], b = cz[k];
            uint32_t xo = 0u, zo = 0u;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int f = (fw >> (8 * j)) & 0xff;
              const int x = (xw >> (8 * j)) & 0xff, z = (zw >> (8 * j)) & 0xff;
              dots[j] += z * a;
              xo |= (uint32_t)M.md(x + f * a) << (8 * j);
              zo |= (uint32_t)M.md(z + f * b) << (8 * j);
            }
            xcol[(size_t)k * S4] = xo;
            zcol[(size_t)k * S4] = zo;
            if (((k - rr) / R & 3) == 3) {
#pragma unroll
              for (int j = 0; j < 4; ++j) dots[j] = M.md(dots[j]);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int g = 4 * w + j;
          if (g < nc && ((fw >> (8 * j)) & 0xff)) atomicAdd(&DOT[g], M.md(dots[j]));
        }
      }
    }
    tm.sync();
  }
};

// One measurement (every CTA of the cluster runs it).
template <int DD, int K, bool kStream>
__device__ void cluster_measure(ClusterU8<DD, K, kStream>& e, const TraceDescU8& td, int q, uint32_t mord,
                                uint32_t nord, bool reset) {
  constexpr int H = K / 2;
  const int size = e.tm.size(), t = e.tm.t;
  const int n = e.n, SL = e.SL, np = e.np, nc = e.nc, C0 = e.C0, sw = td.sw, r = e.r, cs = e.c;
  const ModU8<DD>& M = e.M;
  uint8_t* X = e.X;
  uint8_t* Z = e.Z;
  uint8_t* Cp = e.Cp;
  const uint8_t* xq = X + (size_t)q * SL;
  uint8_t* row = td.mrow + (size_t)mord * 2 * sw;
  uint8_t* b = e.buf(mord);
  const int par = (int)(mord & 1u);
  // ---- before the barrier: factors, candidates and candidate columns.  The
  // column owners read only what they wrote themselves since the last
  // barrier.
  int mine = INT_MAX;
  for (int j = t; j < SL; j += size) {
    const int x = j < nc ? xq[j] : 0;
    e.FW[j] = (uint8_t)M.neg(x);
    e.DOT[j] = 0;
    if (x && j < mine) mine = j;
  }
  if (t == 0) e.HS[2] = 0;
  if (e.stab) {
    if (mine < nc) atomicMin(&e.HS[par], mine);
  } else {
    // the factors of stabilizer slice c are x_q over destabilizer slice c:
    // their words and each word's G_j, for the slice sums of a
    // deterministic outcome (this CTA waits at the cluster barrier anyway)
    e.tm.sync();
    const int cw = ((C0 + 15) & ~15) >> 2;
    const uint32_t fa = peer_addr(b + e.L.f, (uint32_t)cs), ga = peer_addr(b + e.L.g, (uint32_t)cs);
    for (int w = t; w < cw; w += size) {
      int f[4];
      uint32_t fw = 0u;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        f[j] = 4 * w + j < nc ? xq[4 * w + j] : 0;
        fw |= (uint32_t)f[j] << (8 * j);
      }
      st_peer_u32(fa + 4u * (uint32_t)w, fw);
      if constexpr (DD == 3 || DD == 5 || DD == 7) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint32_t gj = (uint32_t)((f[j] * (f[j] - 1)) >> 1) << (8 * j);
#pragma unroll
          for (int i = 0; i < j; ++i) gj |= (uint32_t)(f[i] * f[j]) << (8 * i);
          st_peer_u32(ga + 16u * (uint32_t)w + 4u * (uint32_t)j, gj);
        }
      }
    }
  }
  if (e.stab) {
    e.tm.sync();
    const int lm = e.HS[par];
    const int cand = lm < nc ? cs * C0 + lm : INT_MAX;
    uint8_t* slot = b + cs * e.L.slot;
    if (t < K) {
      const uint32_t a = peer_addr(slot, (uint32_t)t);
      st_peer_u32(a, (uint32_t)cand);
      if (lm < nc) {
        st_peer_u32(a + 4u, xq[lm]);
        st_peer_u32(a + 8u, Cp[lm]);
      }
    }
    if (lm < nc) {
      // the candidate column, four rows to a word, to every CTA
      const int np4 = np >> 2;
      for (int i = t; i < 2 * np4 * K; i += size) {
        const int rk = i / (2 * np4), rem = i - rk * 2 * np4;
        const int zs = rem >= np4 ? 1 : 0, w = rem - zs * np4;
        const uint8_t* col = (zs ? Z : X) + lm;
        uint32_t v = 0u;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = 4 * w + j;
          v |= (uint32_t)(k < n ? col[(size_t)k * SL] : 0) << (8 * j);
        }
        st_peer_u32(peer_addr(slot + 16 + zs * np + 4 * w, (uint32_t)rk), v);
      }
    }
    if (t == 0) e.HS[par ^ 1] = INT_MAX;  // its last reader passed this barrier
  }
  cluster_sync_all();
  // ---- after the barrier
  int p = INT_MAX, owner = -1;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const int ci = *reinterpret_cast<const int*>(b + i * e.L.slot);
    if (ci < p) {
      p = ci;
      owner = i;
    }
  }
  if (p < n) {
    const uint8_t* slot = b + owner * e.L.slot;
    const int xv = reinterpret_cast<const int*>(slot)[1], cpraw = reinterpret_cast<const int*>(slot)[2];
    const uint8_t* pcx = slot + 16;
    const uint8_t* pcz = pcx + np;
    const int ex = xv == 1 ? 1 : M.inv(xv);
    const bool own = r == owner;  // the stabilizer CTA holding column p
    const int pl = p - cs * C0;   // its local column, in the owner's slice
    const int maskw = own ? (pl >> 2) : -1;
    const uint32_t keep = ~(0xffu << (8 * (pl & 3)));
    e.rank1(pcx, pcz, ex, maskw, keep);
    const int s0 = M.md(e.HS[2]);
    const int s1 = M.md(M.md(ex * ex) * s0);
    const int phc = ex == 1 ? cpraw : M.mo(cpraw * ex + M.md(s0 * M.md((ex * (ex - 1)) >> 1)) * M.phi);
    for (int j = t; j < nc; j += size) {
      const int f = (own && j == pl) ? 0 : (int)e.FW[j];
      row[e.g0 + j] = (uint8_t)f;
      if (f == 0) continue;
      const int dot = M.md(ex * e.DOT[j]);
      const int half = M.md(s1 * ((f * (f - 1)) >> 1));
      Cp[j] = (uint8_t)M.mo(Cp[j] + phc * f + M.phi * M.md(f * dot) + M.phi * M.phi * half);
    }
    if (r == 0)
      for (int g = 2 * n + t; g < sw; g += size) row[g] = 0;
    // pivot columns: stabilizer p <- Z_q, destabilizer n + p <- stabilizer p exponentiated
    if (cs == owner) {
      for (int k = t; k < n; k += size) {
        if (e.stab) {
          X[(size_t)k * SL + pl] = 0;
          Z[(size_t)k * SL + pl] = (uint8_t)(k == q);
        } else {
          X[(size_t)k * SL + pl] = (uint8_t)M.md(ex * pcx[k]);
          Z[(size_t)k * SL + pl] = (uint8_t)M.md(ex * pcz[k]);
        }
      }
      if (t == pl % size) Cp[pl] = e.stab ? (uint8_t)0 : (uint8_t)phc;  // after its own phase update above
    }
    if (r == 0 && e.tm.leader())
      td.mhdr[mord] = make_uint4((reset ? 2u : 0u) | ((uint32_t)ex << 8), (uint32_t)p, nord, 0u);
    e.tm.sync();
  } else {
    if (e.stab) {
      // deterministic: this slice's sums to global memory.  sum_j f_j c_j
      // here; the f_j (f_j - 1) / 2 (x_j . z_j) term of this slice is summed
      // row by row below
      const uint8_t* fb = b + e.L.f;
      uint8_t* ds = td.dsum + (size_t)mord * cluster_det_bytes(n, K) + (size_t)cs * cluster_det_slice(n);
      int pl_sum = 0, dl = 0;
      for (int j = t; j < nc; j += size) {
        const int fj = fb[j];
        row[cs * C0 + j] = (uint8_t)fj;  // this slice of the factor row
        if (fj) pl_sum += fj * Cp[j];
      }
      int al = 0;
      const int nw = (nc + 3) >> 2;
      const uint32_t* fq = reinterpret_cast<const uint32_t*>(fb);
      if constexpr (DD == 3 || DD == 5 || DD == 7) {
        // per word: Z_w = f . z, X_w = f . x, and the in-word terms
        // sum_{i < j} f_i f_j z_i x_j + sum_j f_j (f_j - 1) / 2 x_j z_j as
        // sum_j x_j (z . G_j): byte dot products.  The two sums meet with
        // equal weight in the phase (phi = 1 for odd d), so A_c holds both.
        const uint4* gq = reinterpret_cast<const uint4*>(b + e.L.g);
        for (int k = t; k < np; k += size) {
          int pre = 0, acc = 0, xs = 0;
          if (k < n) {
            const uint32_t* xr = reinterpret_cast<const uint32_t*>(X + (size_t)k * SL);
            const uint32_t* zr = reinterpret_cast<const uint32_t*>(Z + (size_t)k * SL);
            for (int w = 0; w < nw; ++w) {
              const uint32_t fw = fq[w];
              if (!fw) continue;
              const uint32_t xw = xr[w], zw = zr[w];
              const uint4 G = gq[w];
              const int zs = (int)__dp4a(zw, fw, 0u), xsw = (int)__dp4a(xw, fw, 0u);
              int in = (int)(xw & 0xffu) * (int)__dp4a(zw, G.x, 0u);
              in += (int)((xw >> 8) & 0xffu) * (int)__dp4a(zw, G.y, 0u);
              in += (int)((xw >> 16) & 0xffu) * (int)__dp4a(zw, G.z, 0u);
              in += (int)(xw >> 24) * (int)__dp4a(zw, G.w, 0u);
              acc = M.md(acc + pre * xsw + in);
              pre = M.md(pre + zs);
              xs += xsw;
            }
          }
          ds[k] = (uint8_t)pre;
          ds[np + k] = (uint8_t)M.md(xs);
          al += acc;
        }
      } else {
        for (int k = t; k < np; k += size) {
          int pre = 0, acc = 0, xs = 0, dd = 0;
          if (k < n) {
            const uint32_t* xr = reinterpret_cast<const uint32_t*>(X + (size_t)k * SL);
            const uint32_t* zr = reinterpret_cast<const uint32_t*>(Z + (size_t)k * SL);
            for (int w = 0; w < nw; ++w) {
              const uint32_t fw = fq[w];
              if (!fw) continue;
              const uint32_t xw = xr[w], zw = zr[w];
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const int fj = (fw >> (8 * j)) & 0xff;
                if (fj) {
                  const int xv = (int)((xw >> (8 * j)) & 0xff), zv = (int)((zw >> (8 * j)) & 0xff);
                  acc = M.md(acc + fj * xv * pre);
                  pre = M.md(pre + fj * zv);
                  xs = M.md(xs + fj * xv);
                  dd = M.half_xz(dd, fj, xv, zv);
                }
              }
            }
          }
          ds[k] = (uint8_t)pre;
          ds[np + k] = (uint8_t)xs;
          al += acc;
          dl += M.md(dd);
        }
      }
      // per-warp partials; the header pass adds them up
      for (int off = 16; off > 0; off >>= 1) {
        pl_sum += __shfl_xor_sync(0xffffffffu, pl_sum, off);
        al += __shfl_xor_sync(0xffffffffu, al, off);
        dl += __shfl_xor_sync(0xffffffffu, dl, off);
      }
      if ((t & 31) == 0) {
        int* part = reinterpret_cast<int*>(ds + 2 * np) + 3 * (t >> 5);
        part[0] = pl_sum;
        part[1] = al;
        part[2] = dl;
      }
      // every row was read across the slice's columns: the column owners
      // may write them again (the next gate) only after this barrier
      e.tm.sync();
    } else {
      for (int j = t; j < nc; j += size) row[e.g0 + j] = 0;
    }
    if (r == 0) {
      for (int g = 2 * n + t; g < sw; g += size) row[g] = 0;
      if (e.tm.leader()) td.mhdr[mord] = make_uint4(reset ? 3u : 1u, 0u, nord, 0u);
    }
  }
  if (reset) {
    // the columns are as the owners or a barrier left them
    const uint8_t* zq = Z + (size_t)q * SL;
    for (int j = t; j < nc; j += size) row[sw + e.g0 + j] = zq[j];
    if (r == 0)
      for (int g = 2 * n + t; g < sw; g += size) row[sw + g] = 0;
  }
}

// Deterministic outcomes of the cluster x / z pass, after it: one warp per
// measurement adds the stabilizer slices' partial sums and the cross-slice
// term sum_k sum_{c' < c} Z_c'[k] X_c[k], and writes the common phase
// P + phi T + phi^2 D into the header (w).
template <int K>
__device__ void cluster_det_header(const TraceDescU8& td, int m, int lane) {
  constexpr int H = K / 2;
  const uint4 h = td.mhdr[m];
  if (!(h.x & 1u)) return;
  const ModU8<0> M(td.c.d);
  const int n = td.c.n, np = SlotU8::npad(n);
  const size_t sb = cluster_det_slice(n);
  const uint8_t* base = td.dsum + (size_t)m * cluster_det_bytes(n, K);
  int cl = 0, P = 0, A = 0, D = 0;
  for (int k = lane; k < n; k += 32) {
    int zb = 0, ck = 0;
#pragma unroll
    for (int s = 0; s < H; ++s) {
      ck += zb * (int)base[s * sb + np + k];
      zb += (int)base[s * sb + k];
    }
    cl += M.md(ck);
  }
  constexpr int nw = kTracePassThreads / 32;
  for (int i = lane; i < H * nw; i += 32) {
    const int* part = reinterpret_cast<const int*>(base + (size_t)(i / nw) * sb + 2 * np) + 3 * (i % nw);
    P += part[0];
    A += part[1];
    D += part[2];
  }
  for (int off = 16; off > 0; off >>= 1) {
    cl += __shfl_xor_sync(0xffffffffu, cl, off);
    P += __shfl_xor_sync(0xffffffffu, P, off);
    A += __shfl_xor_sync(0xffffffffu, A, off);
    D += __shfl_xor_sync(0xffffffffu, D, off);
  }
  if (lane == 0) {
    const int T = M.md(M.md(A) + M.md(cl));
    td.mhdr[m].w = (uint32_t)M.mo(M.mo(P) + M.phi * T + M.phi * M.phi * M.md(D));
  }
}

// Runs the shared part of td's program on the cluster and writes its trace.
template <int DD, int K, bool kStream>
__device__ void cluster_program(const TraceDescU8& td, ClusterU8<DD, K, kStream>& e, uint2* win, int* status) {
  const CircuitDesc& c = td.c;
  e.init();
  const int t = e.tm.t, size = e.tm.size();
  const int n = c.n, d = c.d, SL = e.SL, sw = td.sw, r = e.r, nc = e.nc;
  const uint2* ops = td.lay ? td.lay : c.ops;
  const int nops = td.lay ? td.nlay : c.nops;
  uint32_t mord = 0, nord = 0;
  const bool colless = (t & ~31) >= nc;  // this thread's warp holds no column
  int skip_to = 0;
  for (int i = 0; i < nops; ++i) {
    if ((i & (kOpWindow - 1)) == 0) {  // stage the next window of instructions
      e.tm.sync();
      const int cnt = min(kOpWindow, nops - i);
      for (int j = t; j < cnt; j += size) win[j] = __ldg(ops + i + j);
      e.tm.sync();
    }
    if (i < skip_to) {  // a warp with no column passes a run of gates, stopping at window starts
      i = min(skip_to, (i | (kOpWindow - 1)) + 1) - 1;
      continue;
    }
    const uint2 cur = win[i & (kOpWindow - 1)];
    const uint32_t op = cur.x & kOpMask;
    const int q = (int)(cur.x >> 8);
    // every CTA reads the same stream and leaves at the same instruction
    if (q >= n) {
      if (t == 0 && r == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      break;
    }
    bool bad = false;
    switch (op) {
      case OP_NOP: break;
      case OP_RUN:
        if (colless) skip_to = i + 1 + (int)cur.y;
        break;
      case OP_GROUP: {  // never straddles a window; the column owners apply it
        const int cnt = (int)cur.y;
        const uint2* gops = win + ((i + 1) & (kOpWindow - 1));
        for (int j = t; j < nc; j += size) gate_group_column(gops, cnt, e.X, e.Z, (size_t)SL, e.Cp, j, e.M);
        i += cnt;
        break;
      }
      case OP_X: e.pauli(q, d - 1, 0); break;
      case OP_X_INV: e.pauli(q, 1, 0); break;
      case OP_Z: e.pauli(q, 0, 1); break;
      case OP_Z_INV: e.pauli(q, 0, d - 1); break;
      case OP_H: e.h(q); break;
      case OP_H_INV: e.h_inv(q); break;
      case OP_P: e.p(q, false); break;
      case OP_P_INV: e.p(q, true); break;
      case OP_CNOT:
      case OP_CNOT_INV: {
        const int tq = (int)cur.y;
        if (tq >= n) {
          if (t == 0 && r == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
          bad = true;
          break;
        }
        e.cnot(q, tq, op == OP_CNOT_INV);
        break;
      }
      case OP_M:
      case OP_RESET:
        if ((int)mord >= td.nm) {
          if (t == 0 && r == 0) atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
          bad = true;
          break;
        }
        cluster_measure(e, td, q, mord, nord, op == OP_RESET);
        ++mord;
        break;
      case OP_N1D:
      case OP_N1F:
      case OP_N1P:
      case OP_N1OFF:
        if ((int)nord >= td.nn1) {
          if (t == 0 && r == 0) atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
          bad = true;
          break;
        }
        if (t == 0 && r == 0) td.nhdr[nord] = make_uint2(op == OP_N1OFF ? 0xffffffffu : cur.y, op);
        if (op != OP_N1OFF) {
          const uint8_t* xr = e.X + (size_t)q * SL;
          const uint8_t* zr = e.Z + (size_t)q * SL;
          uint8_t* dst = td.nrow + (size_t)nord * 2 * sw;
          for (int j = t; j < nc; j += size) {
            dst[e.g0 + j] = xr[j];
            dst[sw + e.g0 + j] = zr[j];
          }
          if (r == 0)
            for (int g = 2 * n + t; g < sw; g += size) {
              dst[g] = 0;
              dst[sw + g] = 0;
            }
        }
        ++nord;
        break;
      default:
        if (t == 0 && r == 0) atomicCAS(status, DEV_OK, DEV_BAD_OPCODE);
        bad = true;
        break;
    }
    if (bad) break;
  }
  e.tm.sync();
  cluster_sync_all();  // no CTA leaves or starts the next program while a partner may still write into it
}

}  // namespace sdim
