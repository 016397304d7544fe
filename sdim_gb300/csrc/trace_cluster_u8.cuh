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
// applies every gate to its own columns.
//
// A measurement on qudit q takes exactly two cluster barriers on every CTA,
// whatever its outcome, so all CTAs pass the same barriers:
//   before barrier 1: stabilizer CTA c publishes its lowest column with
//     x_q != 0 (its pivot candidate) to every CTA; destabilizer CTA H + c
//     sends stabilizer CTA c its slice of x_q (the factors f of a
//     deterministic outcome);
//   between the barriers: every CTA knows p = the lowest candidate.  If there
//     is one (random outcome), its owner exponentiates its column p when
//     needed and broadcasts (p, s1, phc, e, x_p, z_p) to every CTA.  If not
//     (deterministic), each stabilizer CTA c sends CTA 0 its partial sums
//     P_c = sum f_i c_i, D_c = sum f_i (f_i - 1) / 2 x_i.z_i and the in-slice
//     cross term A_c, and per row k the slice sums Z_c[k] = sum f_i z_k[i]
//     and X_c[k] = sum f_i x_k[i];
//   after barrier 2: a random measurement runs its rank-1 update, phases and
//     pivot columns on every CTA; for a deterministic one CTA 0 adds the
//     cross-slice term sum_k sum_{c' < c} Z_c'[k] X_c[k] and writes the header.
// Exchange buffers alternate by measurement parity: a CTA writes the buffer
// of measurement m + 2 only after the barriers of m + 1, which its partners
// pass only after they finished reading m's.  The arithmetic per column is
// that of group_u8.cuh and the trace written is the one of trace_u8.cuh.
#pragma once
#include "trace_split_u8.cuh"

namespace sdim {

__host__ __device__ inline int cluster_cols(int n, int K) { return (n + K / 2 - 1) / (K / 2); }

// Byte offsets inside one exchange buffer: candidates int[H]; pivot words
// (p, s1, phc, e), x_p[np], z_p[np]; factors f[cpad]; per stabilizer slice
// the words (P, A, D, 0), Z_c[np], X_c[np].
struct ClusterXchg {
  int mins, piv, f, det, slot, total;
  __host__ __device__ ClusterXchg(int n, int K) {
    const int H = K / 2, np = SlotU8::npad(n), cpad = (cluster_cols(n, K) + 15) & ~15;
    mins = 0;
    piv = (4 * H + 15) & ~15;
    f = piv + 16 + 2 * np;
    det = f + cpad;
    slot = 16 + 2 * np;
    total = det + H * slot;
  }
};

// Shared memory of one CTA besides its columns: phases and factors (SL
// each), the staged pivot column (np each), the dots (int[SL]), 16 bytes of
// staged words and two exchange buffers.
__host__ __device__ inline size_t cluster_hot_bytes(int n, int K) {
  const size_t sl = (size_t)split_stride(cluster_cols(n, K)), np = (size_t)SlotU8::npad(n);
  return round_up(2 * sl + 2 * np, 16) + 4 * sl + 16 + 2 * round_up((size_t)ClusterXchg(n, K).total, 16);
}

// The columns of one CTA: X and Z, n rows of SL bytes each.
__host__ __device__ inline size_t cluster_xz_bytes(int n, int K) {
  return round_up(2 * (size_t)n * (size_t)split_stride(cluster_cols(n, K)), 16);
}

template <int DD, int K, bool kStream>
struct ClusterU8 {
  static constexpr int H = K / 2;
  CtaTeam tm;
  ModU8<DD> M;
  int r, c, stab;             // cluster rank, slice, 1 for a stabilizer CTA
  int n, nc, C0, g0, SL, np;  // local columns, columns per slice, first generator held
  uint8_t *X, *Z, *Cp, *FW, *CX, *CZ, *HS;
  int* DOT;
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
    CX = FW + SL;
    CZ = CX + np;
    DOT = reinterpret_cast<int*>(hot + round_up(2 * (size_t)SL + 2 * (size_t)np, 16));
    HS = reinterpret_cast<uint8_t*>(DOT + SL);
    xb = HS + 16;
    xbytes = (int)round_up((size_t)L.total, 16);
  }
  __device__ uint8_t* buf(uint32_t mord) const { return xb + (size_t)(mord & 1u) * xbytes; }

  __device__ void init() {
    uint32_t* w = reinterpret_cast<uint32_t*>(X);
    const size_t words = (2 * (size_t)n * SL) >> 2;
    for (size_t i = tm.t; i < words; i += tm.size()) w[i] = 0u;
    for (int j = tm.t; j < 2 * SL; j += tm.size()) Cp[j] = 0;  // phases and factors
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

  // Rank-1 update of the local columns with pivot column (cx, cz) and the
  // factors in FW, with the dots DOT[j] = z_j . cx of the columns before it:
  // the arithmetic of SplitU8::rank1 over nc columns.  RF rows are in flight
  // per thread (their loads issued before any store): 16 when the columns
  // stream from global memory, 4 in shared memory.
  __device__ void rank1(const uint8_t* cx, const uint8_t* cz) {
    const int size = tm.size(), t = tm.t;
    const int words = (nc + 3) >> 2;
    for (int j = t; j < nc; j += size) DOT[j] = 0;
    tm.sync();
    if (words > 0) {
      const int R = size >= words ? size / words : 1;
      const int act = size >= words ? R * words : size;
      if (t < act) {
        const int w0 = size >= words ? t % words : t;
        const int rr = size >= words ? t / words : 0;
        const uint32_t* fws = reinterpret_cast<const uint32_t*>(FW);
        const int S4 = SL >> 2;
        for (int w = w0; w < words; w += (size >= words ? words : size)) {
          const uint32_t fw = fws[w];
          if (fw == 0u) continue;
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
            if (g < nc && ((fw >> (8 * j)) & 0xff)) {
              if (R > 1)
                atomicAdd(&DOT[g], M.md(dots[j]));
              else
                DOT[g] = M.md(dots[j]);
            }
          }
        }
      }
    }
    tm.sync();
  }
};

// Writes bytes [0, len) of src (4-byte aligned, len a multiple of 4) to the
// same offset as dst_local in CTA `rank` of the cluster.
__device__ __forceinline__ void put_peer_bytes(uint8_t* dst_local, const uint8_t* src, int len, uint32_t rank, int t,
                                               int size) {
  const uint32_t base = peer_addr(dst_local, rank);
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  for (int i = t; i < (len >> 2); i += size) st_peer_u32(base + 4u * (uint32_t)i, s[i]);
}

// One measurement (every CTA of the cluster runs it).
template <int DD, int K, bool kStream>
__device__ void cluster_measure(ClusterU8<DD, K, kStream>& e, const TraceDescU8& td, int q, uint32_t mord,
                                uint32_t nord, bool reset) {
  constexpr int H = K / 2;
  e.tm.sync();
  const int size = e.tm.size(), t = e.tm.t;
  const int n = e.n, SL = e.SL, np = e.np, nc = e.nc, C0 = e.C0, sw = td.sw, r = e.r, cs = e.c;
  const ModU8<DD>& M = e.M;
  uint8_t* X = e.X;
  uint8_t* Z = e.Z;
  uint8_t* Cp = e.Cp;
  const uint8_t* xq = X + (size_t)q * SL;
  uint8_t* row = td.mrow + (size_t)mord * 2 * sw;
  uint8_t* b = e.buf(mord);
  const int* mins = reinterpret_cast<const int*>(b + e.L.mins);
  const int* ph = reinterpret_cast<const int*>(b + e.L.piv);  // p, s1, phc, e
  const uint8_t* pcx = b + e.L.piv + 16;
  const uint8_t* pcz = pcx + np;
  const uint8_t* fb = b + e.L.f;
  // ---- before barrier 1: candidates and factors
  if (e.stab) {
    int mine = INT_MAX;
    for (int j = t; j < nc; j += size)
      if (xq[j]) {
        mine = j;
        break;
      }
    const int lm = e.tm.min(mine);
    const int cand = lm < nc ? cs * C0 + lm : INT_MAX;
    if (t < K) st_peer_u32(peer_addr(b + e.L.mins + 4 * r, (uint32_t)t), (uint32_t)cand);
  } else {
    // the factors of stabilizer slice c are x_q over destabilizer slice c
    const int cpad = (C0 + 15) & ~15;
    for (int i = 4 * t; i < cpad; i += 4 * size) {
      uint32_t v = 0u;
#pragma unroll
      for (int j = 0; j < 4; ++j) v |= (uint32_t)(i + j < nc ? xq[i + j] : 0) << (8 * j);
      st_peer_u32(peer_addr(b + e.L.f + i, (uint32_t)cs), v);
    }
  }
  cluster_sync_all();
  // ---- between the barriers
  int p = INT_MAX;
#pragma unroll
  for (int i = 0; i < H; ++i) p = min(p, mins[i]);
  const bool random = p < n;
  const int owner = random ? p / C0 : -1;  // slice holding stabilizer p
  const int pl = p - cs * C0;              // its local column, in the owner's slice
  if (random) {
    if (r == owner) {
      const int xv = xq[pl];
      int ex = 1;
      if (xv != 1) {
        ex = M.inv(xv);
        int sl = 0;
        for (int k = t; k < n; k += size) sl += X[(size_t)k * SL + pl] * Z[(size_t)k * SL + pl];
        const int s0 = M.md(e.tm.add(sl));
        if (e.tm.leader()) Cp[pl] = (uint8_t)M.mo(Cp[pl] * ex + M.md(s0 * M.md((ex * (ex - 1)) >> 1)) * M.phi);
        for (int k = t; k < n; k += size) {
          X[(size_t)k * SL + pl] = (uint8_t)M.md(X[(size_t)k * SL + pl] * ex);
          Z[(size_t)k * SL + pl] = (uint8_t)M.md(Z[(size_t)k * SL + pl] * ex);
        }
        e.tm.sync();
      }
      int sl = 0;
      for (int k = t; k < np; k += size) {
        const int a = k < n ? X[(size_t)k * SL + pl] : 0, bb = k < n ? Z[(size_t)k * SL + pl] : 0;
        e.CX[k] = (uint8_t)a;
        e.CZ[k] = (uint8_t)bb;
        sl += a * bb;
      }
      const int s1 = M.md(e.tm.add(sl));
      if (e.tm.leader()) {
        int* hs = reinterpret_cast<int*>(e.HS);
        hs[0] = p;
        hs[1] = s1;
        hs[2] = Cp[pl];
        hs[3] = ex;
      }
      e.tm.sync();
      for (int rk = 0; rk < K; ++rk) {
        put_peer_bytes(b + e.L.piv + 16, e.CX, np, (uint32_t)rk, t, size);
        put_peer_bytes(b + e.L.piv + 16 + np, e.CZ, np, (uint32_t)rk, t, size);
        put_peer_bytes(b + e.L.piv, e.HS, 16, (uint32_t)rk, t, size);
      }
    }
  } else if (e.stab) {
    // deterministic: this slice's partial sums to CTA 0
    // sum_j f_j c_j here; the f_j (f_j - 1) / 2 (x_j . z_j) term of this
    // slice is summed row by row in the cross-term pass below
    int pl_sum = 0, dl = 0;
    for (int j = t; j < nc; j += size) {
      const int fj = fb[j];
      if (fj) pl_sum += fj * Cp[j];
    }
    int al = 0;
    const int nw = (nc + 3) >> 2;
    const uint32_t* fq = reinterpret_cast<const uint32_t*>(fb);
    for (int k = t; k < np; k += size) {  // Z_c[k] staged in CX, X_c[k] in CZ
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
      e.CX[k] = (uint8_t)pre;
      e.CZ[k] = (uint8_t)xs;
      al += acc;
      dl += M.md(dd);
    }
    e.tm.add3(pl_sum, al, dl);  // its barriers also publish CX / CZ
    const int P = M.mo(pl_sum);
    const int A = M.md(al);
    const int Dd = M.md(dl);
    uint8_t* slot = b + e.L.det + cs * e.L.slot;
    // the slice's sums straight to CTA 0 (every thread holds them)
    if (t < 4) st_peer_u32(peer_addr(slot + 4 * t, 0u), (uint32_t)(t == 0 ? P : t == 1 ? A : t == 2 ? Dd : 0));
    put_peer_bytes(slot + 16, e.CX, np, 0u, t, size);
    put_peer_bytes(slot + 16 + np, e.CZ, np, 0u, t, size);
    for (int j = t; j < nc; j += size) row[cs * C0 + j] = fb[j];  // this slice of the factor row
  }
  cluster_sync_all();
  // ---- after barrier 2
  if (random) {
    const int s1 = ph[1], phc = ph[2], ex = ph[3];
    const bool own = r == owner;
    for (int j = t; j < SL; j += size)
      e.FW[j] = (j < nc && !(own && j == pl)) ? (uint8_t)M.neg(xq[j]) : (uint8_t)0;
    e.tm.sync();
    for (int j = t; j < nc; j += size) row[e.g0 + j] = e.FW[j];
    if (r == 0)
      for (int g = 2 * n + t; g < sw; g += size) row[g] = 0;
    e.rank1(pcx, pcz);
    for (int j = t; j < nc; j += size) {
      const int f = e.FW[j];
      if (f == 0) continue;
      const int half = M.md(s1 * ((f * (f - 1)) >> 1));
      Cp[j] = (uint8_t)M.mo(Cp[j] + phc * f + M.phi * M.md(f * e.DOT[j]) + M.phi * M.phi * half);
    }
    e.tm.sync();
    // pivot columns: stabilizer p <- Z_q, destabilizer n + p <- stabilizer p as broadcast
    if (cs == owner) {
      for (int k = t; k < n; k += size) {
        if (e.stab) {
          X[(size_t)k * SL + pl] = 0;
          Z[(size_t)k * SL + pl] = (uint8_t)(k == q);
        } else {
          X[(size_t)k * SL + pl] = pcx[k];
          Z[(size_t)k * SL + pl] = pcz[k];
        }
      }
      if (e.tm.leader()) Cp[pl] = e.stab ? (uint8_t)0 : (uint8_t)phc;
    }
    if (r == 0 && e.tm.leader())
      td.mhdr[mord] = make_uint4((reset ? 2u : 0u) | ((uint32_t)ex << 8), (uint32_t)p, nord, 0u);
    e.tm.sync();
  } else {
    if (!e.stab)
      for (int j = t; j < nc; j += size) row[e.g0 + j] = 0;
    if (r == 0) {
      for (int g = 2 * n + t; g < sw; g += size) row[g] = 0;
      // cross-slice term sum_k sum_{c' < c} Z_c'[k] X_c[k]
      int cl = 0;
      for (int k = t; k < n; k += size) {
        int zb = 0;
        for (int s = 0; s < H; ++s) {
          const uint8_t* sl = b + e.L.det + s * e.L.slot;
          cl += zb * (int)sl[16 + np + k];
          zb = M.md(zb + (int)sl[16 + k]);
        }
        cl = M.md(cl);
      }
      const int cross = M.md(e.tm.add(cl));
      int P = 0, A = 0, Dd = 0;
      for (int s = 0; s < H; ++s) {
        const int* hd = reinterpret_cast<const int*>(b + e.L.det + s * e.L.slot);
        P += hd[0];
        A += hd[1];
        Dd += hd[2];
      }
      const int T = M.md(A + cross);
      const int aphc = M.mo(M.mo(P) + M.phi * T + M.phi * M.phi * M.md(Dd));
      if (e.tm.leader()) td.mhdr[mord] = make_uint4(reset ? 3u : 1u, 0u, nord, (uint32_t)aphc);
    }
    e.tm.sync();
  }
  if (reset) {
    e.tm.sync();
    const uint8_t* zq = Z + (size_t)q * SL;
    for (int j = t; j < nc; j += size) row[sw + e.g0 + j] = zq[j];
    if (r == 0)
      for (int g = 2 * n + t; g < sw; g += size) row[sw + g] = 0;
  }
}

// Runs the shared part of td's program on the cluster and writes its trace.
template <int DD, int K, bool kStream>
__device__ void cluster_program(const TraceDescU8& td, ClusterU8<DD, K, kStream>& e, uint2* win, int* status) {
  const CircuitDesc& c = td.c;
  e.init();
  const int t = e.tm.t, size = e.tm.size();
  const int n = c.n, d = c.d, SL = e.SL, sw = td.sw, r = e.r, nc = e.nc;
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
    // every CTA reads the same stream and leaves at the same instruction
    if (q >= n) {
      if (t == 0 && r == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      break;
    }
    bool bad = false;
    switch (op) {
      case OP_NOP: break;
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
