// x / z pass of the odd-d trace engine on a cluster of two CTAs: CTA 0
// keeps the stabilizer columns [0, n) of X, Z and the phases, CTA 1 the
// destabilizer columns [n, 2n), each in its own shared memory (n x n bytes
// per block), so tableaux up to n ~ 330 stay on chip where one CTA would
// spill them to global memory.
//
// Gates act on every generator column the same way, so each CTA applies
// every gate to its own columns with no exchange.  A measurement on qudit q
// needs one cluster barrier: before it, CTA 1 writes its half of x_q (the
// destabilizer factors f of a deterministic outcome) into CTA 0's exchange
// buffer, and CTA 0 finds the pivot p, exponentiates column p and writes p,
// the pivot column (CX, CZ = column p of X, Z) and its phase scalars into
// CTA 1's buffer (distributed shared memory).  After it, a random
// measurement runs its rank-1 update, phase updates and pivot columns on
// both halves (CTA 1's column p is the destabilizer n + p), and a
// deterministic one is evaluated by CTA 0 alone.  Exchange buffers alternate
// by measurement parity, so the next measurement's writes never meet this
// one's reads.  Arithmetic per column is that of group_u8.cuh; the trace
// written is the one of trace_u8.cuh.
#pragma once
#include "trace_u8.cuh"

namespace sdim {

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory address of the same offset in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t peer_addr(const void* local, uint32_t rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(local), out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(a), "r"(rank));
  return out;
}

__device__ __forceinline__ void st_peer_u32(uint32_t addr, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// Local column stride: a multiple of 4 bytes with an odd word count, so the
// 32 rows a warp walks down one column sit in 32 different banks.
__host__ __device__ inline int split_stride(int n) {
  const int s = (n + 3) & ~3;
  return ((s >> 2) & 1) ? s : s + 4;
}

// Bytes of an exchange buffer: ints p, s1, phc, ex, then cx[np], cz[np], f[np].
__host__ __device__ inline int split_xchg_bytes(int n) { return 16 + 3 * SlotU8::npad(n); }

// Dynamic shared memory of one CTA of the pair.
__host__ __device__ inline size_t split_smem_bytes(int n) {
  const size_t sl = (size_t)split_stride(n), np = (size_t)SlotU8::npad(n);
  return round_up(2 * (size_t)n * sl + 2 * sl + 2 * np, 16) + 4 * sl + 2 * round_up((size_t)split_xchg_bytes(n), 16);
}

template <int DD>
struct SplitU8 {
  CtaTeam tm;
  ModU8<DD> M;
  int r;        // 0: stabilizer columns, 1: destabilizer columns
  int n, SL, np;
  uint8_t *X, *Z, *C, *FW, *CX, *CZ;
  int* DOT;
  uint8_t* xb;  // two exchange buffers
  int xbytes;

  __device__ SplitU8(uint8_t* smem, int n_, int d, int* red) : tm(red), M(d), n(n_) {
    r = (int)cluster_rank();
    SL = split_stride(n_);
    np = SlotU8::npad(n_);
    X = smem;
    Z = X + (size_t)n * SL;
    C = Z + (size_t)n * SL;
    FW = C + SL;
    CX = FW + SL;
    CZ = CX + np;
    DOT = reinterpret_cast<int*>(smem + round_up(2 * (size_t)n * SL + 2 * (size_t)SL + 2 * (size_t)np, 16));
    xb = reinterpret_cast<uint8_t*>(DOT + SL);
    xbytes = (int)round_up((size_t)split_xchg_bytes(n_), 16);
  }
  __device__ uint8_t* buf(uint32_t mord) const { return xb + (size_t)(mord & 1u) * xbytes; }

  __device__ void init() {
    uint32_t* w = reinterpret_cast<uint32_t*>(X);
    const size_t words = (2 * (size_t)n * SL + 2 * (size_t)SL) >> 2;
    for (size_t i = tm.t; i < words; i += tm.size()) w[i] = 0u;
    tm.sync();
    // stabilizer k = Z_k (CTA 0), destabilizer k = X_k (CTA 1)
    for (int k = tm.t; k < n; k += tm.size()) (r == 0 ? Z : X)[(size_t)k * SL + k] = 1;
    tm.sync();
  }

  // ---- gates on the local columns (column g owned by thread g mod size)
  __device__ __forceinline__ void h(int q) {
    uint8_t* xr = X + (size_t)q * SL;
    uint8_t* zr = Z + (size_t)q * SL;
    for (int g = tm.t; g < n; g += tm.size()) {
      const int x = xr[g], z = zr[g];
      const int nx = M.neg(z);
      C[g] = (uint8_t)M.mo(C[g] + M.phi * nx * x);
      xr[g] = (uint8_t)nx;
      zr[g] = (uint8_t)x;
    }
  }
  __device__ __forceinline__ void h_inv(int q) {
    uint8_t* xr = X + (size_t)q * SL;
    uint8_t* zr = Z + (size_t)q * SL;
    for (int g = tm.t; g < n; g += tm.size()) {
      const int x = xr[g], z = zr[g];
      const int nz = M.neg(x);
      C[g] = (uint8_t)M.mo(C[g] + M.phi * z * nz);
      xr[g] = (uint8_t)z;
      zr[g] = (uint8_t)nz;
    }
  }
  __device__ __forceinline__ void p(int q, bool inverse) {
    const uint8_t* xr = X + (size_t)q * SL;
    uint8_t* zr = Z + (size_t)q * SL;
    for (int g = tm.t; g < n; g += tm.size()) {
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
    uint8_t* xc = X + (size_t)c * SL;
    uint8_t* xt = X + (size_t)t * SL;
    uint8_t* zc = Z + (size_t)c * SL;
    uint8_t* zt = Z + (size_t)t * SL;
    for (int g = tm.t; g < n; g += tm.size()) {
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
    const uint8_t* xr = X + (size_t)q * SL;
    const uint8_t* zr = Z + (size_t)q * SL;
    for (int g = tm.t; g < n; g += tm.size()) C[g] = (uint8_t)M.mo(C[g] + M.phi * (cz * zr[g] + cx * xr[g]));
  }

  // Rank-1 update of the local columns with pivot column (cx, cz): the
  // arithmetic of TGroupU8::word_update / rank1 over n local columns.
  __device__ void rank1(const uint8_t* cx, const uint8_t* cz) {
    const int size = tm.size(), t = tm.t;
    const int words = SL >> 2;
    for (int g = t; g < n; g += size) DOT[g] = 0;
    tm.sync();
    const int R = size >= words ? size / words : 1;
    const int act = size >= words ? R * words : size;
    if (t < act) {
      const int w0 = size >= words ? t % words : t;
      const int rr = size >= words ? t / words : 0;
      const uint32_t* fws = reinterpret_cast<const uint32_t*>(FW);
      for (int w = w0; w < words; w += (size >= words ? words : size)) {
        const uint32_t fw = fws[w];
        if (fw == 0u) continue;
        int dots[4] = {0, 0, 0, 0};
        uint32_t* xcol = reinterpret_cast<uint32_t*>(X) + w;
        uint32_t* zcol = reinterpret_cast<uint32_t*>(Z) + w;
        const int S4 = SL >> 2;
        if constexpr (DD == 3 || DD == 5 || DD == 7) {
          // four residues per operation: f a <= (d-1)^2 and x + f a <= d^2 - d
          // stay inside a byte, and the dots z a add up in 16-bit lanes
          int k = rr;
          uint32_t dlo = 0u, dhi = 0u;
          int rows = 0;
          // four rows in flight: their loads are issued before any store
          for (; k + 3 * R < n; k += 4 * R) {
            uint32_t xw[4], zw[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              xw[i] = xcol[(size_t)(k + i * R) * S4];
              zw[i] = zcol[(size_t)(k + i * R) * S4];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const uint32_t a = cx[k + i * R], b = cz[k + i * R];
              dlo += (zw[i] & 0x00FF00FFu) * a;
              dhi += ((zw[i] >> 8) & 0x00FF00FFu) * a;
              xcol[(size_t)(k + i * R) * S4] = packed_mod<DD>(xw[i] + fw * a);
              zcol[(size_t)(k + i * R) * S4] = packed_mod<DD>(zw[i] + fw * b);
            }
            if ((rows += 4) >= 1024) {  // 1024 (d-1)^2 < 2^16
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
            uint32_t xw = xcol[(size_t)k * S4], zw = zcol[(size_t)k * S4];
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
          if (g < n && ((fw >> (8 * j)) & 0xff)) {
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
};

// One measurement (both CTAs of the pair run it).
template <int DD>
__device__ void split_measure(SplitU8<DD>& e, const TraceDescU8& td, int q, uint32_t mord, uint32_t nord,
                              bool reset) {
  e.tm.sync();
  const int size = e.tm.size(), t = e.tm.t;
  const int n = e.n, SL = e.SL, np = e.np, r = e.r, sw = td.sw;
  const ModU8<DD>& M = e.M;
  uint8_t* X = e.X;
  uint8_t* Z = e.Z;
  uint8_t* C = e.C;
  const uint8_t* xq = X + (size_t)q * SL;
  uint8_t* row = td.mrow + (size_t)mord * 2 * sw;
  uint8_t* b = e.buf(mord);
  int* bh = reinterpret_cast<int*>(b);  // p, s1, phc, ex
  uint8_t* bcx = b + 16;
  uint8_t* bcz = bcx + np;
  uint8_t* bf = bcz + np;
  const uint32_t peer = (uint32_t)(r ^ 1);
  // ---- phase A
  int p = INT_MAX, s1 = 0, phc = 0, ex = 1;
  if (r == 1) {
    for (int i = 4 * t; i < np; i += 4 * size) {
      uint32_t v = 0u;
#pragma unroll
      for (int j = 0; j < 4; ++j) v |= (uint32_t)(i + j < n ? xq[i + j] : 0) << (8 * j);
      st_peer_u32(peer_addr(bf + i, peer), v);
    }
  } else {
    int mine = INT_MAX;
    for (int g = t; g < n; g += size)
      if (xq[g]) {
        mine = g;
        break;
      }
    p = e.tm.min(mine);
    if (p < n) {
      const int xv = xq[p];
      if (xv != 1) {
        ex = M.inv(xv);
        int sl = 0;
        for (int k = t; k < n; k += size) sl += X[(size_t)k * SL + p] * Z[(size_t)k * SL + p];
        const int s0 = M.md(e.tm.add(sl));
        e.tm.sync();
        if (e.tm.leader()) C[p] = (uint8_t)M.mo(C[p] * ex + M.md(s0 * M.md((ex * (ex - 1)) >> 1)) * M.phi);
        for (int k = t; k < n; k += size) {
          X[(size_t)k * SL + p] = (uint8_t)M.md(X[(size_t)k * SL + p] * ex);
          Z[(size_t)k * SL + p] = (uint8_t)M.md(Z[(size_t)k * SL + p] * ex);
        }
        e.tm.sync();
      }
      int sl = 0;
      for (int k = t; k < np; k += size) {
        const int a = k < n ? X[(size_t)k * SL + p] : 0, bb = k < n ? Z[(size_t)k * SL + p] : 0;
        e.CX[k] = (uint8_t)a;
        e.CZ[k] = (uint8_t)bb;
        sl += a * bb;
      }
      s1 = M.md(e.tm.add(sl));
      phc = C[p];
      e.tm.sync();
      for (int i = 4 * t; i < np; i += 4 * size) {
        st_peer_u32(peer_addr(bcx + i, peer), *reinterpret_cast<const uint32_t*>(e.CX + i));
        st_peer_u32(peer_addr(bcz + i, peer), *reinterpret_cast<const uint32_t*>(e.CZ + i));
      }
    }
    if (e.tm.leader()) {
      st_peer_u32(peer_addr(bh + 0, peer), (uint32_t)p);
      st_peer_u32(peer_addr(bh + 1, peer), (uint32_t)s1);
      st_peer_u32(peer_addr(bh + 2, peer), (uint32_t)phc);
      st_peer_u32(peer_addr(bh + 3, peer), (uint32_t)ex);
    }
  }
  cluster_sync_all();
  // ---- phase B
  if (r == 1) {
    p = bh[0];
    s1 = bh[1];
    phc = bh[2];
  }
  if (p < n) {
    const uint8_t* cx = r == 0 ? e.CX : bcx;
    const uint8_t* cz = r == 0 ? e.CZ : bcz;
    for (int g = t; g < SL; g += size)
      e.FW[g] = (g < n && !(r == 0 && g == p)) ? (uint8_t)M.neg(xq[g]) : (uint8_t)0;
    e.tm.sync();
    for (int g = t; g < n; g += size) row[r * n + g] = e.FW[g];
    if (r == 1)
      for (int g = 2 * n + t; g < sw; g += size) row[g] = 0;
    e.rank1(cx, cz);
    for (int g = t; g < n; g += size) {
      const int f = e.FW[g];
      if (f == 0) continue;
      const int half = M.md(s1 * ((f * (f - 1)) >> 1));
      C[g] = (uint8_t)M.mo(C[g] + phc * f + M.phi * M.md(f * e.DOT[g]) + M.phi * M.phi * half);
    }
    e.tm.sync();
    // pivot columns: stabilizer p <- Z_q (CTA 0), destabilizer n + p <- old stabilizer p (CTA 1)
    for (int k = t; k < n; k += size) {
      if (r == 0) {
        X[(size_t)k * SL + p] = 0;
        Z[(size_t)k * SL + p] = (uint8_t)(k == q);
      } else {
        X[(size_t)k * SL + p] = cx[k];
        Z[(size_t)k * SL + p] = cz[k];
      }
    }
    if (e.tm.leader()) {
      C[p] = r == 0 ? (uint8_t)0 : (uint8_t)phc;
      if (r == 0) td.mhdr[mord] = make_uint4((reset ? 2u : 0u) | ((uint32_t)ex << 8), (uint32_t)p, nord, 0u);
    }
    e.tm.sync();
  } else if (r == 0) {
    // deterministic: f from CTA 1, stabilizer columns here
    for (int i = t; i < np; i += size) e.CX[i] = i < n ? bf[i] : (uint8_t)0;
    e.tm.sync();
    // sum_i f_i c_i here; the f_i (f_i - 1) / 2 (x_i . z_i) term is summed
    // row by row in the cross-term pass below (one pass over the tableau)
    int pl = 0, dl = 0;
    for (int i = t; i < n; i += size) {
      const int f = e.CX[i];
      if (f) pl += f * C[i];
    }
    int tl = 0;
    const int nw = (n + 3) >> 2;
    const uint32_t* fq = reinterpret_cast<const uint32_t*>(e.CX);
    for (int k = t; k < n; k += size) {
      const uint32_t* xr = reinterpret_cast<const uint32_t*>(X + (size_t)k * SL);
      const uint32_t* zr = reinterpret_cast<const uint32_t*>(Z + (size_t)k * SL);
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
    for (int g = t; g < sw; g += size) row[g] = g < n ? e.CX[g] : (uint8_t)0;
    e.tm.add3(pl, tl, dl);
    const int P = M.mo(pl);
    const int T = M.md(tl);
    const int Dd = M.md(dl);
    const int aphc = M.mo(P + M.phi * T + M.phi * M.phi * Dd);
    if (e.tm.leader()) td.mhdr[mord] = make_uint4(reset ? 3u : 1u, 0u, nord, (uint32_t)aphc);
    e.tm.sync();
  }
  if (reset) {
    e.tm.sync();
    const uint8_t* zq = Z + (size_t)q * SL;
    for (int g = t; g < n; g += size) row[sw + r * n + g] = zq[g];
    if (r == 1)
      for (int g = 2 * n + t; g < sw; g += size) row[sw + g] = 0;
  }
}

// Runs the shared part of td's program on the CTA pair and writes its trace.
template <int DD>
__device__ void split_program(const TraceDescU8& td, SplitU8<DD>& e, uint2* win, int* status) {
  const CircuitDesc& c = td.c;
  e.init();
  const int t = e.tm.t, size = e.tm.size();
  const int n = c.n, d = c.d, SL = e.SL, sw = td.sw, r = e.r;
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
    // both CTAs read the same stream and leave at the same instruction
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
        split_measure(e, td, q, mord, nord, op == OP_RESET);
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
          for (int g = t; g < n; g += size) {
            dst[r * n + g] = xr[g];
            dst[sw + r * n + g] = zr[g];
          }
          if (r == 1)
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
  cluster_sync_all();  // neither CTA leaves while its partner may still write into it
}


}  // namespace sdim
