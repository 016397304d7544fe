// Trace engine for odd prime d (residue bytes), device side.
//
// As for d = 2 (trace_bits.cuh), the x / z blocks and the common phase c of
// the shot-group engine (group_u8.cuh) are the same in every shot, so one
// CTA runs them once per program (the x / z pass, a TGroupU8 team with no
// live shots) and records what the per-shot phase deltas read:
//   mhdr[k] : x = bit 0 deterministic, bit 1 RESET, bits 8.. exponent e of
//             the pivot (random), y = pivot p, z = N1 ordinals before k,
//             w = common outcome phase aph_c (deterministic)
//   mrow[k][0][SW] : random: factors FW_g over the 2n generators;
//                    deterministic: f_i = destabilizer x_q[n + i], i < n
//   mrow[k][1][SW] : z_q after the measurement (RESET)
//   nrow[j][0..1][SW] : x_q, z_q at N1 ordinal j
// (SW = 2n rounded up to 16 bytes, rows zero past 2n).  The phase pass then
// replays every shot's delta (residues mod d over the 2n generators, in
// shared memory) exactly as the group engine applies it:
//   N1 fired (X^a Z^b)      : delta += (d - a) z_q + b x_q
//   random M (pivot p, e)   : delta_p *= e; delta_g += FW_g delta_p;
//                             delta_{n+p} = delta_p; delta_p = -m_s
//   deterministic M         : m_s = -(aph_c + sum_i f_i delta_i)
//   RESET                   : delta += m_s z_q
// with the same streams, so records match the other engines.  A CTA of the
// phase pass holds 32 shots; thread t serves shot t % 32 and the generators
// g = t / 32 (mod chunks).
#pragma once
#include "group_u8.cuh"
#include "kernels.cuh"
#include "trace.cuh"

namespace sdim {

// ---------------------------------------------------------------- x / z pass

template <int DD, class Team>
__device__ void trace_measure_u8(TGroupU8<DD, Team>& e, const TraceDescU8& td, int q, uint32_t mord, uint32_t nord,
                                 bool reset) {
  e.tm.sync();
  const int size = e.tm.size(), t = e.tm.t;
  const int n = e.n, S = e.S, sw = td.sw;
  const ModU8<DD>& M = e.M;
  uint8_t* X = e.X;
  uint8_t* Z = e.Z;
  uint8_t* C = e.C;
  const uint8_t* xq = X + (size_t)q * S;
  uint8_t* row = td.mrow + (size_t)mord * 2 * sw;
  int mine = INT_MAX;
  for (int g = t; g < n; g += size)
    if (xq[g]) {
      mine = g;
      break;
    }
  const int p = e.tm.min(mine);
  if (p < n) {
    const int xv = xq[p];
    int ex = 1;
    if (xv != 1) {
      ex = M.inv(xv);
      int sl = 0;
      for (int k = t; k < n; k += size) sl += X[(size_t)k * S + p] * Z[(size_t)k * S + p];
      const int s0 = M.md(e.tm.add(sl));
      e.tm.sync();
      if (e.tm.leader()) C[p] = (uint8_t)M.mo(C[p] * ex + M.md(s0 * M.md((ex * (ex - 1)) >> 1)) * M.phi);
      for (int k = t; k < n; k += size) {
        X[(size_t)k * S + p] = (uint8_t)M.md(X[(size_t)k * S + p] * ex);
        Z[(size_t)k * S + p] = (uint8_t)M.md(Z[(size_t)k * S + p] * ex);
      }
      e.tm.sync();
    }
    int sl = 0;
    for (int k = t; k < n; k += size) {
      const int a = X[(size_t)k * S + p], b = Z[(size_t)k * S + p];
      e.CX[k] = (uint8_t)a;
      e.CZ[k] = (uint8_t)b;
      sl += a * b;
    }
    for (int g = t; g < S; g += size) e.FW[g] = (g < 2 * n && g != p) ? (uint8_t)M.neg(xq[g]) : (uint8_t)0;
    const int s1 = M.md(e.tm.add(sl));
    const int phc = C[p];
    e.tm.sync();
    for (int g = t; g < sw; g += size) row[g] = g < 2 * n ? e.FW[g] : (uint8_t)0;
    e.rank1(p);
    for (int g = t; g < 2 * n; g += size) {
      const int f = e.FW[g];
      if (f == 0) continue;
      const int half = M.md(s1 * ((f * (f - 1)) >> 1));
      C[g] = (uint8_t)M.mo(C[g] + phc * f + M.phi * M.md(f * e.DOT[g]) + M.phi * M.phi * half);
    }
    e.tm.sync();
    for (int k = t; k < n; k += size) {
      X[(size_t)k * S + n + p] = e.CX[k];
      Z[(size_t)k * S + n + p] = e.CZ[k];
      X[(size_t)k * S + p] = 0;
      Z[(size_t)k * S + p] = (uint8_t)(k == q);
    }
    if (e.tm.leader()) {
      C[n + p] = (uint8_t)phc;
      C[p] = 0;
      td.mhdr[mord] = make_uint4((reset ? 2u : 0u) | ((uint32_t)ex << 8), (uint32_t)p, nord, 0u);
    }
    e.tm.sync();
  } else {
    for (int i = t; i < SlotU8::npad(n); i += size) e.CX[i] = i < n ? xq[n + i] : (uint8_t)0;
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
    const uint8_t* zq = Z + (size_t)q * S;
    for (int g = t; g < sw; g += size) row[sw + g] = g < 2 * n ? zq[g] : (uint8_t)0;
    e.tm.sync();
  }
}

// Column j of a group of cnt <= kGateGroup gates on pairwise disjoint qudits
// (ops: their instruction words, in shared memory): X, Z rows of `stride`
// bytes, phases C.  Every operand is loaded before any result is stored, so
// the loads of the group overlap; the gates commute and their phase terms
// add, so the order within the group does not matter.  Per gate the arithmetic of
// TGroupU8's h, h_inv, p, cnot and pauli (group_u8.cuh).
template <class Mod>
__device__ __forceinline__ void gate_group_column(const uint2* ops, int cnt, uint8_t* X, uint8_t* Z, size_t stride,
                                                  uint8_t* C, int j, const Mod& M) {
  // operands of gate g packed in v[g]: x_a | z_a << 8 | x_b << 16 | z_b << 24
  // (b: a CNOT's target), one register a gate
  uint32_t v[kGateGroup];
#pragma unroll
  for (int g = 0; g < kGateGroup; ++g) {
    if (g < cnt) {
      const uint2 w = ops[g];
      const size_t qa = (size_t)(w.x >> 8) * stride + j;
      uint32_t a = (uint32_t)X[qa] | ((uint32_t)Z[qa] << 8);
      const uint32_t op = w.x & kOpMask;
      if (op == OP_CNOT || op == OP_CNOT_INV) {
        const size_t qb = (size_t)w.y * stride + j;
        a |= ((uint32_t)X[qb] << 16) | ((uint32_t)Z[qb] << 24);
      }
      v[g] = a;
    }
  }
  int ph = C[j];
  const int d = M.d;
#pragma unroll
  for (int g = 0; g < kGateGroup; ++g) {
    if (g < cnt) {
      const uint2 w = ops[g];
      const size_t qa = (size_t)(w.x >> 8) * stride + j;
      const int x = (int)(v[g] & 0xffu), z = (int)((v[g] >> 8) & 0xffu);
      switch (w.x & kOpMask) {
        case OP_X: ph += M.phi * (d - 1) * z; break;
        case OP_X_INV: ph += M.phi * z; break;
        case OP_Z: ph += M.phi * x; break;
        case OP_Z_INV: ph += M.phi * (d - 1) * x; break;
        case OP_H: {
          const int nx = M.neg(z);
          ph += M.phi * nx * x;
          X[qa] = (uint8_t)nx;
          Z[qa] = (uint8_t)x;
          break;
        }
        case OP_H_INV: {
          const int nz = M.neg(x);
          ph += M.phi * z * nz;
          X[qa] = (uint8_t)z;
          Z[qa] = (uint8_t)nz;
          break;
        }
        case OP_P: ph += M.mo((x * (x - 1)) >> 1); Z[qa] = (uint8_t)M.md(z + x); break;
        case OP_P_INV: ph += M.ord - M.mo((x * (x - 1)) >> 1); Z[qa] = (uint8_t)M.md(z + d - x); break;
        case OP_CNOT:
        case OP_CNOT_INV: {
          const int xb = (int)((v[g] >> 16) & 0xffu), zb = (int)(v[g] >> 24);
          const bool inv = (w.x & kOpMask) == OP_CNOT_INV;
          X[(size_t)w.y * stride + j] = (uint8_t)M.md(inv ? xb + d - x : xb + x);
          Z[qa] = (uint8_t)M.md(inv ? z + zb : z + d - zb);
          break;
        }
        default: break;
      }
    }
  }
  C[j] = (uint8_t)M.mo(ph);
}

// Runs the shared part of td's program and writes its trace; win: room for
// kOpWindow instructions in shared memory.
template <int DD, class Team>
__device__ void trace_program_u8(const TraceDescU8& td, TGroupU8<DD, Team>& e, uint2* win, int* status) {
  const CircuitDesc& c = td.c;
  e.init(0);
  const int t = e.tm.t, size = e.tm.size();
  const int n = c.n, d = c.d, S = e.S, sw = td.sw;
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
        trace_measure_u8(e, td, q, mord, nord, op == OP_RESET);
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
          // column g of row q was last written by thread g mod size: no barrier needed
          const uint8_t* xr = e.X + (size_t)q * S;
          const uint8_t* zr = e.Z + (size_t)q * S;
          uint8_t* dst = td.nrow + (size_t)nord * 2 * sw;
          for (int g = t; g < sw; g += size) {
            dst[g] = g < 2 * n ? xr[g] : (uint8_t)0;
            dst[sw + g] = g < 2 * n ? zr[g] : (uint8_t)0;
          }
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

// ---------------------------------------------------------------- phase pass

// Shared memory of a phase-pass CTA: deltas D[32][sd] (sd = SlotU8::stride),
// two staging buffers of a measurement's rows (2 x 2 sw bytes), then ints
// shot_m[32], shot_acc[32], shot_ab[32].
__host__ __device__ inline size_t phase_u8_smem(int n) {
  return (size_t)32 * SlotU8::stride(n) + (size_t)4 * trace_row_bytes_u8(n) + 4 * 32 * 3;
}

// Starts the copy of measurement k's two rows (2 sw bytes, 16-byte chunks)
// into buf with cp.async; the caller commits the group.
__device__ __forceinline__ void stage_rows_u8(const uint8_t* src, uint8_t* buf, int bytes, int t, int nt) {
  for (int i = 16 * t; i < bytes; i += 16 * nt) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(buf + i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src + i) : "memory");
  }
}

// One 32-shot group of td; the CTA's threads are (shot, chunk) pairs.  The
// rows of measurement k + 1 are copied into shared memory while k runs.
template <int DD>
__device__ void phase_program_u8(const TraceDescU8* __restrict__ tdp, long long group, uint8_t* smem) {
  const int t = threadIdx.x, nt = blockDim.x;
  const int s = t & 31, ch = t >> 5, nch = nt >> 5;
  const CircuitDesc c = tdp->c;
  const int n = c.n, d = c.d, sw = tdp->sw, nm = tdp->nm;
  const uint32_t nn1 = (uint32_t)tdp->nn1;
  const ModU8<DD> M(d);
  const int sd = SlotU8::stride(n);
  uint8_t* ds = smem + (size_t)s * sd;
  uint8_t* rows = smem + (size_t)32 * sd;  // [2][2 sw]
  int* shot_m = reinterpret_cast<int*>(rows + 4 * (size_t)sw);
  int* shot_acc = shot_m + 32;
  int* shot_ab = shot_acc + 32;
  const long long rel = group * 32 + s;
  const bool live = rel < (long long)c.nshots;
  const long long shot = c.shot0 + rel;
  uint8_t* out = c.out + (live ? rel : 0) * (long long)c.nmeas;
  const uint8_t* mrow = tdp->mrow;
  for (int i = t; i < 32 * sd / 4; i += nt) reinterpret_cast<uint32_t*>(smem)[i] = 0u;
  if (nm > 0) stage_rows_u8(mrow, rows, 2 * sw, t, nt);
  asm volatile("cp.async.commit_group;" ::: "memory");
  uint4 hn = nm > 0 ? __ldg(tdp->mhdr) : make_uint4(0u, 0u, 0u, 0u);
  CoinCache coins;
  uint32_t nord = 0;
  for (int k = 0; k < nm; ++k) {
    const uint4 h = hn;
    if (k + 1 < nm) {
      hn = __ldg(tdp->mhdr + k + 1);
      stage_rows_u8(mrow + (size_t)(k + 1) * 2 * sw, rows + (size_t)((k + 1) & 1) * 2 * sw, 2 * sw, t, nt);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 1;" ::: "memory");  // this measurement's rows have landed
    __syncthreads();
    const uint32_t nend = h.z < nn1 ? h.z : nn1;
    for (; nord < nend; ++nord) {
      const uint2 nh = __ldg(tdp->nhdr + nord);
      if (nh.y == OP_N1OFF) continue;
      int fire = 0;
      if (ch == 0) {
        int ab = 0;
        if (live && coins.coin(c.seed, shot, nord) >= nh.x) {
          const int2 v = noise_choice(nh.y, d, c.seed, shot, nord);
          ab = (v.x ? d - v.x : 0) | (v.y << 8);
          fire = 1;
        }
        shot_ab[s] = ab;
      }
      if (__syncthreads_or(fire)) {
        const int ab = shot_ab[s];
        const int cz = ab & 0xff, cx = ab >> 8;
        if (cz | cx) {
          const uint8_t* xr = tdp->nrow + (size_t)nord * 2 * sw;
          const uint8_t* zr = xr + sw;
          for (int g = ch; g < 2 * n; g += nch) ds[g] = (uint8_t)M.mo(ds[g] + M.phi * (cz * zr[g] + cx * xr[g]));
        }
        __syncthreads();
      }
    }
    const uint8_t* row = rows + (size_t)(k & 1) * 2 * sw;
    const bool det = h.x & 1u;
    // d in {3, 5, 7}: four residues per 32-bit word (packed_mod, __dp4a)
    constexpr bool kPacked = DD == 3 || DD == 5 || DD == 7;
    uint32_t* dw = reinterpret_cast<uint32_t*>(ds);
    const uint32_t* rw = reinterpret_cast<const uint32_t*>(row);
    const int nw2 = (2 * n + 3) >> 2, nw1 = (n + 3) >> 2;
    if (!det) {
      const int p = (int)h.y, ex = (int)(h.x >> 8);
      if (ex != 1) {
        if (ch == 0) ds[p] = (uint8_t)M.mo(ds[p] * ex);
        __syncthreads();
      }
      const int dp = ds[p];  // the rowsum below never writes generator p (FW_p = 0)
      if (dp) {
        if constexpr (kPacked) {
          for (int w = ch; w < nw2; w += nch) {
            const uint32_t fw = rw[w];
            if (fw) dw[w] = packed_mod<DD>(dw[w] + fw * (uint32_t)dp);
          }
        } else {
          for (int g = ch; g < 2 * n; g += nch) {
            const int f = row[g];
            if (f) ds[g] = (uint8_t)M.mo(ds[g] + f * dp);
          }
        }
      }
      __syncthreads();
      if (ch == 0) {
        const int m = live ? mulshift(stream_block(c.seed, shot, (uint32_t)k, 0u).x, (uint32_t)d) : 0;
        ds[n + p] = (uint8_t)dp;
        ds[p] = (uint8_t)M.mo(M.ord - M.mo(m * M.phi));
        shot_m[s] = m;
      }
    } else {
      if (ch == 0) shot_acc[s] = 0;
      __syncthreads();
      int acc = 0;
      if constexpr (kPacked) {
        // factor bytes past n are zero, so whole words of the first n generators add up
        for (int w = ch; w < nw1; w += nch) acc = (int)__dp4a(rw[w], dw[w], (unsigned)acc);
      } else {
        for (int i = ch; i < n; i += nch) {
          const int f = row[i];
          if (f) acc += f * ds[i];
        }
      }
      if (acc) atomicAdd(&shot_acc[s], acc);
      __syncthreads();
      if (ch == 0) shot_m[s] = M.md(M.d - M.mo((int)h.w + M.mo(shot_acc[s])));
    }
    __syncthreads();
    const int m = shot_m[s];
    if ((h.x & 2u) && m) {
      const uint8_t* zq = row + sw;
      if constexpr (kPacked) {
        const uint32_t* zw = reinterpret_cast<const uint32_t*>(zq);
        for (int w = ch; w < nw2; w += nch) {
          const uint32_t z = zw[w];
          if (z) dw[w] = packed_mod<DD>(dw[w] + z * (uint32_t)m);
        }
      } else {
        for (int g = ch; g < 2 * n; g += nch) ds[g] = (uint8_t)M.mo(ds[g] + M.phi * m * zq[g]);
      }
    }
    if (ch == 0 && live && k < c.nmeas) out[k] = (uint8_t)(m | ((int)det << 7));
    __syncthreads();  // the deltas are final, and buffer k & 1 is free for measurement k + 2
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ int find_trace_desc_u8(const TraceDescU8* descs, int ndesc, long long it) {
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (descs[mid].c.item_begin <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace sdim
