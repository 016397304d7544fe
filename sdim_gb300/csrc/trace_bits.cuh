// Trace engine for d = 2, device side.
//
// The shot-group engine (group_bits.cuh) rests on x / z and the common phase
// c following the same updates in every shot, with only delta_s (ph_s = c +
// delta_s mod 4) depending on the shot's outcomes and noise.  Nothing forces
// the sharing to stop at 32 shots: the x / z pass runs x / z / c once per
// program and records in a trace (trace.cuh) every value the delta updates
// read; the phase pass then gives every shot a lane (or half of one),
// delta_s in registers (its high bit plane over the 2n generators, TW words;
// the low plane is always zero, see phase_program), and replays
//   N1 before measurement k : coin per ordinal; on a fire with Pauli
//                             X^a Z^b, delta ^= 2 (a z_q + b x_q)
//   random M (pivot p)      : delta_g += delta_p for g in FW;
//                             delta_{n+p} = delta_p; delta_p = 2 m_s with
//                             m_s from the outcome stream
//   deterministic M         : m_s = (aph_c + sum_{i in f} delta_i) / 2
//   RESET                   : delta ^= 2 m_s z_q
// exactly as the group engine applies them, so records are identical to the
// group and per-shot engines (same streams, same arithmetic).  N1 after the
// last measurement changes no record and is not replayed.
//
// The x / z pass is one CTA per program walking the host-built layered
// schedule instead of the instruction stream:
//   gate layer : ops on pairwise disjoint qudits touch disjoint rows; their
//                common-phase updates are xors into C1 (atomicXor), except a
//                P's carry into C0, and a layer holds at most one P.  Every
//                (op, word) pair is one task.
//   measurement block (consecutive M / RESET): a deterministic measurement
//                only reads the tableau, so the pivot searches of the whole
//                block run at once, every deterministic measurement before
//                the first random one is evaluated in parallel (one task per
//                (measurement, qudit row) for the cross term), the random one
//                runs on the whole CTA, and the rest of the block repeats.
#pragma once
#include "group_bits.cuh"
#include "kernels.cuh"
#include "trace.cuh"

namespace sdim {

// Measurements of a block handled per round of the block loop (scratch size).
constexpr int kTraceBlockMeas = 256;

using TraceTab = TGroupBits<CtaTeam>;

// ---------------------------------------------------------------- x / z pass

// Word w of N1 ordinal j's rows (x_q, z_q).
__device__ __forceinline__ void n1_rows(const TraceDesc& td, uint32_t j, int w, uint32_t x, uint32_t z, int* status) {
  if ((int)j >= td.nn1) {
    atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
    return;
  }
  uint32_t* dst = td.nrow + (size_t)j * 2 * td.tw;
  dst[w] = x;
  dst[td.tw + w] = z;
}

// Word w of one op of a gate layer (w in [0, tw); words past 2 Wn only pad
// the N1 rows with zeros).  A gate entry's z (w) holds 1 + the ordinal of an
// N1 on its qudit (target) that follows it with no op on that qudit between
// (the host scheduler folds it in): the same thread writes that N1's rows
// from the words it just produced.
__device__ __forceinline__ void layer_word(TraceTab& e, const TraceDesc& td, const uint4 lo, int w, int* status) {
  const uint32_t op = lo.x & kOpMask;
  const int q = (int)(lo.x >> 8);
  const int n = e.n, W2 = e.W2, RS = e.RS;
  if (q >= n) {
    atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
    return;
  }
  const bool in = w < W2;
  uint32_t* xr = e.X + (size_t)q * RS;
  uint32_t* zr = e.Z + (size_t)q * RS;
  uint32_t xa = 0u, za = 0u;  // word w of x_q, z_q after the op (0 past 2 Wn)
  switch (op) {
    case OP_H:
    case OP_H_INV:
      if (in) {
        const uint32_t x = xr[w], z = zr[w];
        if (x & z) atomicXor(&e.C1[w], x & z);
        xr[w] = z;
        zr[w] = x;
        xa = z;
        za = x;
      }
      break;
    case OP_P:
    case OP_P_INV:
      if (in) {
        const uint32_t x = xr[w], lo0 = e.C0[w];
        const uint32_t c = (op == OP_P_INV) ? (~lo0 & x) : (lo0 & x);
        e.C0[w] = lo0 ^ x;  // the layer's only P
        if (c) atomicXor(&e.C1[w], c);
        za = zr[w] ^ x;
        zr[w] = za;
        xa = x;
      }
      break;
    case OP_CNOT:
    case OP_CNOT_INV: {
      const int tq = (int)lo.y;
      if (tq >= n) {
        atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
        return;
      }
      uint32_t xb = 0u, zb = 0u;
      if (in) {
        uint32_t* xt = e.X + (size_t)tq * RS + w;
        const uint32_t zt = e.Z[(size_t)tq * RS + w];
        xa = xr[w];
        xb = *xt ^ xa;
        *xt = xb;
        za = zr[w] ^ zt;
        zr[w] = za;
        zb = zt;
      }
      if (lo.w) n1_rows(td, lo.w - 1u, w, xb, zb, status);
      break;
    }
    case OP_X:
    case OP_X_INV:  // d = 2: phase += 2 z_q
      if (in) {
        xa = xr[w];
        za = zr[w];
        if (za) atomicXor(&e.C1[w], za);
      }
      break;
    case OP_Z:
    case OP_Z_INV:  // d = 2: phase += 2 x_q
      if (in) {
        xa = xr[w];
        za = zr[w];
        if (xa) atomicXor(&e.C1[w], xa);
      }
      break;
    case OP_N1D:
    case OP_N1F:
    case OP_N1P:
    case OP_N1OFF:  // an N1 of its own: its ordinal in z
      n1_rows(td, lo.z, w, in ? xr[w] : 0u, in ? zr[w] : 0u, status);
      return;
    case OP_NOP:
      return;
    default:
      atomicCAS(status, DEV_OK, DEV_BAD_OPCODE);
      return;
  }
  if (lo.z) n1_rows(td, lo.z - 1u, w, xa, za, status);  // a gate's folded N1
}

// Ordinal of entry k of a block in the program's measurement order: its own
// for an M / RESET (z), the next measurement's for an N1 (w, set by the host
// scheduler), so ordinal(r) - ordinal(s) counts the measurements in [s, r).
__device__ __forceinline__ uint32_t block_ordinal(const uint4* M, int k, int B) {
  if (k >= B) {
    const uint4 m = M[B - 1];
    const uint32_t op = m.x & kOpMask;
    return (op == OP_M || op == OP_RESET) ? m.z + 1u : m.w;
  }
  const uint4 m = M[k];
  const uint32_t op = m.x & kOpMask;
  return (op == OP_M || op == OP_RESET) ? m.z : m.w;
}

// The snapshot a run of deterministic entries M[s..r) takes (trace.cuh:
// TraceDesc::snap), or -1 for none: no measurement among them, no snapshot
// buffer, or all its slots used (then the cross terms are summed here).
// Read by every thread before the barrier after trace_det_tasks; sc[2]
// counts the slots used and advances in trace_det_headers.
__device__ __forceinline__ int det_snapshot(const TraceDesc& td, const uint4* M, int s, int r, int B, const int* sc) {
  if (!td.snap || block_ordinal(M, r, B) == block_ordinal(M, s, B)) return -1;
  return sc[2] < td.nsnap ? sc[2] : -1;
}

// Work of entries M[s..r) of a block -- deterministic measurements and N1 --
// all on the current tableau, without barriers (M may point into shared
// memory: plain loads).  tacc / pacc of the entries must be zero.  With a
// snapshot slot (snap >= 0) the stabilizer halves of x and z go there and
// the cross terms are left to the header pass (k_header_pass), which sums
// them on all SMs; they are this pass's largest share of work on its one SM.
__device__ __forceinline__ void trace_det_tasks(TraceTab& e, const TraceDesc& td, const uint4* M, int s, int r,
                                                int* tacc, int* pacc, int* status, int snap) {
  const int t = e.tm.t, size = e.tm.size();
  const int n = e.n, Wn = e.Wn, W2 = e.W2, RS = e.RS, tw = td.tw;
  const int cnt = r - s;
  const int lg = __ffs(tw) - 1;
  // N1 rows; common part of the factor sum, factor rows, RESET rows
  for (int task = t; task < (cnt << lg); task += size) {
    const int k = s + (task >> lg), w = task & (tw - 1);
    const uint4 m = M[k];
    const uint32_t op = m.x & kOpMask;
    if (op != OP_M && op != OP_RESET) {
      layer_word(e, td, m, w, status);
      continue;
    }
    const int q = (int)(m.x >> 8);
    uint32_t* row = td.mrow + (size_t)m.z * 2 * tw;
    uint32_t f = 0u;
    if (w < Wn) {
      f = e.X[(size_t)q * RS + Wn + w];
      const int pl = __popc(f & e.C0[w]) + 2 * __popc(f & e.C1[w]);
      if (pl) atomicAdd(&pacc[k], pl);
    }
    row[w] = f;
    if (op == OP_RESET) row[tw + w] = w < W2 ? e.Z[(size_t)q * RS + w] : 0u;
  }
  if (snap >= 0) {
    uint32_t* sx = td.snap + (size_t)snap * 2 * n * Wn;
    uint32_t* sz = sx + (size_t)n * Wn;
    for (int i = t; i < n * Wn; i += size) {
      const int k = i / Wn, w = i - k * Wn;
      sx[i] = e.X[(size_t)k * RS + w];
      sz[i] = e.Z[(size_t)k * RS + w];
    }
    return;
  }
  // cross term T: one task per (entry, qudit row), walked without divisions
  int kk = t / n, kr = t - (t / n) * n;
  const int dk = size / n, dr = size - (size / n) * n;
  for (; kk < cnt; kk += dk, kr += dr) {
    if (kr >= n) {
      kr -= n;
      ++kk;
      if (kk >= cnt) break;
    }
    const uint4 m = M[s + kk];
    const uint32_t op = m.x & kOpMask;
    if (op != OP_M && op != OP_RESET) continue;
    const uint32_t* fq = e.X + (size_t)(m.x >> 8) * RS + Wn;
    const uint32_t* xr = e.X + (size_t)kr * RS;
    const uint32_t* zr = e.Z + (size_t)kr * RS;
    uint32_t carry = 0u, tpar = 0u;
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
    if (tpar) atomicXor(&tacc[s + kk], 1);
  }
}

// Trace headers of the deterministic measurements among M[s..r) (after the
// barrier that ends trace_det_tasks).  With a snapshot the header carries
// flag 4 and the slot in y, and w holds the phase without the cross term.
__device__ __forceinline__ void trace_det_headers(TraceTab& e, const TraceDesc& td, const uint4* M, int s, int r,
                                                  const int* tacc, const int* pacc, int snap, int* sc) {
  for (int k = s + e.tm.t; k < r; k += e.tm.size()) {
    const uint4 m = M[k];
    const uint32_t op = m.x & kOpMask;
    if (op != OP_M && op != OP_RESET) continue;
    const uint32_t flags = (op == OP_RESET ? 3u : 1u) | (snap >= 0 ? 4u : 0u);
    td.mhdr[m.z] = make_uint4(flags, snap >= 0 ? (uint32_t)snap : 0u, m.w, (uint32_t)((pacc[k] + 2 * tacc[k]) & 3));
  }
  if (e.tm.t == 0 && snap >= 0) sc[2] = snap + 1;
}

// A random measurement with pivot p, on the whole CTA: the rowsum (two
// barriers inside), one barrier, then the pivot columns, the factor row and
// the header in one phase (and the RESET row after one more barrier).  The
// caller's next phase must not touch x / z before its own barrier.
__device__ void trace_random(TraceTab& e, const TraceDesc& td, const uint4 m, int p) {
  const int t = e.tm.t, size = e.tm.size();
  const int n = e.n, Wn = e.Wn, W2 = e.W2, RS = e.RS, tw = td.tw;
  const int q = (int)(m.x >> 8);
  const bool reset = (m.x & kOpMask) == OP_RESET;
  const int wp = p >> 5, bp = p & 31, wd = Wn + wp;
  const uint32_t pbit = 1u << bp;
  const int phc = (int)((e.C0[wp] >> bp) & 1u) | (int)(((e.C1[wp] >> bp) & 1u) << 1);
  e.rowsum(q, p, phc);
  e.tm.sync();
  uint32_t* row = td.mrow + (size_t)m.z * 2 * tw;
  for (int w = t; w < tw; w += size) row[w] = w < W2 ? e.FW[w] : 0u;
  for (int k = t; k < n; k += size) {
    uint32_t* xr = e.X + (size_t)k * RS;
    uint32_t* zr = e.Z + (size_t)k * RS;
    const uint32_t xs = xr[wp], zs = zr[wp];
    xr[wd] = (xr[wd] & ~pbit) | (xs & pbit);
    zr[wd] = (zr[wd] & ~pbit) | (zs & pbit);
    xr[wp] = xs & ~pbit;
    zr[wp] = (zs & ~pbit) | ((k == q) ? pbit : 0u);
  }
  if (e.tm.leader()) {
    e.C0[wd] = (e.C0[wd] & ~pbit) | ((uint32_t)(phc & 1) << bp);
    e.C1[wd] = (e.C1[wd] & ~pbit) | ((uint32_t)(phc >> 1) << bp);
    e.C0[wp] &= ~pbit;
    e.C1[wp] &= ~pbit;
    td.mhdr[m.z] = make_uint4(reset ? 2u : 0u, (uint32_t)p, m.w, 0u);
  }
  if (reset) {
    e.tm.sync();
    const uint32_t* zq = e.Z + (size_t)q * RS;
    for (int w = t; w < tw; w += size) row[tw + w] = w < W2 ? zq[w] : 0u;
  }
}

// A block of consecutive M / RESET with the N1 between them (schedule ops
// L[0..count), in shared or global memory).  Per round of the loop: find the
// first random measurement r at or after s (one atomicMin), evaluate the
// deterministic entries before it and r's pivot in the same phase, write
// their headers and run r.  sc: three ints of scratch (the third counts
// snapshot slots).
__device__ void trace_block(TraceTab& e, const TraceDesc& td, const uint4* L, int count, int* sc, int* tacc,
                            int* pacc, int* status) {
  const int t = e.tm.t, size = e.tm.size();
  const int n = e.n, Wn = e.Wn, RS = e.RS;
  for (int c0 = 0; c0 < count; c0 += kTraceBlockMeas) {
    const int B = min(kTraceBlockMeas, count - c0);
    const uint4* M = L + c0;
    for (int k = t; k < B; k += size) {
      const uint4 m = M[k];
      const uint32_t op = m.x & kOpMask;
      const bool meas = op == OP_M || op == OP_RESET;
      if ((int)(m.x >> 8) >= n || (meas ? (int)m.z >= td.nm : (int)m.z >= td.nn1))
        atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
    }
    if (e.tm.any(*(volatile int*)status != DEV_OK)) return;
    int s = 0;
    while (s < B) {
      if (t == 0) {
        sc[0] = INT_MAX;
        sc[1] = INT_MAX;
      }
      for (int k = s + t; k < B; k += size) {
        tacc[k] = 0;
        pacc[k] = 0;
      }
      e.tm.sync();
      for (int task = t; task < (B - s) * Wn; task += size) {
        const int kk = task / Wn, w = task - kk * Wn;
        const uint4 m = M[s + kk];
        const uint32_t op = m.x & kOpMask;
        if (op != OP_M && op != OP_RESET) continue;
        if (e.X[(size_t)(m.x >> 8) * RS + w]) atomicMin(&sc[0], s + kk);
      }
      e.tm.sync();
      const int first = sc[0];
      const int r = first == INT_MAX ? B : first;
      if (r < B && t < Wn) {
        const uint32_t v = e.X[(size_t)(M[r].x >> 8) * RS + t];
        if (v) atomicMin(&sc[1], (t << 5) + __ffs(v) - 1);
      }
      const int snap = r > s ? det_snapshot(td, M, s, r, B, sc) : -1;
      if (r > s) trace_det_tasks(e, td, M, s, r, tacc, pacc, status, snap);
      e.tm.sync();
      if (r > s) trace_det_headers(e, td, M, s, r, tacc, pacc, snap, sc);
      if (r < B) trace_random(e, td, M[r], sc[1]);
      s = r + 1;
    }
    e.tm.sync();
  }
}

// Row groups of the fused random-measurement phase: W2p threads (the
// factor words rounded up to a power of two) per group, all in one warp, and
// at most 32 tableau rows per thread, so a thread's pivot bits fit one word.
__device__ __forceinline__ bool trace_fused_rows(const TraceTab& e) {
  int W2p = 1;
  while (W2p < e.W2) W2p <<= 1;
  const int R = e.tm.size() / W2p;
  return W2p <= 32 && R > 0 && (e.n + R - 1) / R <= 32;
}

// First entry at or after s of a block whose x_q has a set bit in the
// stabilizer half (the next random measurement) into *first.
__device__ __forceinline__ void trace_pivot_search(const TraceTab& e, const uint4* M, int s, int B, int* first) {
  const int t = e.tm.t, size = e.tm.size(), Wn = e.Wn, RS = e.RS;
  for (int task = t; task < (B - s) * Wn; task += size) {
    const int kk = task / Wn, w = task - kk * Wn;
    const uint4 m = M[s + kk];
    const uint32_t op = m.x & kOpMask;
    if (op != OP_M && op != OP_RESET) continue;
    if (e.X[(size_t)(m.x >> 8) * RS + w]) atomicMin(first, s + kk);
  }
}

// trace_block with three CTA barriers per random measurement instead of six
// or seven (when trace_fused_rows holds).  A round of the loop:
//   phase 1 (after the pivot search's barrier): r = the first random entry;
//     its pivot p (atomicMin), its factor words FW = x_q (bit p cleared when
//     read), CW = 0, and the deterministic entries before r evaluated;
//   phase 2 (barrier C): their headers; the rowsum of the rows with x_p = 1
//     by rows, the pivot columns folded in: each row group of W2p threads is
//     one warp, reads the pivot bits of all its rows before any of its
//     threads writes (__syncwarp), and writes only its own words, so the
//     pivot-column fix-ups need no barrier; commute parities into CW;
//   phase 3 (barrier E): the common phase words and their pivot bits, the
//     factor row, the header and the RESET row; and the next round's pivot
//     search, whose barrier starts the next round.
// Rounds with no random entry left end the block after phase 2's headers.
__device__ void trace_block_fused(TraceTab& e, const TraceDesc& td, const uint4* L, int count, int* sc, int* tacc,
                                  int* pacc, int* status) {
  const int t = e.tm.t, size = e.tm.size();
  const int n = e.n, Wn = e.Wn, W2 = e.W2, RS = e.RS, tw = td.tw;
  int W2p = 1;
  while (W2p < W2) W2p <<= 1;
  const int R = size / W2p;
  const int gw = t & (W2p - 1), gr = t / W2p;  // word and row group of this thread
  const bool gact = gw < W2 && gr < R;
  const unsigned gbase = (unsigned)(t & 31) & ~(unsigned)(W2p - 1);
  const unsigned gmask = (W2 >= 32 ? 0xffffffffu : ((1u << W2) - 1u)) << gbase;
  for (int c0 = 0; c0 < count; c0 += kTraceBlockMeas) {
    const int B = min(kTraceBlockMeas, count - c0);
    const uint4* M = L + c0;
    for (int k = t; k < B; k += size) {
      const uint4 m = M[k];
      const uint32_t op = m.x & kOpMask;
      const bool meas = op == OP_M || op == OP_RESET;
      if ((int)(m.x >> 8) >= n || (meas ? (int)m.z >= td.nm : (int)m.z >= td.nn1))
        atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      tacc[k] = 0;
      pacc[k] = 0;
    }
    if (t == 0) {
      sc[0] = INT_MAX;
      sc[1] = INT_MAX;
    }
    if (e.tm.any(*(volatile int*)status != DEV_OK)) return;
    trace_pivot_search(e, M, 0, B, &sc[0]);  // the first round's
    e.tm.sync();
    int s = 0;
    while (s < B) {
      // phase 1
      const int first = sc[0];
      const int r = first == INT_MAX ? B : first;
      const int qr = r < B ? (int)(M[r].x >> 8) : 0;
      if (r < B) {
        if (t < Wn) {
          const uint32_t v = e.X[(size_t)qr * RS + t];
          if (v) atomicMin(&sc[1], (t << 5) + __ffs(v) - 1);
        }
        for (int w = t; w < W2; w += size) {
          e.FW[w] = e.X[(size_t)qr * RS + w];
          e.CW[w] = 0u;
        }
      }
      const int snap = r > s ? det_snapshot(td, M, s, r, B, sc) : -1;
      if (r > s) trace_det_tasks(e, td, M, s, r, tacc, pacc, status, snap);
      e.tm.sync();  // C
      // phase 2
      if (r > s) trace_det_headers(e, td, M, s, r, tacc, pacc, snap, sc);
      if (r >= B) break;
      const uint4 mr = M[r];
      const int p = sc[1];
      const int wp = p >> 5, bp = p & 31, wd = Wn + wp;
      const uint32_t pbit = 1u << bp;
      const int phc = (int)((e.C0[wp] >> bp) & 1u) | (int)(((e.C1[wp] >> bp) & 1u) << 1);
      if (t == 0) sc[0] = INT_MAX;  // r was read by every thread before barrier C
      uint32_t F = 0u, Cp = 0u;
      if (gact) {
        F = e.FW[gw];
        if (gw == wp) F &= ~pbit;
        uint32_t xpm = 0u, zpm = 0u;
        int i = 0;
        for (int k = gr; k < n; k += R, ++i) {
          xpm |= ((e.X[(size_t)k * RS + wp] >> bp) & 1u) << i;
          zpm |= ((e.Z[(size_t)k * RS + wp] >> bp) & 1u) << i;
        }
        __syncwarp(gmask);  // the group's pivot bits are read before any of its threads writes
        i = 0;
        for (int k = gr; k < n; k += R, ++i) {
          uint32_t* xr = e.X + (size_t)k * RS;
          uint32_t* zr = e.Z + (size_t)k * RS;
          const uint32_t xpk = (xpm >> i) & 1u, zpk = (zpm >> i) & 1u;
          const uint32_t zk = zr[gw];
          Cp ^= zk & (0u - xpk);
          uint32_t xn = xr[gw] ^ (F & (0u - xpk));
          uint32_t zn = zk ^ (F & (0u - zpk));
          if (gw == wd) {  // x_{n+p}, z_{n+p} := the pivot bits before the rowsum
            xn = (xn & ~pbit) | (xpk << bp);
            zn = (zn & ~pbit) | (zpk << bp);
          } else if (gw == wp) {  // x_p := 0, z_p := [k == q]
            xn &= ~pbit;
            zn = (zn & ~pbit) | (k == qr ? pbit : 0u);
          }
          xr[gw] = xn;
          zr[gw] = zn;
        }
      }
      // commute parities: the row groups of a warp by shuffles, then one
      // atomic per warp and word
      if (W2p < 32)
        for (int off = W2p; off < 32; off <<= 1) Cp ^= __shfl_xor_sync(0xffffffffu, Cp, off);
      if (gact && (t & 31) < W2p && Cp) atomicXor(&e.CW[gw], Cp);
      e.tm.sync();  // E
      // phase 3
      const bool reset = (mr.x & kOpMask) == OP_RESET;
      uint32_t* row = td.mrow + (size_t)mr.z * 2 * tw;
      if (gact && gr == 0) {
        const uint32_t lo_m = (phc & 1) ? 0xffffffffu : 0u;
        const uint32_t hi_m = (phc & 2) ? 0xffffffffu : 0u;
        const uint32_t lo = e.C0[gw];
        const uint32_t a_lo = F & lo_m;
        uint32_t c0 = lo ^ a_lo;
        uint32_t c1 = e.C1[gw] ^ (F & (hi_m ^ e.CW[gw])) ^ (lo & a_lo);
        if (gw == wd) {
          c0 = (c0 & ~pbit) | ((uint32_t)(phc & 1) << bp);
          c1 = (c1 & ~pbit) | ((uint32_t)(phc >> 1) << bp);
        } else if (gw == wp) {
          c0 &= ~pbit;
          c1 &= ~pbit;
        }
        e.C0[gw] = c0;
        e.C1[gw] = c1;
      }
      for (int w = t; w < tw; w += size) {
        uint32_t f = w < W2 ? e.FW[w] : 0u;
        if (w == wp) f &= ~pbit;
        row[w] = f;
        if (reset) row[tw + w] = w < W2 ? e.Z[(size_t)qr * RS + w] : 0u;
      }
      if (t == 0) {
        td.mhdr[mr.z] = make_uint4(reset ? 2u : 0u, (uint32_t)p, mr.w, 0u);
        sc[1] = INT_MAX;
      }
      // the next round's pivot search (x / z are final since barrier E)
      s = r + 1;
      trace_pivot_search(e, M, s, B, &sc[0]);
      e.tm.sync();  // the next round's pivot-search barrier
    }
    e.tm.sync();
  }
}

// Runs the shared part of td's program over its layered schedule and writes
// the trace.  Each schedule window is staged in shared memory (win: room for
// kTraceWinSteps steps, then kTraceWinOps ops) with one cooperative load.
__device__ void trace_program(const TraceDesc& td, TraceTab& e, uint4* win, int* sc, int* tacc, int* pacc,
                              int* status) {
  e.init(0);
  const int t = e.tm.t, size = e.tm.size(), tw = td.tw;
  if (t == 0) sc[2] = 0;  // snapshot slots used (the window load's barrier publishes it)
  const int lg = __ffs(tw) - 1;
  const bool fused = trace_fused_rows(e);
  uint4* wsteps = win;
  uint4* wops = win + kTraceWinSteps;
  for (int wi = 0; wi < td.nwins; ++wi) {
    const uint4 wd = __ldg(td.wins + wi);
    const int nst = min((int)wd.y, kTraceWinSteps);
    const bool staged = wd.w <= (uint32_t)kTraceWinOps;
    for (int i = t; i < nst; i += size) wsteps[i] = __ldg(td.steps + wd.x + i);
    if (staged)
      for (int i = t; i < (int)wd.w; i += size) wops[i] = __ldg(td.lops + wd.z + i);
    e.tm.sync();
    for (int si = 0; si < nst; ++si) {
      const uint4 st = wsteps[si];
      if (staged && (st.y < wd.z || st.y - wd.z + st.z > wd.w)) {
        if (t == 0) atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
        break;
      }
      const uint4* L = staged ? wops + (st.y - wd.z) : td.lops + st.y;
      if (st.x == 0u) {
        const int total = (int)st.z << lg;
        for (int task = t; task < total; task += size) layer_word(e, td, L[task >> lg], task & (tw - 1), status);
        e.tm.sync();
      } else if (fused) {
        trace_block_fused(e, td, L, (int)st.z, sc, tacc, pacc, status);
      } else {
        trace_block(e, td, L, (int)st.z, sc, tacc, pacc, status);
      }
    }
    e.tm.sync();
  }
  e.tm.sync();
}

// ---------------------------------------------------------------- phase pass

// Philox4x32-10 (the function of philox4x32_10) with its round keys
// precomputed from the seed.  In a phase-pass warp the seed is uniform, so
// the keys sit in uniform registers and each round is two 32x32->64
// multiplies and two three-input xors.
struct PhiloxKeys {
  uint32_t k0[10], k1[10];
  __device__ explicit PhiloxKeys(unsigned long long seed) {
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      k0[r] = a;
      k1[r] = b;
      a += 0x9E3779B9u;
      b += 0xBB67AE85u;
    }
  }
  __device__ __forceinline__ uint4 block(uint4 c) const {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      unsigned long long p0, p1;  // one 32x32->64 multiply each
      asm("mul.wide.u32 %0, %1, %2;" : "=l"(p0) : "r"(c.x), "r"(0xD2511F53u));
      asm("mul.wide.u32 %0, %1, %2;" : "=l"(p1) : "r"(c.z), "r"(0xCD9E8D57u));
      c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0[r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1[r],
                     (uint32_t)p0);
    }
    return c;
  }
};

// Fire mask of N1 ordinals [cb, cb + 32) of one shot (cb a multiple of 32):
// eight coin blocks, unrolled so their Philox chains overlap, against the
// thresholds; the exact bits are built only when a block has a fire.
__device__ __forceinline__ uint32_t coin_mask(const PhiloxKeys& K, const uint32_t* nthr, uint32_t cb, uint32_t shot_lo,
                                              uint32_t shot_hi) {
  uint32_t m = 0u;
  const uint4* t4 = reinterpret_cast<const uint4*>(nthr + cb);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const uint4 c = K.block(make_uint4((cb >> 2) + (uint32_t)b, shot_lo, shot_hi, 1u));
    const uint4 th = __ldg(t4 + b);
    if ((c.x >= th.x) | (c.y >= th.y) | (c.z >= th.z) | (c.w >= th.w))
      m |= ((uint32_t)(c.x >= th.x) | ((uint32_t)(c.y >= th.y) << 1) | ((uint32_t)(c.z >= th.z) << 2) |
            ((uint32_t)(c.w >= th.w) << 3)) << (4 * b);
  }
  return m;
}

template <int N>
__device__ __forceinline__ void load_row(const uint32_t* p, uint32_t (&r)[N]) {
  if constexpr (N % 4 == 0) {
    const uint4* p4 = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
      const uint4 v = __ldg(p4 + i);
      r[4 * i] = v.x;
      r[4 * i + 1] = v.y;
      r[4 * i + 2] = v.z;
      r[4 * i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) r[i] = __ldg(p + i);
  }
}

// Delta of a d = 2 shot is a multiple of 2 mod 4 at every point: it starts
// at 0, and every update adds 2 (a z_q + b x_q) (N1), 2 m z_q (RESET), 2 m
// (the new delta_p) or f_g delta_p with delta_p already even.  So only its
// high bit plane is kept: d1, one bit per generator.
//
// Registers hold what every measurement uses (header and row pointers, the
// shot, d1); the arrays of the N1 paths are read from the descriptor when a
// fire needs them.  The next measurement's header and factor half-row are
// loaded one iteration ahead.
// Records are staged per warp in shared memory, rec[32][kRecStride] bytes
// (row = lane, column = measurement mod 64; 17 words per row keep the lanes
// on distinct banks), and every 64 measurements the warp writes each shot's
// 64-byte run with contiguous byte stores: the group's rows are adjacent in
// the output, so one store instruction covers one or two 32-byte sectors
// instead of 32.
constexpr int kRecWindow = 64;
constexpr int kRecStride = 68;

__device__ __forceinline__ void flush_records(const uint8_t* rec, uint8_t* __restrict__ g, int nmeas, int rows,
                                              int k0, int cnt, int lane) {
  __syncwarp();
  for (int r = 0; r < rows; ++r) {
    const uint8_t* b = rec + r * kRecStride;
    uint8_t* o = g + (size_t)r * nmeas + k0;
    if (lane < cnt) o[lane] = b[lane];
    if (lane + 32 < cnt) o[lane + 32] = b[lane + 32];
  }
  __syncwarp();
}

// Word w of d, w warp-uniform: a tree of uniform branches rather than a
// compare and select per word.
template <int LO, int HI, int TW>
__device__ __forceinline__ uint32_t word_at(const uint32_t (&d)[TW], int w) {
  if constexpr (HI - LO == 1) {
    return d[LO];
  } else {
    constexpr int MID = (LO + HI) / 2;
    if (w < MID) return word_at<LO, MID>(d, w);
    return word_at<MID, HI>(d, w);
  }
}

// Sets bit b of word w of d to v (w warp-uniform, v in {0, 1}).
template <int LO, int HI, int TW>
__device__ __forceinline__ void put_bit(uint32_t (&d)[TW], int w, int b, uint32_t v) {
  if constexpr (HI - LO == 1) {
    d[LO] = (d[LO] & ~(1u << b)) | (v << b);
  } else {
    constexpr int MID = (LO + HI) / 2;
    if (w < MID)
      put_bit<LO, MID>(d, w, b, v);
    else
      put_bit<MID, HI>(d, w, b, v);
  }
}

// The next N1 fire of one shot, read from the coin pass's chunk map and
// fire masks: a shot with F fires loads F mask pairs and its chunk-map
// words, and a measurement with no fire before it costs one compare.
struct FireCursor {
  const uint2* masks;
  const uint32_t* cmap;
  int nshots, rel, nchunk, ncw;
  int cw;           // chunk-map word in use
  uint32_t cbits;   // its chunks not yet loaded
  uint32_t ax, bz;  // masks of the loaded chunk, applied fires cleared
  uint32_t base;    // first ordinal of the loaded chunk
  uint32_t next;    // ordinal of the next fire, 0xffffffff when there is none

  __device__ __forceinline__ void advance() {
    uint32_t pend = ax | bz;
    while (!pend) {
      while (!cbits) {
        if (++cw >= ncw) {
          next = 0xffffffffu;
          return;
        }
        cbits = __ldg(cmap + (size_t)cw * nshots + rel);
        if (cw == ncw - 1 && (nchunk & 31)) cbits &= (1u << (nchunk & 31)) - 1u;
      }
      const int b = __ffs(cbits) - 1;
      cbits &= cbits - 1u;
      const int c = 32 * cw + b;
      const uint2 m = __ldg(masks + (size_t)c * nshots + rel);
      ax = m.x;
      bz = m.y;
      base = 32u * (uint32_t)c;
      pend = ax | bz;
    }
    next = base + (uint32_t)(__ffs(pend) - 1);
  }
};

// One 32-shot group of a program (lane = shot).  With coin-pass masks
// (kMasks) the N1 fires come from a FireCursor; without, the coins of each
// 32-ordinal chunk are drawn here when the replay reaches it.
template <int TW, bool kMasks>
__device__ __forceinline__ void phase_program(const TraceDesc* __restrict__ tdp, long long group, int lane,
                                              uint8_t* rec) {
  constexpr int FH = TW / 2;  // factor words of a deterministic measurement
  constexpr bool kAhead = FH <= 8;
  const uint4* __restrict__ mhdr = tdp->mhdr;
  const uint32_t* __restrict__ mrow = tdp->mrow;
  const int nm = tdp->nm, wn = tdp->wn, nmeas = tdp->c.nmeas;
  const uint32_t nn1 = (uint32_t)tdp->nn1;
  const unsigned long long seed = tdp->c.seed;
  const long long rel = group * 32 + lane;
  const bool active = rel < (long long)tdp->c.nshots;
  const long long shot = tdp->c.shot0 + rel;
  const uint32_t shot_lo = (uint32_t)(unsigned long long)shot, shot_hi = (uint32_t)((unsigned long long)shot >> 32);
  const long long first = group * 32;
  const int rows = (int)min(32LL, (long long)tdp->c.nshots - first);  // shots of this group
  uint8_t* __restrict__ gout = tdp->c.out + first * (long long)nmeas;
  uint8_t* myrec = rec + lane * kRecStride;
  const PhiloxKeys K(seed);
  uint32_t d1[TW];
#pragma unroll
  for (int w = 0; w < TW; ++w) d1[w] = 0u;
  FireCursor fc;
  // without masks: N1 ordinals [nord, cend) of the current 32-ordinal chunk
  // are not yet replayed; bit i of pend is ordinal nord + i
  uint32_t nord = 0, cend = 0, pend = 0u;
  if constexpr (kMasks) {
    fc.masks = reinterpret_cast<const uint2*>(tdp->masks);
    fc.cmap = tdp->cmap;
    fc.nshots = tdp->c.nshots;
    fc.rel = (int)rel;
    fc.nchunk = tdp->nchunk;
    fc.ncw = (tdp->nchunk + 31) >> 5;
    fc.cw = -1;
    fc.cbits = fc.ax = fc.bz = fc.base = 0u;
    fc.next = 0xffffffffu;
    if (active) fc.advance();
  }
  uint4 hn = make_uint4(0u, 0u, 0u, 0u);
  uint32_t fn[FH];
  if (nm > 0) {
    hn = __ldg(mhdr);
    if constexpr (kAhead) load_row<FH>(mrow, fn);
  }
  for (int k = 0; k < nm; ++k) {
    const uint4 h = hn;
    uint32_t f[FH];
    if constexpr (kAhead) {
#pragma unroll
      for (int w = 0; w < FH; ++w) f[w] = fn[w];
      if (k + 1 < nm) {
        hn = __ldg(mhdr + k + 1);
        load_row<FH>(mrow + (size_t)(k + 1) * 2 * TW, fn);
      }
    } else {
      if (k + 1 < nm) hn = __ldg(mhdr + k + 1);
    }
    const uint32_t nend = h.z < nn1 ? h.z : nn1;
    if constexpr (kMasks) {
      while (fc.next < nend) {
        const uint32_t j = fc.next, bit = 1u << (j & 31u);
        const uint32_t mz = (fc.ax & bit) ? 0xffffffffu : 0u, mx = (fc.bz & bit) ? 0xffffffffu : 0u;
        fc.ax &= ~bit;
        fc.bz &= ~bit;
        const uint32_t* nr = tdp->nrow + (size_t)j * 2 * TW;
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[w] ^= (__ldg(nr + TW + w) & mz) ^ (__ldg(nr + w) & mx);
        fc.advance();
      }
    } else {
      while (nord < nend) {
        if (nord == cend) {
          // the Paulis are drawn on a fire below
          pend = coin_mask(K, tdp->nthr, nord, shot_lo, shot_hi);
          cend = nord + 32;
        }
        const uint32_t hi = nend < cend ? nend : cend;
        const uint32_t take = hi - nord;  // 1 .. 32
        const uint32_t lim = take >= 32 ? 0xffffffffu : ((1u << take) - 1u);
        uint32_t due = active ? (pend & lim) : 0u;
        pend = take >= 32 ? 0u : (pend >> take);
        while (due) {
          const int i = __ffs(due) - 1;
          due &= due - 1u;
          const uint32_t j = nord + (uint32_t)i;
          const uint2 nh = __ldg(tdp->nhdr + j);
          if (nh.y == OP_N1OFF) continue;  // threshold 0xffffffff: a coin of 0xffffffff is not a fire
          const int2 ab = noise_choice(nh.y, 2, seed, shot, j);
          const uint32_t mz = ab.x ? 0xffffffffu : 0u, mx = (ab.y & 1) ? 0xffffffffu : 0u;
          const uint32_t* nr = tdp->nrow + (size_t)j * 2 * TW;
#pragma unroll
          for (int w = 0; w < TW; ++w) d1[w] ^= (__ldg(nr + TW + w) & mz) ^ (__ldg(nr + w) & mx);
        }
        nord = hi;
      }
    }
    const uint32_t* row = mrow + (size_t)k * 2 * TW;
    const uint32_t det = h.x & 1u;
    int m;
    if (!det) {
      // delta_g += delta_p (g in the factor row), delta_{n+p} = delta_p,
      // delta_p = 2 m
      const int p = (int)h.y, wp = p >> 5, bp = p & 31;
      const uint32_t dp = (word_at<0, TW>(d1, wp) >> bp) & 1u;
      if (dp) {
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[w] ^= __ldg(row + w);
      }
      m = active ? mulshift(K.block(make_uint4((uint32_t)k, shot_lo, shot_hi, 0u)).x, 2u) : 0;
      put_bit<0, TW>(d1, wn + wp, bp, dp);
      put_bit<0, TW>(d1, wp, bp, (uint32_t)m);
    } else {
      if constexpr (!kAhead) load_row<FH>(row, f);
      int s = 0;
#pragma unroll
      for (int w = 0; w < FH; ++w) s += __popc(f[w] & d1[w]);
      m = (((((int)h.w + 2 * s) & 3) + 1) >> 1) & 1;
    }
    if ((h.x & 2u) && (m & 1)) {
#pragma unroll
      for (int w = 0; w < TW; ++w) d1[w] ^= __ldg(row + TW + w);
    }
    myrec[k & (kRecWindow - 1)] = (uint8_t)(m | (int)(det << 7));
    if ((k & (kRecWindow - 1)) == kRecWindow - 1 || k == nm - 1) {
      const int k0 = k & ~(kRecWindow - 1);
      flush_records(rec, gout, nmeas, rows, k0, min(k + 1, nmeas) - k0, lane);
    }
  }
}

// S shots per lane (coin-pass masks only; the kernels use S = 2): lane l of group g
// carries shots 32 S g + 32 s + l, s < S, each with its own delta and fire
// cursor, while the per-measurement work that does not depend on the shot --
// header and factor-row loads, the measurement kind, the loop -- is done once
// for all S; the S outcome draws of a random measurement are independent
// Philox chains the lane interleaves.  Records of the group's 32 S rows are
// staged in rec[32 S][kRecStride].
template <int TW, int S>
__device__ __forceinline__ void phase_program_multi(const TraceDesc* __restrict__ tdp, long long group, int lane,
                                                    uint8_t* rec) {
  constexpr int FH = TW / 2;
  constexpr bool kAhead = FH <= 8;
  const uint4* __restrict__ mhdr = tdp->mhdr;
  const uint32_t* __restrict__ mrow = tdp->mrow;
  const int nm = tdp->nm, wn = tdp->wn, nmeas = tdp->c.nmeas, nshots = tdp->c.nshots;
  const uint32_t nn1 = (uint32_t)tdp->nn1;
  const long long first = group * 32 * S;
  const int rows = (int)min(32LL * S, (long long)nshots - first);
  uint8_t* __restrict__ gout = tdp->c.out + first * (long long)nmeas;
  const PhiloxKeys K(tdp->c.seed);
  uint32_t d1[S][TW];
  bool active[S];
  uint32_t slo[S], shi[S];
  FireCursor fc[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
#pragma unroll
    for (int w = 0; w < TW; ++w) d1[s][w] = 0u;
    const long long rel = first + 32 * s + lane;
    active[s] = rel < (long long)nshots;
    const unsigned long long shot = (unsigned long long)(tdp->c.shot0 + rel);
    slo[s] = (uint32_t)shot;
    shi[s] = (uint32_t)(shot >> 32);
    fc[s].masks = reinterpret_cast<const uint2*>(tdp->masks);
    fc[s].cmap = tdp->cmap;
    fc[s].nshots = nshots;
    fc[s].rel = (int)rel;
    fc[s].nchunk = tdp->nchunk;
    fc[s].ncw = (tdp->nchunk + 31) >> 5;
    fc[s].cw = -1;
    fc[s].cbits = fc[s].ax = fc[s].bz = fc[s].base = 0u;
    fc[s].next = 0xffffffffu;
    if (active[s]) fc[s].advance();
  }
  uint4 hn = make_uint4(0u, 0u, 0u, 0u);
  uint32_t fn[FH];
  if (nm > 0) {
    hn = __ldg(mhdr);
    if constexpr (kAhead) load_row<FH>(mrow, fn);
  }
  for (int k = 0; k < nm; ++k) {
    const uint4 h = hn;
    uint32_t f[FH];
    if constexpr (kAhead) {
#pragma unroll
      for (int w = 0; w < FH; ++w) f[w] = fn[w];
      if (k + 1 < nm) {
        hn = __ldg(mhdr + k + 1);
        load_row<FH>(mrow + (size_t)(k + 1) * 2 * TW, fn);
      }
    } else {
      if (k + 1 < nm) hn = __ldg(mhdr + k + 1);
    }
    const uint32_t nend = h.z < nn1 ? h.z : nn1;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      while (fc[s].next < nend) {
        const uint32_t j = fc[s].next, bit = 1u << (j & 31u);
        const uint32_t mz = (fc[s].ax & bit) ? 0xffffffffu : 0u, mx = (fc[s].bz & bit) ? 0xffffffffu : 0u;
        fc[s].ax &= ~bit;
        fc[s].bz &= ~bit;
        const uint32_t* nr = tdp->nrow + (size_t)j * 2 * TW;
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[s][w] ^= (__ldg(nr + TW + w) & mz) ^ (__ldg(nr + w) & mx);
        fc[s].advance();
      }
    }
    const uint32_t* row = mrow + (size_t)k * 2 * TW;
    const uint32_t det = h.x & 1u;
    int m[S];
    if (!det) {
      const int p = (int)h.y, wp = p >> 5, bp = p & 31;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const uint32_t dp = (word_at<0, TW>(d1[s], wp) >> bp) & 1u;
        if (dp) {
#pragma unroll
          for (int w = 0; w < TW; ++w) d1[s][w] ^= __ldg(row + w);
        }
        m[s] = active[s] ? mulshift(K.block(make_uint4((uint32_t)k, slo[s], shi[s], 0u)).x, 2u) : 0;
        put_bit<0, TW>(d1[s], wn + wp, bp, dp);
        put_bit<0, TW>(d1[s], wp, bp, (uint32_t)m[s]);
      }
    } else {
      if constexpr (!kAhead) load_row<FH>(row, f);
#pragma unroll
      for (int s = 0; s < S; ++s) {
        int acc = 0;
#pragma unroll
        for (int w = 0; w < FH; ++w) acc += __popc(f[w] & d1[s][w]);
        m[s] = (((((int)h.w + 2 * acc) & 3) + 1) >> 1) & 1;
      }
    }
    if (h.x & 2u) {
#pragma unroll
      for (int s = 0; s < S; ++s)
        if (m[s] & 1) {
#pragma unroll
          for (int w = 0; w < TW; ++w) d1[s][w] ^= __ldg(row + TW + w);
        }
    }
#pragma unroll
    for (int s = 0; s < S; ++s) rec[(32 * s + lane) * kRecStride + (k & (kRecWindow - 1))] = (uint8_t)(m[s] | (int)(det << 7));
    if ((k & (kRecWindow - 1)) == kRecWindow - 1 || k == nm - 1) {
      const int k0 = k & ~(kRecWindow - 1);
      flush_records(rec, gout, nmeas, rows, k0, min(k + 1, nmeas) - k0, lane);
    }
  }
}

// Coin pass item it of td: shot it % nshots, chunks kCoinChunksPerItem *
// (it / nshots) onwards.  For every fired N1 (rare) the Pauli is drawn here,
// so masks[c * nshots + s] = (x mask, z mask): bit i of .x set when ordinal
// 32 c + i applies X^a with a odd (the phase update reads z_q), of .y when it
// applies Z^b with b odd (reads x_q); an N1 with probability 0 never fires.
// The item's byte of the chunk map (byte cg % 4 of word cg / 4) marks which
// of its chunks have a non-zero pair.
__device__ __forceinline__ void coin_item(const TraceDesc* __restrict__ tdp, long long it) {
  const int nshots = tdp->c.nshots;
  const long long cg = it / nshots;
  const int rel = (int)(it - cg * nshots);
  const long long shot = tdp->c.shot0 + rel;
  const unsigned long long seed = tdp->c.seed;
  const PhiloxKeys K(seed);
  const uint32_t* nthr = tdp->nthr;
  uint2* out = reinterpret_cast<uint2*>(tdp->masks) + rel;
  const int nchunk = tdp->nchunk;
  const int c0 = (int)cg * kCoinChunksPerItem;
  const int c1 = min(nchunk, c0 + kCoinChunksPerItem);
  uint32_t any = 0u;
  for (int c = c0; c < c1; ++c) {
    const uint32_t cb = (uint32_t)c * kCoinChunk;
    uint32_t f = coin_mask(K, nthr, cb, (uint32_t)(unsigned long long)shot, (uint32_t)((unsigned long long)shot >> 32));
    uint32_t ax = 0u, bz = 0u;
    while (f) {
      const int i = __ffs(f) - 1;
      f &= f - 1u;
      const uint2 nh = __ldg(tdp->nhdr + cb + i);
      if (nh.y == OP_N1OFF) continue;  // threshold 0xffffffff: a coin of 0xffffffff is not a fire
      const int2 ab = noise_choice(nh.y, 2, seed, shot, cb + i);
      ax |= (uint32_t)(ab.x & 1) << i;
      bz |= (uint32_t)(ab.y & 1) << i;
    }
    out[(size_t)c * nshots] = make_uint2(ax, bz);
    any |= (uint32_t)((ax | bz) != 0u) << (c - c0);
  }
  reinterpret_cast<uint8_t*>(tdp->cmap + (size_t)(cg >> 2) * nshots + rel)[cg & 3] = (uint8_t)any;
}

__device__ __forceinline__ int find_coin_desc(const TraceDesc* descs, int ndesc, long long it) {
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (descs[mid].coin_begin <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_trace_desc(const TraceDesc* descs, int ndesc, long long it) {
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (descs[mid].c.item_begin <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace sdim
