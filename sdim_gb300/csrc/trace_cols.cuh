// Record columns of the d = 2 trace engine, device side.
//
// Over GF(2) the phase replay of phase_program (trace_bits.cuh) is affine in
// a shot's random inputs: every update of the delta plane d1 is linear in d1
// (d1 ^= d1_p row, d1_{n+p} := d1_p, RESET d1 ^= m z_q), the deterministic
// outcome is aph_c's constant plus the parity of f . d1, and the inputs enter
// additively -- the outcome m of a random measurement (d1_p := m, record m)
// and the two odd-exponent bits of a fired N1 (d1 ^= z_q for X^a, ^= x_q for
// Z^b).  So the records of a shot are
//   rec = C ^ sum_{random k, m_k = 1} O_k ^ sum_{fired ordinal j} (a_j A_j ^ b_j B_j)
// with one column per input: C the records of the shot with every input 0,
// O_k, A_j, B_j the records each input flips.  The columns depend on the
// program alone; the column pass computes them from the trace, one lane per
// column walking the measurements from the column's input on, and the record
// pass gives each shot its outcome draws (the same Philox blocks as the
// replay) and its fires (the coin pass's masks) and XORs the columns in:
// records identical to the replay's bit for bit.
//
// Column table of one program (cols, nw words per column, bit k of word k/32
// = record k, words past the records zero):
//   column 0: C;  column 1 + k: O_k for random measurement k (unused for a
//   deterministic k);  column 1 + nm + 2 j: A_j,  2 + nm + 2 j: B_j
//   (j < nused, the N1 ordinals before the last measurement).
#pragma once
#include "trace_bits.cuh"

namespace sdim {

// First measurement that ordinal j's N1 update precedes (mhdr[k].z counts
// the ordinals before measurement k, nondecreasing in k; j < mhdr[nm-1].z).
__device__ __forceinline__ int fire_measurement(const uint4* __restrict__ mhdr, int nm, uint32_t j) {
  int lo = 0, hi = nm - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&mhdr[mid].z) > j) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Constant of a deterministic outcome: m = c ^ (s & 1) for the common phase
// aph_c and the factor sum s (the replay's ((aph_c + 2 s) mod 4 + 1) / 2 mod 2).
__device__ __forceinline__ uint32_t det_constant(uint32_t aph) { return (((aph & 3u) + 1u) >> 1) & 1u; }

// N words of a row staged in shared memory (16-byte aligned when N % 4 == 0).
template <int N>
__device__ __forceinline__ void srow_load(const uint32_t* p, uint32_t (&r)[N]) {
  if constexpr (N % 4 == 0) {
    const uint4* p4 = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
      const uint4 v = p4[i];
      r[4 * i] = v.x;
      r[4 * i + 1] = v.y;
      r[4 * i + 2] = v.z;
      r[4 * i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) r[i] = p[i];
  }
}

// Measurements of the trace a column-pass block stages in shared memory at
// a time: headers and both rows of each, within 48 KB.
template <int TW>
__host__ __device__ constexpr int column_window() {
  return TW <= 2 ? 1024 : TW <= 8 ? 512 : TW == 16 ? 256 : 128;
}

// Columns 32 WARPS g .. of one program, lane = column (warp w of the block:
// columns 32 (WARPS g + w) onwards).  The block stages the trace window by
// window in shared memory (shdr, srow: column_window<TW>() measurements);
// each warp walks the measurements from the earliest input of its lanes on
// (warp-uniform loop, broadcast shared-memory loads); a lane's delta is zero
// until its input enters, so its bits before that stay zero.
template <int TW, int WARPS>
__device__ __forceinline__ void column_block(const TraceDesc* __restrict__ tdp, long long g, uint4* shdr,
                                             uint32_t* srow, int* smin) {
  constexpr int FH = TW / 2;
  constexpr int WIN = column_window<TW>();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint4* __restrict__ mhdr = tdp->mhdr;
  const uint32_t* __restrict__ mrow = tdp->mrow;
  const int nm = tdp->nm, wn = tdp->wn, nw = tdp->nw;
  const long long ncols = column_count(nm, tdp->nused);
  const long long i = (g * WARPS + warp) * 32 + lane;
  // kind: 0 inactive, 1 the constant column, 2 an outcome, 3 a fire input
  int kind = 0, start = nm;
  const uint32_t* inj = nullptr;  // the fire input's row (z_q for A_j, x_q for B_j)
  if (i == 0) {
    kind = 1;
    start = 0;
  } else if (i <= nm) {
    const int k = (int)(i - 1);
    if (!(__ldg(&mhdr[k].x) & 1u)) {  // deterministic measurements have no outcome column
      kind = 2;
      start = k;
    }
  } else if (i < ncols) {
    const uint32_t j = (uint32_t)((i - 1 - nm) >> 1);
    kind = 3;
    start = fire_measurement(mhdr, nm, j);
    inj = tdp->nrow + (size_t)j * 2 * TW + (((i - 1 - nm) & 1) ? 0 : TW);
  }
  uint32_t* __restrict__ out = tdp->cols + (size_t)i * nw;
  int k0 = start;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) k0 = min(k0, __shfl_xor_sync(0xffffffffu, k0, o));
  if (threadIdx.x == 0) *smin = nm;
  __syncthreads();
  if (lane == 0) atomicMin(smin, k0);
  __syncthreads();
  const int kb0 = *smin;  // the block's first measurement
  if (kind)
    for (int w = 0; w < (k0 >> 5); ++w) out[w] = 0u;
  uint32_t d1[TW];
#pragma unroll
  for (int w = 0; w < TW; ++w) d1[w] = 0u;
  uint32_t acc = 0u;
  for (int wb = kb0; wb < nm; wb += WIN) {
    const int we = min(nm, wb + WIN);
    __syncthreads();  // the previous window is done
    for (int t = threadIdx.x; t < we - wb; t += 32 * WARPS) shdr[t] = __ldg(mhdr + wb + t);
    {
      const uint4* src = reinterpret_cast<const uint4*>(mrow + (size_t)wb * 2 * TW);
      uint4* dst = reinterpret_cast<uint4*>(srow);
      const int n4 = (we - wb) * 2 * TW / 4;
      for (int t = threadIdx.x; t < n4; t += 32 * WARPS) dst[t] = __ldg(src + t);
    }
    __syncthreads();
    int k = max(wb, k0);
    while (k < we) {
      const uint4 h = shdr[k - wb];
      const uint32_t* row = srow + (size_t)(k - wb) * 2 * TW;
      if (kind == 3 && start == k) {
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[w] ^= __ldg(inj + w);
      }
      if (!(h.x & 1u)) {
        // a random measurement: the rowsum and the pivot bits
        uint32_t r[TW];
#pragma unroll
        for (int w = 0; w < TW; ++w) r[w] = row[w];
        const int p = (int)h.y, wp = p >> 5, bp = p & 31;
        const uint32_t dp = (word_at<0, TW>(d1, wp) >> bp) & 1u;
        const uint32_t mk = 0u - dp;
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[w] ^= r[w] & mk;
        const uint32_t bit = (kind == 2 && start == k) ? 1u : 0u;  // the outcome itself
        put_bit<0, TW>(d1, wn + wp, bp, dp);
        put_bit<0, TW>(d1, wp, bp, bit);
        if (h.x & 2u) {
#pragma unroll
          for (int w = 0; w < TW; ++w) d1[w] ^= row[TW + w] & (0u - bit);
        }
        acc |= bit << (k & 31);
        if ((k & 31) == 31 || k == nm - 1) {
          if (kind) out[k >> 5] = acc;
          acc = 0u;
        }
        ++k;
        continue;
      }
      // a run of up to 32 deterministic measurements [k, ke): every factor
      // parity from the delta at the run's start (independent, so they
      // overlap), each outcome corrected by the earlier RESETs of the run
      // that its factor sees (the header pass's coupling mask in y against
      // the run's outcomes so far), then the run's RESET rows XORed in.  A
      // fire input entering inside the run adds its own parities from its
      // start on (its outcomes before that are zero).
      int ke = k + 1;
      while (ke < we && ke - k < 32 && (shdr[ke - wb].x & 1u)) ++ke;
      const int len = ke - k;
      const bool late = kind == 3 && start > k && start < ke;
      const uint32_t cst = kind == 1 ? 0xffffffffu : 0u;
      uint32_t hist = 0u, bits = 0u;
      if (__any_sync(0xffffffffu, late)) {
        uint32_t v[TW];
#pragma unroll
        for (int w = 0; w < TW; ++w) v[w] = late ? __ldg(inj + w) : 0u;
        for (int i = 0; i < len; ++i) {
          const uint4 hi = shdr[k + i - wb];
          uint32_t f[FH];
          srow_load<FH>(srow + (size_t)(k + i - wb) * 2 * TW, f);
          uint32_t x = 0u, y = 0u;
#pragma unroll
          for (int w = 0; w < FH; ++w) {
            x ^= f[w] & d1[w];
            y ^= f[w] & v[w];
          }
          uint32_t b = ((uint32_t)__popc(x) ^ (k + i >= start ? (uint32_t)__popc(y) : 0u)) & 1u;
          b ^= (det_constant(hi.w) & cst) ^ ((uint32_t)__popc(hi.y & hist) & 1u);
          hist = (hist << 1) | b;
        }
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[w] ^= v[w];
      } else {
#pragma unroll 4
        for (int i = 0; i < len; ++i) {
          const uint4 hi = shdr[k + i - wb];
          uint32_t f[FH];
          srow_load<FH>(srow + (size_t)(k + i - wb) * 2 * TW, f);
          uint32_t x = 0u;
#pragma unroll
          for (int w = 0; w < FH; ++w) x ^= f[w] & d1[w];
          const uint32_t b = ((uint32_t)__popc(x) ^ (det_constant(hi.w) & cst) ^ (uint32_t)__popc(hi.y & hist)) & 1u;
          hist = (hist << 1) | b;
        }
      }
      // hist holds the run's outcomes, the last in bit 0: bit i of bits =
      // measurement k + i
      bits = __brev(hist) >> (32 - len);
      for (int i = 0; i < len; ++i) {
        if (!(shdr[k + i - wb].x & 2u)) continue;
        uint32_t z[TW];
        srow_load<TW>(srow + (size_t)(k + i - wb) * 2 * TW + TW, z);
        const uint32_t mk = 0u - ((bits >> i) & 1u);
#pragma unroll
        for (int w = 0; w < TW; ++w) d1[w] ^= z[w] & mk;
      }
      // the run's outcomes into the record words: word k / 32 completes when
      // the run reaches its end
      const int sh = k & 31;
      acc |= bits << sh;
      if (sh + len >= 32) {
        if (kind) out[k >> 5] = acc;
        acc = sh + len > 32 ? bits >> (32 - sh) : 0u;
      }
      if (ke == nm && (nm & 31)) {
        if (kind) out[(nm - 1) >> 5] = acc;
        acc = 0u;
      }
      k = ke;
    }
  }
  if (kind)
    for (int w = ((nm - 1) >> 5) + 1; w < nw; ++w) out[w] = 0u;
}

// Four record bytes from four record bits and four deterministic flags
// (nibbles): byte b = bit b | flag b << 7.
__device__ __forceinline__ uint32_t record_bytes(uint32_t bits4, uint32_t det4) {
  return ((bits4 * 0x00204081u) & 0x01010101u) | (((det4 * 0x00204081u) & 0x01010101u) << 7);
}

// One 32-shot group (lane = shot) from the column table: NW words of record
// bits per lane.  Fires come from the coin pass's masks; the outcome draws
// are the replay's (measurement k, shot, domain 0).  Records are staged per
// 64 measurements in rec[32][kRecStride] and written as the replay does.
template <int NW>
__device__ __forceinline__ void record_group(const TraceDesc* __restrict__ tdp, long long group, int lane,
                                             uint8_t* rec) {
  const uint4* __restrict__ mhdr = tdp->mhdr;
  const uint32_t* __restrict__ cols = tdp->cols;
  const int nm = tdp->nm, nmeas = tdp->c.nmeas;
  const uint32_t nused = (uint32_t)tdp->nused;
  const long long rel = group * 32 + lane;
  const bool active = rel < (long long)tdp->c.nshots;
  const long long shot = tdp->c.shot0 + rel;
  const uint32_t shot_lo = (uint32_t)(unsigned long long)shot, shot_hi = (uint32_t)((unsigned long long)shot >> 32);
  const long long first = group * 32;
  const int rows = (int)min(32LL, (long long)tdp->c.nshots - first);
  uint8_t* __restrict__ gout = tdp->c.out + first * (long long)nmeas;
  uint32_t* myrec = reinterpret_cast<uint32_t*>(rec + lane * kRecStride);
  const PhiloxKeys K(tdp->c.seed);
  uint32_t b[NW];
  load_row<NW>(cols, b);
  // fires: every fired ordinal before the last measurement
  if (active && nused > 0u && tdp->masks) {
    FireCursor fc;
    fc.masks = reinterpret_cast<const uint2*>(tdp->masks);
    fc.cmap = tdp->cmap;
    fc.nshots = tdp->c.nshots;
    fc.rel = (int)rel;
    fc.nchunk = tdp->nchunk;
    fc.ncw = (tdp->nchunk + 31) >> 5;
    fc.cw = -1;
    fc.cbits = fc.ax = fc.bz = fc.base = 0u;
    fc.next = 0xffffffffu;
    fc.advance();
    while (fc.next < nused) {
      const uint32_t j = fc.next, bit = 1u << (j & 31u);
      const uint32_t ma = (fc.ax & bit) ? 0xffffffffu : 0u, mb = (fc.bz & bit) ? 0xffffffffu : 0u;
      fc.ax &= ~bit;
      fc.bz &= ~bit;
      const uint32_t* ca = cols + (size_t)(1 + nm + 2 * (size_t)j) * NW;
#pragma unroll
      for (int w = 0; w < NW; ++w) b[w] ^= (__ldg(ca + w) & ma) ^ (__ldg(ca + NW + w) & mb);
      fc.advance();
    }
  }
  // windows of 64 measurements: the outcomes drawn in the window flip its
  // records and later ones only, so the window is final once they are in
#pragma unroll
  for (int q = 0; q < NW / 2; ++q) {
    const int kb = 64 * q;
    if (kb >= nm) break;
    uint32_t det[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = kb + 32 * h + lane;
      const uint32_t x = k < nm ? __ldg(&mhdr[k].x) : 1u;
      uint32_t rnd = __ballot_sync(0xffffffffu, k < nm && !(x & 1u));
      det[h] = __ballot_sync(0xffffffffu, k < nm && (x & 1u));
      while (rnd) {
        const int kk = kb + 32 * h + __ffs(rnd) - 1;
        rnd &= rnd - 1u;
        const uint32_t m = active ? mulshift(K.block(make_uint4((uint32_t)kk, shot_lo, shot_hi, 0u)).x, 2u) : 0u;
        const uint32_t mm = 0u - m;
        const uint32_t* co = cols + (size_t)(1 + kk) * NW;
#pragma unroll
        for (int w = 2 * q; w < NW; ++w) b[w] ^= __ldg(co + w) & mm;  // words before 2q are zero
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int t = 0; t < 8; ++t)
        myrec[8 * h + t] = record_bytes((b[2 * q + h] >> (4 * t)) & 15u, (det[h] >> (4 * t)) & 15u);
    flush_records(rec, gout, nmeas, rows, kb, min(64, nm - kb), lane);
  }
}

}  // namespace sdim
