// Trace engine kernels (d = 2): the x / z pass, one CTA per program over its
// layered schedule, the phase pass, one lane per shot, and the column and
// record passes that replace the phase pass for a single program.
#include "trace_bits.cuh"
#include "trace_cols.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

// One program per block (grid-stride over programs), THREADS threads.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_trace_pass(const TraceDesc* __restrict__ descs, int ndesc,
                                                                  uint8_t* gxz, size_t xz_bytes, size_t hot_bytes,
                                                                  int xz_in_smem, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[kTeamRedInts];
  __shared__ int sc[3], tacc[kTraceBlockMeas], pacc[kTraceBlockMeas];
  uint8_t* hot = smem;
  uint8_t* xz = xz_in_smem ? smem + hot_bytes : gxz + (size_t)blockIdx.x * xz_bytes;
  uint4* win = reinterpret_cast<uint4*>(smem + hot_bytes + (xz_in_smem ? xz_bytes : 0));
  for (int i = blockIdx.x; i < ndesc; i += gridDim.x) {
    const TraceDesc td = descs[i];
    TraceTab e(xz, hot, td.c.n, 2, CtaTeam(red));
    trace_program(td, e, win, sc, tacc, pacc, status);
    __syncthreads();
  }
}

// One warp per measurement k of descs[0], for its deterministic ones:
//  * with flag 4 in the header, the cross term T = sum over qudit rows of the
//    pairs i < j of the factor f with f_i z_i f_j x_j (mod 2), from the
//    snapshot of the stabilizer halves its x / z pass took, is added to its
//    common phase: w += 2 T (mod 4) (lane = qudit rows, one ballot);
//  * the coupling mask goes into y: bit t = f_k . z_j (mod 2) for the RESET
//    j = k - 1 - t when no random measurement lies in [j, k) (the column
//    pass evaluates such runs of deterministic measurements at once and
//    corrects each outcome by the earlier RESETs it sees; lane = t).
__global__ void __launch_bounds__(128) k_header_pass(const TraceDesc* __restrict__ descs, const int* status) {
  if (*(volatile const int*)status != DEV_OK) return;
  const TraceDesc* tdp = descs;
  const int k = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= tdp->nm) return;
  const uint4 h = tdp->mhdr[k];
  if (!(h.x & 1u)) return;  // random (uniform over the warp)
  const int n = tdp->c.n, wn = tdp->wn, tw = tdp->tw;
  const uint32_t* f = tdp->mrow + (size_t)k * 2 * tw;
  uint32_t cm;
  {
    const int j = k - 1 - lane;
    // read x alone: another warp may be rewriting that header's other words
    const uint32_t xj = j >= 0 ? *(volatile const uint32_t*)&tdp->mhdr[j].x : 0u;
    const uint32_t stop = __ballot_sync(0xffffffffu, j < 0 || !(xj & 1u));  // random or before the start
    const uint32_t in_run = stop ? (1u << (__ffs(stop) - 1)) - 1u : 0xffffffffu;
    uint32_t c = 0u;
    if (((in_run >> lane) & 1u) && (xj & 2u)) {
      const uint32_t* zj = tdp->mrow + (size_t)j * 2 * tw + tw;
      uint32_t v = 0u;
      for (int w = 0; w < wn; ++w) v ^= f[w] & zj[w];
      c = (uint32_t)__popc(v) & 1u;
    }
    cm = __ballot_sync(0xffffffffu, c != 0u);
  }
  if (!(h.x & 4u)) {
    if (lane == 0) tdp->mhdr[k] = make_uint4(h.x, cm, h.z, h.w);
    return;
  }
  const uint32_t* sx = tdp->snap + (size_t)h.y * 2 * n * wn;
  const uint32_t* sz = sx + (size_t)n * wn;
  uint32_t tpar = 0u;
  for (int kr = lane; kr < n; kr += 32) {
    uint32_t carry = 0u;
    for (int w = 0; w < wn; ++w) {
      const uint32_t fw = f[w];
      if (!fw) continue;
      const uint32_t a = sx[(size_t)kr * wn + w] & fw, b = sz[(size_t)kr * wn + w] & fw;
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
  }
  const uint32_t par = (uint32_t)__popc(__ballot_sync(0xffffffffu, tpar != 0u)) & 1u;
  if (lane == 0) tdp->mhdr[k] = make_uint4(h.x & ~4u, cm, h.z, (h.w + 2u * par) & 3u);
}

// One single-warp block per group of 32 SPL shots (groups of all programs
// are numbered through descs[].c.item_begin).  With the group index taken
// from blockIdx alone, every per-program value and the whole measurement loop
// control are provably warp-uniform, so they stay out of the per-lane
// registers.  Up to 16-word rows and one shot per lane, 32 blocks per SM at
// 64 registers; wider rows or two shots per lane get 128.
template <int TW, int SPL>
__global__ void __launch_bounds__(32, TW >= 64 ? 8 : (TW >= 16 || SPL == 2) ? 16 : 32)
    k_phase_pass(const TraceDesc* __restrict__ descs, int ndesc, long long total_groups, const int* status) {
  __shared__ uint8_t rec[32 * SPL * kRecStride];
  if (*(volatile const int*)status != DEV_OK) return;  // the trace is incomplete
  const long long g = blockIdx.x;
  if (g >= total_groups) return;
  const int i = find_trace_desc(descs, ndesc, g);
  const long long lg = g - descs[i].c.item_begin;
  if constexpr (SPL >= 2) {
    if (descs[i].masks) {
      phase_program_multi<TW, SPL>(descs + i, lg, threadIdx.x, rec);
    } else {  // no masks: the 32-shot parts one after the other
      for (int h = 0; h < SPL; ++h)
        if ((SPL * lg + h) * 32 < (long long)descs[i].c.nshots)
          phase_program<TW, false>(descs + i, SPL * lg + h, threadIdx.x, rec);
    }
  } else {
    if (descs[i].masks)
      phase_program<TW, true>(descs + i, lg, threadIdx.x, rec);
    else
      phase_program<TW, false>(descs + i, lg, threadIdx.x, rec);
  }
}

// One block of kColumnWarps warps per 32 kColumnWarps record columns of
// descs[0], the trace staged in shared memory a window at a time.
template <int TW>
__global__ void __launch_bounds__(32 * kColumnWarps) k_column_pass(const TraceDesc* __restrict__ descs,
                                                                   const int* status) {
  __shared__ uint4 shdr[column_window<TW>()];
  __shared__ __align__(16) uint32_t srow[column_window<TW>() * 2 * TW];
  __shared__ int smin;
  if (*(volatile const int*)status != DEV_OK) return;  // the trace is incomplete (uniform over the block)
  column_block<TW, kColumnWarps>(descs, blockIdx.x, shdr, srow, &smin);
}

// One single-warp block per 32-shot group of descs[0], from its record
// columns: up to 16 column words, 32 blocks per SM at 64 registers.
template <int NW>
__global__ void __launch_bounds__(32, NW >= 32 ? 16 : 32)
    k_record_pass(const TraceDesc* __restrict__ descs, long long g0, long long groups, const int* status) {
  __shared__ __align__(16) uint8_t rec[32 * kRecStride];
  if (*(volatile const int*)status != DEV_OK) return;
  if ((long long)blockIdx.x >= groups) return;
  record_group<NW>(descs, g0 + blockIdx.x, threadIdx.x, rec);
}

// One thread per (chunk group, shot) item of the coin pass; descs with
// masks only, numbered through coin_begin.  Three blocks per SM leave 80
// registers a thread: the eight interleaved Philox chains and their round
// keys fit without spills.
__global__ void __launch_bounds__(256, 3) k_coin_pass(const TraceDesc* __restrict__ descs, int ndesc,
                                                      long long total) {
  const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= total) return;
  const int i = find_coin_desc(descs, ndesc, it);
  coin_item(descs + i, it - descs[i].coin_begin);
}

// Philox throughput probe: every thread draws iters x 8 blocks (eight
// independent chains per step, as the coin pass does) under a key loaded per
// thread, and folds them so the work stays live.
__global__ void __launch_bounds__(256) k_philox_probe(const unsigned long long* __restrict__ seeds, int iters,
                                                      uint4* sink) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const PhiloxKeys K(seeds[t & 255]);
  uint4 acc = make_uint4(0u, 0u, 0u, 0u);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const uint4 c = K.block(make_uint4((uint32_t)(it * 8 + b), (uint32_t)t, 0u, 1u));
      acc.x ^= c.x;
      acc.y ^= c.y;
      acc.z ^= c.z;
      acc.w ^= c.w;
    }
  }
  if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9e3779b9u) sink[t & 255] = acc;
}

}  // namespace

void launch_philox_probe(int grid, cudaStream_t s, const unsigned long long* seeds, int iters, uint4* sink) {
  k_philox_probe<<<grid, 256, 0, s>>>(seeds, iters, sink);
}

void launch_header_pass(int grid, cudaStream_t s, const TraceDesc* descs, const int* status) {
  k_header_pass<<<grid, 128, 0, s>>>(descs, status);
}

void launch_coin_pass(int grid, int block, size_t smem, cudaStream_t s, const TraceDesc* descs, int ndesc,
                      long long total) {
  k_coin_pass<<<grid, block, smem, s>>>(descs, ndesc, total);
}

size_t trace_pass_hot_bytes(int n) { return round16(TraceTab::hot_bytes(n)); }
size_t trace_pass_xz_bytes(int n) { return round16(TraceTab::xz_bytes(n)); }

cudaError_t trace_set_smem(int optin) {
  const cudaError_t e = set_dynamic_smem(k_trace_pass<256>, optin);
  return e != cudaSuccess ? e : set_dynamic_smem(k_trace_pass<512>, optin);
}

void launch_trace_pass(int threads, int grid, size_t smem, cudaStream_t s, const TraceDesc* descs, int ndesc,
                       uint8_t* gxz, size_t xz_bytes, size_t hot_bytes, int xz_in_smem, int* status) {
  if (threads >= 512)
    k_trace_pass<512><<<grid, 512, smem, s>>>(descs, ndesc, gxz, xz_bytes, hot_bytes, xz_in_smem, status);
  else
    k_trace_pass<256><<<grid, 256, smem, s>>>(descs, ndesc, gxz, xz_bytes, hot_bytes, xz_in_smem, status);
}

template <int SPL>
bool launch_phase_spl(int tw, int grid, int block, cudaStream_t s, const TraceDesc* descs, int ndesc,
                      long long total_groups, int* status) {
  switch (tw) {
    case 2: k_phase_pass<2, SPL><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 4: k_phase_pass<4, SPL><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 8: k_phase_pass<8, SPL><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 16: k_phase_pass<16, SPL><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 32: k_phase_pass<32, SPL><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    default: break;
  }
  if constexpr (SPL == 1) {  // wider rows: one shot per lane (n <= 2048)
    switch (tw) {
      case 64: k_phase_pass<64, 1><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
      case 128: k_phase_pass<128, 1><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
      default: break;
    }
  }
  return false;
}

bool launch_column_pass(int tw, int grid, cudaStream_t s, const TraceDesc* descs, const int* status) {
  switch (tw) {
    case 2: k_column_pass<2><<<grid, 32 * kColumnWarps, 0, s>>>(descs, status); return true;
    case 4: k_column_pass<4><<<grid, 32 * kColumnWarps, 0, s>>>(descs, status); return true;
    case 8: k_column_pass<8><<<grid, 32 * kColumnWarps, 0, s>>>(descs, status); return true;
    case 16: k_column_pass<16><<<grid, 32 * kColumnWarps, 0, s>>>(descs, status); return true;
    case 32: k_column_pass<32><<<grid, 32 * kColumnWarps, 0, s>>>(descs, status); return true;
    default: return false;
  }
}

bool launch_record_pass(int nw, long long g0, int grid, cudaStream_t s, const TraceDesc* descs, long long groups,
                        const int* status) {
  switch (nw) {
    case 2: k_record_pass<2><<<grid, 32, 0, s>>>(descs, g0, groups, status); return true;
    case 4: k_record_pass<4><<<grid, 32, 0, s>>>(descs, g0, groups, status); return true;
    case 8: k_record_pass<8><<<grid, 32, 0, s>>>(descs, g0, groups, status); return true;
    case 16: k_record_pass<16><<<grid, 32, 0, s>>>(descs, g0, groups, status); return true;
    case 32: k_record_pass<32><<<grid, 32, 0, s>>>(descs, g0, groups, status); return true;
    default: return false;
  }
}

bool launch_phase_pass(int tw, int spl, int grid, int block, cudaStream_t s, const TraceDesc* descs, int ndesc,
                       long long total_groups, int* status) {
  return spl == 2 ? launch_phase_spl<2>(tw, grid, block, s, descs, ndesc, total_groups, status)
                  : launch_phase_spl<1>(tw, grid, block, s, descs, ndesc, total_groups, status);
}

}  // namespace sdim
