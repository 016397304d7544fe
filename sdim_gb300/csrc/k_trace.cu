// Trace engine kernels (d = 2): the x / z pass, one CTA per program over its
// layered schedule, and the phase pass, one lane per shot.
#include "trace_bits.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

// One program per block (grid-stride over programs), kTracePassThreads threads.
__global__ void __launch_bounds__(kTracePassThreads) k_trace_pass(const TraceDesc* __restrict__ descs, int ndesc,
                                                                  uint8_t* gxz, size_t xz_bytes, size_t hot_bytes,
                                                                  int xz_in_smem, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[40];
  __shared__ int piv[kTraceBlockMeas], tacc[kTraceBlockMeas], pacc[kTraceBlockMeas];
  uint8_t* hot = smem;
  uint8_t* xz = xz_in_smem ? smem + hot_bytes : gxz + (size_t)blockIdx.x * xz_bytes;
  uint4* win = reinterpret_cast<uint4*>(smem + hot_bytes + (xz_in_smem ? xz_bytes : 0));
  for (int i = blockIdx.x; i < ndesc; i += gridDim.x) {
    const TraceDesc td = descs[i];
    TraceTab e(xz, hot, td.c.n, 2, CtaTeam(red));
    trace_program(td, e, win, piv, tacc, pacc, status);
    __syncthreads();
  }
}

// One warp per 32-shot group; groups of all programs are numbered through
// descs[].c.item_begin.  Narrow rows leave registers for three blocks per SM
// (24 warps: 100k shots fill every SM in one wave).
template <int TW>
__global__ void __launch_bounds__(256, TW <= 8 ? 3 : 2) k_phase_pass(const TraceDesc* __restrict__ descs, int ndesc,
                                                    long long total_groups, const int* status) {
  if (*(volatile const int*)status != DEV_OK) return;  // the trace is incomplete
  const long long g = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (g >= total_groups) return;
  const int i = find_trace_desc(descs, ndesc, g);
  phase_program<TW>(descs[i], g - descs[i].c.item_begin, threadIdx.x & 31);
}

}  // namespace

size_t trace_pass_hot_bytes(int n) { return round16(TraceTab::hot_bytes(n)); }
size_t trace_pass_xz_bytes(int n) { return round16(TraceTab::xz_bytes(n)); }

cudaError_t trace_set_smem(int optin) { return set_dynamic_smem(k_trace_pass, optin); }

void launch_trace_pass(int grid, size_t smem, cudaStream_t s, const TraceDesc* descs, int ndesc, uint8_t* gxz,
                       size_t xz_bytes, size_t hot_bytes, int xz_in_smem, int* status) {
  k_trace_pass<<<grid, kTracePassThreads, smem, s>>>(descs, ndesc, gxz, xz_bytes, hot_bytes, xz_in_smem, status);
}

bool launch_phase_pass(int tw, int grid, int block, cudaStream_t s, const TraceDesc* descs, int ndesc,
                       long long total_groups, int* status) {
  switch (tw) {
    case 2: k_phase_pass<2><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 4: k_phase_pass<4><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 8: k_phase_pass<8><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 16: k_phase_pass<16><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    case 32: k_phase_pass<32><<<grid, block, 0, s>>>(descs, ndesc, total_groups, status); return true;
    default: return false;
  }
}

}  // namespace sdim
