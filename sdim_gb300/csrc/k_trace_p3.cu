// x / z pass of the odd-d trace engine for d = 3 on bit planes
// (trace_p3.cuh): one program per CTA -- of 64 to 512 threads in batches,
// 1024 for a lone program -- with the tableau in shared memory when it fits
// (n <= 448 on GB300), else in a global-memory slot per CTA with the CTAs
// taking programs, largest first, from an atomic counter.
#include "trace_p3.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

template <int TH>
__global__ void __launch_bounds__(TH, TH > kP3Threads ? 1 : 2)
    k_trace_pass_p3(const TraceDescU8* __restrict__ descs, int ndesc, uint8_t* gxz, size_t xz_bytes,
                    size_t hot_bytes, int xz_in_smem, unsigned* queue, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[kTeamRedInts];
  __shared__ int next;
  uint8_t* hot = smem;
  uint8_t* xz = xz_in_smem ? smem + hot_bytes : gxz + (size_t)blockIdx.x * xz_bytes;
  uint2* win = reinterpret_cast<uint2*>(smem + hot_bytes + (xz_in_smem ? xz_bytes : 0));
  int i = blockIdx.x;
  if (queue) {
    if (threadIdx.x == 0) next = (int)atomicAdd(queue, 1u);
    __syncthreads();
    i = next;
  }
  while (i < ndesc) {
    const TraceDescU8 td = descs[i];
    TabP3 e(xz, hot, td.c.n, CtaTeam(red), (int)blockDim.x);
    trace_program_p3(td, e, win, status);
    __syncthreads();
    if (queue) {
      if (threadIdx.x == 0) next = (int)atomicAdd(queue, 1u);
      __syncthreads();
      i = next;
    } else {
      i += gridDim.x;
    }
  }
}

}  // namespace

size_t trace_p3_hot_bytes(int n, int threads) { return round16(P3Layout(n).hot_bytes(threads)); }
size_t trace_p3_xz_bytes(int n) { return round16(P3Layout(n).xz_bytes()); }

cudaError_t trace_p3_set_smem(int optin) {
  const cudaError_t e = set_dynamic_smem(k_trace_pass_p3<kP3Threads>, optin);
  return e != cudaSuccess ? e : set_dynamic_smem(k_trace_pass_p3<kP3WideThreads>, optin);
}

void launch_trace_p3(int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd, uint8_t* gxz,
                     size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status) {
  if (block > kP3Threads)
    k_trace_pass_p3<kP3WideThreads><<<grid, block, smem, s>>>(d, nd, gxz, xzb, hot, in_smem, queue, status);
  else
    k_trace_pass_p3<kP3Threads><<<grid, block, smem, s>>>(d, nd, gxz, xzb, hot, in_smem, queue, status);
}

}  // namespace sdim
