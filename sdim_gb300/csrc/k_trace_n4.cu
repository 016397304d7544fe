// x / z pass of the odd-d trace engine for d = 5 and 7 on 4-bit residue
// lanes (trace_n4.cuh): one program per CTA -- of 64 to 512 threads in
// batches, 1024 for a lone program -- with the tableau in shared memory when
// it fits, else in a global-memory slot per CTA with the CTAs taking
// programs, largest first, from an atomic counter.
#include "trace_n4.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

template <int DD, int TH>
__global__ void __launch_bounds__(TH, TH > kN4Threads ? 1 : 2)
    k_trace_pass_n4(const TraceDescU8* __restrict__ descs, int ndesc, uint8_t* gxz, size_t xz_bytes,
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
    TabN4<DD> e(xz, hot, td.c.n, CtaTeam(red), (int)blockDim.x);
    trace_program_n4<DD>(td, e, win, status);
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

template <int DD>
void launch_dd(int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* dsc, int nd, uint8_t* gxz,
               size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status) {
  if (block > kN4Threads)
    k_trace_pass_n4<DD, kN4WideThreads><<<grid, block, smem, s>>>(dsc, nd, gxz, xzb, hot, in_smem, queue, status);
  else
    k_trace_pass_n4<DD, kN4Threads><<<grid, block, smem, s>>>(dsc, nd, gxz, xzb, hot, in_smem, queue, status);
}

}  // namespace

size_t trace_n4_hot_bytes(int n, int d, int threads) {
  return round16(d == 5 ? N4Layout<5>(n).hot_bytes(threads) : N4Layout<7>(n).hot_bytes(threads));
}
size_t trace_n4_xz_bytes(int n) { return round16(N4Layout<5>(n).xz_bytes()); }

cudaError_t trace_n4_set_smem(int optin) {
  cudaError_t e = set_dynamic_smem(k_trace_pass_n4<5, kN4Threads>, optin);
  if (e == cudaSuccess) e = set_dynamic_smem(k_trace_pass_n4<7, kN4Threads>, optin);
  if (e == cudaSuccess) e = set_dynamic_smem(k_trace_pass_n4<5, kN4WideThreads>, optin);
  return e != cudaSuccess ? e : set_dynamic_smem(k_trace_pass_n4<7, kN4WideThreads>, optin);
}

void launch_trace_n4(int d, int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* dsc, int nd,
                     uint8_t* gxz, size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status) {
  if (d == 5)
    launch_dd<5>(grid, block, smem, s, dsc, nd, gxz, xzb, hot, in_smem, queue, status);
  else
    launch_dd<7>(grid, block, smem, s, dsc, nd, gxz, xzb, hot, in_smem, queue, status);
}

}  // namespace sdim
