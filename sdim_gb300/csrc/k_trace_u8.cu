// Trace engine kernels for odd prime d: the x / z pass (one CTA per
// program, TGroupU8 team with no live shots) and the phase pass (one CTA
// per 32-shot group, (shot, chunk) threads).  Instantiated for d = 3, 5, 7
// and a generic d.
#include "trace_cluster_u8.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

// One program per CTA at a time.  With queue (x / z in global memory, fewer
// CTAs than programs) every CTA takes the next program from the atomic
// counter, so the programs (largest first) are dealt out as CTAs free up;
// without, CTA b takes programs b, b + grid, ...
// Team: StreamCtaTeam (16 rows in flight) when the tableau streams from
// global memory, CtaTeam (8) when it sits in shared memory, which leaves the
// in-smem kernel registers to spare.
template <int DD, class Team>
__global__ void __launch_bounds__(kTracePassThreads) k_trace_pass_u8(const TraceDescU8* __restrict__ descs, int ndesc,
                                                                     uint8_t* gxz, size_t xz_bytes, size_t hot_bytes,
                                                                     int xz_in_smem, unsigned* queue, int* status) {
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
    TGroupU8<DD, Team> e(xz, hot, td.c.n, td.c.d, Team(red));
    trace_program_u8(td, e, win, status);
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

// One program per CTA pair (cluster of two, grid-stride over programs).
template <int DD>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kTracePassThreads)
    k_trace_pass_split(const TraceDescU8* __restrict__ descs, int ndesc, size_t win_off, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[kTeamRedInts];
  uint2* win = reinterpret_cast<uint2*>(smem + win_off);
  cluster_sync_all();  // both CTAs run before either writes into the other's shared memory
  for (int i = (int)(blockIdx.x >> 1); i < ndesc; i += (int)(gridDim.x >> 1)) {
    const TraceDescU8 td = descs[i];
    SplitU8<DD> e(smem, td.c.n, td.c.d, red);
    split_program(td, e, win, status);
  }
}

// One program per cluster of kTraceClusterCtas CTAs (grid-stride over programs,
// largest first).  kStream: each CTA's columns in its slot of gxz, else in
// its shared memory after the hot region.
template <int DD, bool kStream>
__global__ void __cluster_dims__(kTraceClusterCtas, 1, 1) __launch_bounds__(kTracePassThreads)
    k_trace_pass_cluster(const TraceDescU8* __restrict__ descs, int ndesc, uint8_t* gxz, size_t xz_bytes,
                         size_t hot_bytes, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[kTeamRedInts];
  uint8_t* xz = kStream ? gxz + (size_t)blockIdx.x * xz_bytes : smem + hot_bytes;
  uint2* win = reinterpret_cast<uint2*>(smem + hot_bytes + (kStream ? 0 : xz_bytes));
  cluster_sync_all();  // every CTA of the cluster runs before any writes into its shared memory
  for (int i = (int)(blockIdx.x / kTraceClusterCtas); i < ndesc; i += (int)(gridDim.x / kTraceClusterCtas)) {
    const TraceDescU8 td = descs[i];
    ClusterU8<DD, kTraceClusterCtas, kStream> e(smem, xz, td.c.n, td.c.d, red);
    cluster_program(td, e, win, status);
  }
}

// Deterministic headers of the cluster x / z pass: program blockIdx.y of
// descs, one warp per measurement.
__global__ void __launch_bounds__(128) k_cluster_det_headers(const TraceDescU8* __restrict__ descs, int ndesc,
                                                             const int* status) {
  if (*(volatile const int*)status != DEV_OK) return;  // the trace is incomplete
  const int i = (int)blockIdx.y;
  const int m = (int)blockIdx.x * 4 + (int)(threadIdx.x >> 5);
  if (i >= ndesc || m >= descs[i].nm) return;
  cluster_det_header<kTraceClusterCtas>(descs[i], m, (int)(threadIdx.x & 31));
}

template <int DD>
__global__ void __launch_bounds__(512) k_phase_pass_u8(const TraceDescU8* __restrict__ descs, int ndesc,
                                                       long long total_groups, const int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  if (*(volatile const int*)status != DEV_OK) return;  // the trace is incomplete
  const long long g = blockIdx.x;
  if (g >= total_groups) return;
  const int i = find_trace_desc_u8(descs, ndesc, g);
  phase_program_u8<DD>(descs + i, g - descs[i].c.item_begin, smem);
}

template <int DD>
struct TraceU8 {
  static cudaError_t set_smem(int optin) {
    cudaError_t e = set_dynamic_smem(k_trace_pass_u8<DD, CtaTeam>, optin);
    if (e == cudaSuccess) e = set_dynamic_smem(k_trace_pass_u8<DD, StreamCtaTeam>, optin);
    if (e == cudaSuccess) e = set_dynamic_smem(k_trace_pass_split<DD>, optin);
    if (e == cudaSuccess) e = set_dynamic_smem(k_trace_pass_cluster<DD, false>, optin);
    if (e == cudaSuccess) e = set_dynamic_smem(k_trace_pass_cluster<DD, true>, optin);
    return e != cudaSuccess ? e : set_dynamic_smem(k_phase_pass_u8<DD>, optin);
  }
  static void cluster(int clusters, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd, uint8_t* gxz,
                      size_t xzb, size_t hot, int in_smem, int* status) {
    const int grid = kTraceClusterCtas * clusters;
    if (in_smem)
      k_trace_pass_cluster<DD, false><<<grid, kTracePassThreads, smem, s>>>(d, nd, gxz, xzb, hot, status);
    else
      k_trace_pass_cluster<DD, true><<<grid, kTracePassThreads, smem, s>>>(d, nd, gxz, xzb, hot, status);
  }
  static void split(int pairs, size_t smem, size_t scratch_off, cudaStream_t s, const TraceDescU8* d, int nd,
                    int* status) {
    k_trace_pass_split<DD><<<2 * pairs, kTracePassThreads, smem, s>>>(d, nd, scratch_off, status);
  }
  static void xz(int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd, uint8_t* gxz,
                 size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status) {
    if (in_smem)
      k_trace_pass_u8<DD, CtaTeam><<<grid, block, smem, s>>>(d, nd, gxz, xzb, hot, in_smem, queue, status);
    else
      k_trace_pass_u8<DD, StreamCtaTeam><<<grid, block, smem, s>>>(d, nd, gxz, xzb, hot, in_smem, queue, status);
  }
  static void phase(int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd, long long total,
                    int* status) {
    k_phase_pass_u8<DD><<<grid, block, smem, s>>>(d, nd, total, status);
  }
};

}  // namespace

int trace_u8_variant(int d) { return d == 3 ? 0 : d == 5 ? 1 : d == 7 ? 2 : 3; }

cudaError_t trace_u8_set_smem(int optin) {
  cudaError_t e;
  if ((e = TraceU8<3>::set_smem(optin)) != cudaSuccess) return e;
  if ((e = TraceU8<5>::set_smem(optin)) != cudaSuccess) return e;
  if ((e = TraceU8<7>::set_smem(optin)) != cudaSuccess) return e;
  return TraceU8<0>::set_smem(optin);
}

size_t trace_u8_hot_bytes(int n) { return round16(SlotGroupU8::hot_bytes(n)); }
size_t trace_u8_xz_bytes(int n) { return round16(SlotGroupU8::xz_bytes(n)); }
size_t trace_u8_phase_smem(int n) { return round16(phase_u8_smem(n)); }
size_t trace_u8_split_smem(int n) { return round16(split_smem_bytes(n)); }
size_t trace_u8_window_bytes() { return sizeof(uint2) * kOpWindow; }
size_t trace_u8_cluster_hot(int n) { return round16(cluster_hot_bytes(n, kTraceClusterCtas)); }
size_t trace_u8_cluster_xz(int n) { return round16(cluster_xz_bytes(n, kTraceClusterCtas)); }
size_t trace_u8_cluster_det(int n) { return cluster_det_bytes(n, kTraceClusterCtas); }

void launch_cluster_det_headers(int maxnm, cudaStream_t s, const TraceDescU8* d, int nd, int* status) {
  if (maxnm <= 0) return;
  for (int b = 0; b < nd; b += 65535) {
    const dim3 grid((unsigned)((maxnm + 3) / 4), (unsigned)std::min(65535, nd - b));
    k_cluster_det_headers<<<grid, 128, 0, s>>>(d + b, nd - b, status);
  }
}

void launch_trace_u8_cluster(int variant, int clusters, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd,
                             uint8_t* gxz, size_t xzb, size_t hot, int in_smem, int* status) {
  switch (variant) {
    case 0: TraceU8<3>::cluster(clusters, smem, s, d, nd, gxz, xzb, hot, in_smem, status); break;
    case 1: TraceU8<5>::cluster(clusters, smem, s, d, nd, gxz, xzb, hot, in_smem, status); break;
    case 2: TraceU8<7>::cluster(clusters, smem, s, d, nd, gxz, xzb, hot, in_smem, status); break;
    default: TraceU8<0>::cluster(clusters, smem, s, d, nd, gxz, xzb, hot, in_smem, status); break;
  }
}

void launch_trace_u8_split(int variant, int pairs, size_t smem, size_t scratch_off, cudaStream_t s,
                           const TraceDescU8* d, int nd, int* status) {
  switch (variant) {
    case 0: TraceU8<3>::split(pairs, smem, scratch_off, s, d, nd, status); break;
    case 1: TraceU8<5>::split(pairs, smem, scratch_off, s, d, nd, status); break;
    case 2: TraceU8<7>::split(pairs, smem, scratch_off, s, d, nd, status); break;
    default: TraceU8<0>::split(pairs, smem, scratch_off, s, d, nd, status); break;
  }
}

void launch_trace_u8_xz(int variant, int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd,
                        uint8_t* gxz, size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status) {
  switch (variant) {
    case 0: TraceU8<3>::xz(grid, block, smem, s, d, nd, gxz, xzb, hot, in_smem, queue, status); break;
    case 1: TraceU8<5>::xz(grid, block, smem, s, d, nd, gxz, xzb, hot, in_smem, queue, status); break;
    case 2: TraceU8<7>::xz(grid, block, smem, s, d, nd, gxz, xzb, hot, in_smem, queue, status); break;
    default: TraceU8<0>::xz(grid, block, smem, s, d, nd, gxz, xzb, hot, in_smem, queue, status); break;
  }
}

void launch_trace_u8_phase(int variant, int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d,
                           int nd, long long total, int* status) {
  switch (variant) {
    case 0: TraceU8<3>::phase(grid, block, smem, s, d, nd, total, status); break;
    case 1: TraceU8<5>::phase(grid, block, smem, s, d, nd, total, status); break;
    case 2: TraceU8<7>::phase(grid, block, smem, s, d, nd, total, status); break;
    default: TraceU8<0>::phase(grid, block, smem, s, d, nd, total, status); break;
  }
}

}  // namespace sdim
