// Allocation-free entry point: sdim_run_noalloc.
//
// Some callers cannot call cudaMalloc: code that runs under another
// framework's memory manager (a caching allocator that owns the device
// memory budget), a process whose device memory is fully pre-reserved, or a
// caller that must not create allocations at all on its hot path.  They can
// still provide input and output buffers.  This entry point runs the
// per-shot persistent kernel with every piece of scratch it needs -- the
// work-queue counter, the status word and the device copy of the instruction
// stream -- in one file-scope __device__ array of fixed size, so it never
// allocates device memory and never frees any.
//
// Limits and rules:
//   * scratch is kNoallocScratchBytes (1 MiB + 256 B) per device, held by every
//     device that loads the library until the process exits;
//   * at most kNoallocMaxOps device instructions (131,072; CZ / CZ_INV expand
//     to 3, SWAP to 9, M_X to 2); longer programs are rejected with
//     SDIM_EINVAL and a message;
//   * the tableau of one shot must fit in shared memory (no global-memory
//     tableau slots); larger programs are rejected with SDIM_EINVAL;
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (with that device current) and sets the kernels'
//     shared-memory attribute; make that first call before any stream capture.
//     Host threads that make their first calls at the same time are
//     serialised by a lock; later calls read the published setup without it;
//   * every call shares the array, which keeps the last call's contents: the
//     counter and the status word are cleared at the start of each call, and
//     calls that overlap on the GPU (several streams or host threads at once)
//     race on it;
//   * a program rejected part-way through encoding (a bad gate, qudit or
//     probability after the first 1,024 instructions) has already overwritten
//     the start of the array's instruction area; nothing reads it until the
//     next call rewrites it, so this is harmless under the rules above;
//   * the call is synchronous on the given stream.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/sdim_gb300.h"
#include "kernels.cuh"

using namespace sdim;

namespace {

constexpr size_t kNoallocHeaderBytes = 256;           // counter (8 B) + status (4 B), padded
constexpr int kNoallocMaxOps = 131072;                // device instructions
constexpr size_t kNoallocScratchBytes = kNoallocHeaderBytes + (size_t)kNoallocMaxOps * sizeof(uint2);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

struct DeviceSetup {
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  int smem_optin = 0;
  int num_sms = 0;
  std::atomic<bool> done{false};     // set (release) after the fields above
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_lock;  // serialises first calls; done is re-checked under it

template <class E>
__global__ void __launch_bounds__(1024) k_persistent_noalloc(CircuitDesc c, long long total_items,
                                                             unsigned char* scratch, size_t slot_bytes) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long* counter = reinterpret_cast<unsigned long long*>(scratch);
  int* status = reinterpret_cast<int*>(scratch + 8);
  c.ops = reinterpret_cast<const uint2*>(scratch + kNoallocHeaderBytes);
  uint8_t* slot = smem + (size_t)warp * slot_bytes;
  for (;;) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(counter, 1ull);
    it = __shfl_sync(0xffffffffu, it, 0);
    if ((long long)it >= total_items) break;
    run_shot<E, false>(c, (long long)it, slot, lane, nullptr, SNAP_NONE, status);
    if (*(volatile int*)status != DEV_OK) break;
  }
}

bool prime(int d) {
  if (d < 2) return false;
  for (int k = 2; k * k <= d; ++k)
    if (d % k == 0) return false;
  return true;
}

template <class E>
int launch_noalloc(const DeviceSetup& ds, const CircuitDesc& c, long long nshots, size_t slot, cudaStream_t s) {
  const int warps = (int)std::min<size_t>(32, (size_t)ds.smem_optin / slot);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_persistent_noalloc<E>, warps * 32, warps * slot) !=
      cudaSuccess)
    occ = 1;
  occ = occ < 1 ? 1 : occ;
  long long need = (nshots + warps - 1) / warps;
  long long blocks = (long long)ds.num_sms * occ;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_persistent_noalloc<E><<<(unsigned)blocks, warps * 32, warps * slot, s>>>(c, nshots, ds.scratch, slot);
  return cudaGetLastError() == cudaSuccess ? SDIM_OK : SDIM_ECUDA;
}

template <class E>
cudaError_t set_attr(int bytes) {
  return cudaFuncSetAttribute(k_persistent_noalloc<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace

extern "C" int sdim_run_noalloc(const int32_t* ops, int64_t nops, const double* noise_prob, int n, int d,
                                uint64_t seed, int64_t shot0, int64_t nshots, uint8_t* out_dev, void* stream,
                                char* err, size_t err_len) {
  auto fail = [&](int code, const char* msg) {
    if (err && err_len) {
      std::strncpy(err, msg, err_len - 1);
      err[err_len - 1] = 0;
    }
    return code;
  };
  if ((nops > 0 && !ops) || nops < 0 || nshots < 0) return fail(SDIM_EINVAL, "bad argument");
  if (n < 1 || d < 2) return fail(SDIM_EINVAL, "need n >= 1 and d >= 2");
  if (!prime(d)) return fail(SDIM_EUNSUPPORTED, "composite dimension");
  if (d > 127) return fail(SDIM_EUNSUPPORTED, "dimension above 127");
  if (nshots > 0x7fffffffLL) return fail(SDIM_EINVAL, "too many shots in one call");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(SDIM_ECUDA, "no current CUDA device");
  }
  DeviceSetup& ds = g_setup[dev];
  if (!ds.done.load(std::memory_order_acquire)) {
    // once per device, with that device current
    std::lock_guard<std::mutex> hold(g_setup_lock);
    if (!ds.done.load(std::memory_order_relaxed)) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) {
        cudaGetLastError();
        return fail(SDIM_ECUDA, "cudaGetSymbolAddress of the scratch array failed");
      }
      int smem = 0, sms = 0;
      if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return fail(SDIM_ECUDA, "device attribute query failed");
      }
      if (set_attr<EngineBits>(smem) != cudaSuccess || set_attr<EngineU8<3>>(smem) != cudaSuccess ||
          set_attr<EngineU8<5>>(smem) != cudaSuccess || set_attr<EngineU8<7>>(smem) != cudaSuccess ||
          set_attr<EngineU8<0>>(smem) != cudaSuccess) {
        cudaGetLastError();
        return fail(SDIM_ECUDA, "cudaFuncSetAttribute failed");
      }
      ds.scratch = static_cast<unsigned char*>(p);
      ds.smem_optin = smem;
      ds.num_sms = sms;
      ds.done.store(true, std::memory_order_release);
    }
  }
  const size_t slot = ((d == 2 ? EngineBits::slot_bytes(n) : SlotU8::bytes(n)) + 15) & ~(size_t)15;
  if (slot > (size_t)ds.smem_optin)
    return fail(SDIM_EINVAL, "tableau does not fit in shared memory: sdim_run_noalloc keeps no global slots");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // encode in fixed chunks on the stack and copy them into the scratch array.
  // The chunk is pageable host memory: cudaMemcpyAsync from pageable memory
  // returns only once the source has been staged, so the chunk can be
  // refilled as soon as the call returns.
  uint2 chunk[1024];
  int nchunk = 0, ndev = 0, nmeas = 0;
  auto flush = [&]() -> int {
    if (!nchunk) return SDIM_OK;
    if (cudaMemcpyAsync(ds.scratch + kNoallocHeaderBytes + (size_t)(ndev - nchunk) * sizeof(uint2), chunk,
                        (size_t)nchunk * sizeof(uint2), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return SDIM_ECUDA;
    nchunk = 0;
    return SDIM_OK;
  };
  int bad = 0;
  auto emit = [&](uint32_t op, int q, uint32_t y) {
    if (ndev >= kNoallocMaxOps) { bad = 1; return; }
    chunk[nchunk++] = make_uint2(op | ((uint32_t)q << 8), y);
    ++ndev;
    if (nchunk == 1024 && flush() != SDIM_OK) bad = 2;
  };
  for (int64_t i = 0; i < nops && !bad; ++i) {
    const int id = ops[4 * i], q = ops[4 * i + 1], t = ops[4 * i + 2], ch = ops[4 * i + 3];
    if (id < 0 || id > 17) return fail(SDIM_EINVAL, "Invalid gate value");
    if (q < 0 || q >= n) return fail(SDIM_EINVAL, "qudit index out of range");
    if (id >= 9 && id <= 13 && (t < 0 || t >= n)) return fail(SDIM_EINVAL, "target index out of range");
    switch (id) {
      case 0: emit(OP_NOP, q, 0); break;
      case 1: emit(OP_X, q, 0); break;
      case 2: emit(OP_X_INV, q, 0); break;
      case 3: emit(OP_Z, q, 0); break;
      case 4: emit(OP_Z_INV, q, 0); break;
      case 5: emit(OP_H, q, 0); break;
      case 6: emit(OP_H_INV, q, 0); break;
      case 7: emit(OP_P, q, 0); break;
      case 8: emit(OP_P_INV, q, 0); break;
      case 9: emit(OP_CNOT, q, t); break;
      case 10: emit(OP_CNOT_INV, q, t); break;
      case 11: emit(OP_H_INV, t, 0); emit(OP_CNOT, q, t); emit(OP_H, t, 0); break;
      case 12: emit(OP_H_INV, t, 0); emit(OP_CNOT_INV, q, t); emit(OP_H, t, 0); break;
      case 13:
        emit(OP_CNOT, q, t); emit(OP_H, q, 0); emit(OP_H, t, 0);
        emit(OP_CNOT, q, t); emit(OP_H, q, 0); emit(OP_H, t, 0);
        emit(OP_CNOT, q, t); emit(OP_H, t, 0); emit(OP_H, t, 0);
        break;
      case 14: emit(OP_M, q, 0); ++nmeas; break;
      case 15: emit(OP_H_INV, q, 0); emit(OP_M, q, 0); ++nmeas; break;
      case 16: emit(OP_RESET, q, 0); ++nmeas; break;
      case 17: {
        const double p = noise_prob ? noise_prob[i] : 0.01;
        if (!(p == p)) return fail(SDIM_EINVAL, "noise probability is NaN");
        if (ch < 1 || ch > 3) return fail(SDIM_EINVAL, "Must specify a valid noise channel.");
        const double thr = std::floor((1.0 - p) * 4294967296.0);
        if (thr >= 4294967296.0) emit(OP_N1OFF, q, 0);
        else emit(ch == 1 ? OP_N1D : ch == 2 ? OP_N1F : OP_N1P, q, thr <= 0.0 ? 0u : (uint32_t)thr);
        break;
      }
    }
  }
  if (bad == 1) return fail(SDIM_EINVAL, "program longer than the 131072 device instructions sdim_run_noalloc holds");
  if (bad == 2 || flush() != SDIM_OK) {
    cudaGetLastError();
    return fail(SDIM_ECUDA, "copy of the instruction stream failed");
  }
  if (nshots > 0 && nmeas > 0 && !out_dev) return fail(SDIM_EINVAL, "null output buffer");
  if (cudaMemsetAsync(ds.scratch, 0, kNoallocHeaderBytes, s) != cudaSuccess) {
    cudaGetLastError();
    return fail(SDIM_ECUDA, "clearing the scratch header failed");
  }
  if (nshots == 0) return cudaStreamSynchronize(s) == cudaSuccess ? SDIM_OK : fail(SDIM_ECUDA, "sync failed");
  CircuitDesc c;
  std::memset(&c, 0, sizeof(c));
  c.out = out_dev;
  c.seed = seed;
  c.shot0 = shot0;
  c.nops = ndev;
  c.n = n;
  c.d = d;
  c.nmeas = nmeas;
  c.nshots = (int)nshots;
  int rc;
  switch (d) {
    case 2: rc = launch_noalloc<EngineBits>(ds, c, nshots, slot, s); break;
    case 3: rc = launch_noalloc<EngineU8<3>>(ds, c, nshots, slot, s); break;
    case 5: rc = launch_noalloc<EngineU8<5>>(ds, c, nshots, slot, s); break;
    case 7: rc = launch_noalloc<EngineU8<7>>(ds, c, nshots, slot, s); break;
    default: rc = launch_noalloc<EngineU8<0>>(ds, c, nshots, slot, s); break;
  }
  if (rc != SDIM_OK) return fail(SDIM_ECUDA, "kernel launch failed");
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return fail(SDIM_ECUDA, "kernel failed");
  }
  int st = 0;
  if (cudaMemcpy(&st, ds.scratch + 8, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return fail(SDIM_ECUDA, "status read failed");
  }
  if (st != DEV_OK) return fail(SDIM_EDEVICE, "device reported a bad instruction");
  return SDIM_OK;
}
