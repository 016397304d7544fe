// Launch table of the engine variants.  Each variant's kernels are
// instantiated in their own translation unit (k_pershot.cu, k_group.cu) so
// the library compiles in parallel; abi.cu only sees these function pointers.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sdim {

enum Variant : int {
  // per-shot engines: one warp and one full tableau per shot
  V_BITS = 0,
  V_U8_3,
  V_U8_5,
  V_U8_7,
  V_U8_GEN,
  // shot-group engines: 32 shots share x / z; W = one warp per group, C = one CTA per group
  V_GBITS_W,
  V_GBITS_C,
  V_GU8_3_W,
  V_GU8_5_W,
  V_GU8_7_W,
  V_GU8_GEN_W,
  V_GU8_3_C,
  V_GU8_5_C,
  V_GU8_7_C,
  V_GU8_GEN_C,
  V_COUNT
};

// A slot is a shared-memory part of `hot` bytes plus a part of `big` bytes
// that sits in shared memory right after it (in_smem) or in global memory at
// gbuf + slot_index * big.  Per-shot engines have hot = 0 and keep the whole
// tableau in the big part; group engines keep the x / z blocks there.
struct VariantOps {
  int group;      // 1: items are 32-shot groups
  int cta;        // 1: one CTA per slot (block threads given by the planner)
  int max_block;  // threads per block of the persistent kernel
  size_t (*hot_bytes)(int n);
  size_t (*big_bytes)(int n);
  cudaError_t (*set_smem)(int bytes);
  int (*occupancy)(int block, size_t smem);
  void (*persistent)(dim3 grid, dim3 block, size_t smem, cudaStream_t s, const CircuitDesc* descs, int nc,
                     long long total, unsigned long long* counter, uint8_t* gbuf, size_t big, size_t hot,
                     int in_smem, int* status);
  // per-shot engines: one shot, one warp
  void (*single)(size_t smem, cudaStream_t s, const CircuitDesc* desc, long long shot, uint8_t* gbuf, int in_smem,
                 int* status);
  // tableau export of one shot (per-shot engines: shot index; group engines:
  // group 0 of desc, exported lane)
  void (*snapshot)(dim3 block, size_t smem, cudaStream_t s, const CircuitDesc* desc, long long shot_or_group,
                   uint8_t* gbuf, size_t big, size_t hot, int in_smem, int8_t* snap, int mode, int lane,
                   int* status);
};

// Shared memory the planner leaves for the kernels' static arrays.
constexpr int kStaticSmemReserve = 1024;

// Raises a kernel's dynamic shared-memory cap to the per-block opt-in limit
// minus the kernel's own static shared memory.
template <class K>
inline cudaError_t set_dynamic_smem(K kernel, int optin_bytes) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin_bytes - (int)a.sharedSizeBytes);
}

inline size_t round16(size_t b) { return (b + 15) & ~(size_t)15; }

const VariantOps& pershot_ops(int variant);
const VariantOps& group_ops(int variant);

inline const VariantOps& variant_ops(int v) { return v < V_GBITS_W ? pershot_ops(v) : group_ops(v); }

}  // namespace sdim
