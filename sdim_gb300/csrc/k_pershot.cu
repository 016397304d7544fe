// Per-shot engines (one warp, one full tableau per shot): kernel
// instantiations and their launch table.
#include "kernels.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

template <class E>
struct PerShot {
  static size_t hot_bytes(int) { return 0; }
  static size_t big_bytes(int n) { return round16(E::slot_bytes(n)); }
  static cudaError_t set_smem(int bytes) {
    cudaError_t e = set_dynamic_smem(k_persistent<E>, bytes);
    if (e != cudaSuccess) return e;
    e = set_dynamic_smem(k_single<E>, bytes);
    if (e != cudaSuccess) return e;
    return set_dynamic_smem(k_snapshot<E>, bytes);
  }
  static int occupancy(int block, size_t smem) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_persistent<E>, block, smem) != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return nb < 1 ? 1 : nb;
  }
  static void persistent(dim3 g, dim3 b, size_t smem, cudaStream_t s, const CircuitDesc* descs, int nc,
                         long long total, unsigned long long* counter, uint8_t* gbuf, size_t big, size_t,
                         int in_smem, int* status) {
    k_persistent<E><<<g, b, smem, s>>>(descs, nc, total, counter, gbuf, big, in_smem, status);
  }
  static void single(size_t smem, cudaStream_t s, const CircuitDesc* desc, long long shot, uint8_t* gbuf,
                     int in_smem, int* status) {
    k_single<E><<<1, 32, smem, s>>>(desc, shot, gbuf, in_smem, status);
  }
  static void snapshot(dim3, size_t smem, cudaStream_t s, const CircuitDesc* desc, long long shot, uint8_t* gbuf,
                       size_t, size_t, int in_smem, int8_t* snap, int mode, int, int* status) {
    k_snapshot<E><<<1, 32, smem, s>>>(desc, shot, gbuf, in_smem, snap, mode, status);
  }
  static const VariantOps& ops() {
    static const VariantOps o = {0, 0, 1024, hot_bytes, big_bytes, set_smem, occupancy, persistent, single,
                                 snapshot};
    return o;
  }
};

}  // namespace

const VariantOps& pershot_ops(int v) {
  switch (v) {
    case V_BITS: return PerShot<EngineBits>::ops();
    case V_U8_3: return PerShot<EngineU8<3>>::ops();
    case V_U8_5: return PerShot<EngineU8<5>>::ops();
    case V_U8_7: return PerShot<EngineU8<7>>::ops();
    default: return PerShot<EngineU8<0>>::ops();
  }
}

}  // namespace sdim
