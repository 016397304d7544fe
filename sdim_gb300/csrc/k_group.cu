// Shot-group engines (32 shots share x / z): kernel instantiations and their
// launch table, for warp teams (one warp per group) and CTA teams (one CTA
// per group).
#include "kernels.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

template <class G, bool CTA>
struct Group {
  static size_t hot_bytes(int n) { return round16(G::hot_bytes(n)); }
  static size_t big_bytes(int n) { return round16(G::xz_bytes(n)); }
  static cudaError_t set_smem(int bytes) {
    cudaError_t e;
    if constexpr (CTA)
      e = set_dynamic_smem(k_group_cta<G>, bytes);
    else
      e = set_dynamic_smem(k_group_warp<G>, bytes);
    if (e != cudaSuccess) return e;
    return set_dynamic_smem(k_group_snapshot<G, CTA>, bytes);
  }
  static int occupancy(int block, size_t smem) {
    int nb = 0;
    cudaError_t e;
    if constexpr (CTA)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_group_cta<G>, block, smem);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_group_warp<G>, block, smem);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return nb < 1 ? 1 : nb;
  }
  static void persistent(dim3 g, dim3 b, size_t smem, cudaStream_t s, const CircuitDesc* descs, int nc,
                         long long total, unsigned long long* counter, uint8_t* gbuf, size_t big, size_t hot,
                         int in_smem, int* status) {
    if constexpr (CTA)
      k_group_cta<G><<<g, b, smem, s>>>(descs, nc, total, counter, gbuf, big, hot, in_smem, status);
    else
      k_group_warp<G><<<g, b, smem, s>>>(descs, nc, total, counter, gbuf, big, hot, in_smem, status);
  }
  static void snapshot(dim3 block, size_t smem, cudaStream_t s, const CircuitDesc* desc, long long group,
                       uint8_t* gbuf, size_t big, size_t hot, int in_smem, int8_t* snap, int mode, int lane,
                       int* status) {
    k_group_snapshot<G, CTA><<<1, CTA ? block : dim3(32), smem, s>>>(desc, group, gbuf, big, hot, in_smem, snap,
                                                                     mode, lane, status);
  }
  static const VariantOps& ops() {
    static const VariantOps o = {1, CTA ? 1 : 0, CTA ? 512 : G::kWarpBlockMax, hot_bytes, big_bytes, set_smem,
                                 occupancy, persistent, nullptr, snapshot};
    return o;
  }
};

}  // namespace

const VariantOps& group_ops(int v) {
  switch (v) {
    case V_GBITS_W: return Group<TGroupBits<WarpTeam>, false>::ops();
    case V_GBITS_C: return Group<TGroupBits<CtaTeam>, true>::ops();
    case V_GU8_3_W: return Group<TGroupU8<3, WarpTeam>, false>::ops();
    case V_GU8_5_W: return Group<TGroupU8<5, WarpTeam>, false>::ops();
    case V_GU8_7_W: return Group<TGroupU8<7, WarpTeam>, false>::ops();
    case V_GU8_GEN_W: return Group<TGroupU8<0, WarpTeam>, false>::ops();
    case V_GU8_3_C: return Group<TGroupU8<3, CtaTeam>, true>::ops();
    case V_GU8_5_C: return Group<TGroupU8<5, CtaTeam>, true>::ops();
    case V_GU8_7_C: return Group<TGroupU8<7, CtaTeam>, true>::ops();
    default: return Group<TGroupU8<0, CtaTeam>, true>::ops();
  }
}

}  // namespace sdim
