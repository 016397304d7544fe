// Frame kernel of the Pauli-frame sampler (frame.cuh): one single-warp block
// per 32 frame shots, lane = shot.  The frames live in shared memory as one
// byte per qudit and shot, X[q][32] and Z[q][32], so the gates of the
// warp-uniform instruction stream touch one byte per lane each.  Records are
// staged per warp and written 64 measurements at a time, as in the trace
// engine's phase pass.
#include "engine_u8.cuh"
#include "frame.cuh"
#include "variants.cuh"

namespace sdim {
namespace {

constexpr int kFrameRecWindow = 64;
constexpr int kFrameRecStride = 68;

// The last Philox block of one domain, reused for four consecutive events.
struct BlockCache {
  uint4 blk = make_uint4(0u, 0u, 0u, 0u);
  uint32_t id = 0xffffffffu;
  __device__ __forceinline__ uint32_t word(unsigned long long seed, long long shot, uint32_t event,
                                           uint32_t domain) {
    if ((event >> 2) != id) {
      id = event >> 2;
      blk = stream_block(seed, shot, id, domain);
    }
    const uint32_t j = event & 3u;
    return j == 0 ? blk.x : j == 1 ? blk.y : j == 2 ? blk.z : blk.w;
  }
};

__device__ __forceinline__ void flush_frame_records(const uint8_t* rec, uint8_t* __restrict__ g, int nmeas,
                                                    int rows, int k0, int cnt, int lane) {
  __syncwarp();
  const uint8_t* b = rec + lane;
  uint8_t* o = g + k0 + lane;
  const bool lo = lane < cnt, hi = lane + 32 < cnt;
  for (int r = 0; r < rows; ++r) {
    if (lo) o[0] = b[0];
    if (hi) o[32] = b[32];
    o += nmeas;
    b += kFrameRecStride;
  }
  __syncwarp();
}

// Frame rules of sdim/program.py:82-162 on residues kept in [0, d).
template <int DD>
__global__ void __launch_bounds__(32) k_frame_pass(const FrameDesc fd, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x;
  const int n = fd.n, nmeas = fd.nmeas;
  const long long first = (long long)blockIdx.x * 32;
  if (first >= fd.nshots) return;
  const long long rel = first + lane;
  const bool active = rel < fd.nshots;
  const long long shot = fd.shot0 + rel;
  const unsigned long long seed = fd.seed;
  const ModU8<DD> M(fd.d);
  const uint32_t d = (uint32_t)M.d;
  uint8_t* X = smem;
  uint8_t* Z = X + (size_t)n * 32;
  uint8_t* rec = Z + (size_t)n * 32;
  uint8_t* myrec = rec + lane * kFrameRecStride;
  const int rows = (int)min(32LL, (long long)fd.nshots - first);
  uint8_t* __restrict__ gout = fd.out + first * (long long)nmeas;
  // x = 0, z = a uniform residue (sdim/program.py:63-64)
  BlockCache fr;
  for (int q = 0; q < n; ++q) {
    X[q * 32 + lane] = 0;
    Z[q * 32 + lane] = (uint8_t)mulshift(fr.word(seed, shot, (uint32_t)q, kDomainFrame), d);
  }
  BlockCache coins;
  uint32_t k = 0, j = 0;
  for (int i = 0; i < fd.nops; ++i) {
    const uint2 w = __ldg(fd.ops + i);
    const uint32_t op = w.x & 0xffu;
    const int q = (int)(w.x >> 8);
    const bool two = op >= OP_CNOT && op <= FOP_SWAP;
    if (q >= n || (two && (int)w.y >= n)) {
      if (lane == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      return;
    }
    const int t = two ? (int)w.y : q;
    uint8_t* xq = X + q * 32 + lane;
    uint8_t* zq = Z + q * 32 + lane;
    uint8_t* xt = X + t * 32 + lane;
    uint8_t* zt = Z + t * 32 + lane;
    switch (op) {
      case OP_H: {
        const int a = *xq, b = *zq;
        *xq = (uint8_t)M.neg(b);
        *zq = (uint8_t)a;
        break;
      }
      case OP_H_INV: {
        const int a = *xq, b = *zq;
        *xq = (uint8_t)b;
        *zq = (uint8_t)M.neg(a);
        break;
      }
      case OP_P: *zq = (uint8_t)M.md(*zq + *xq); break;
      case OP_P_INV: *zq = (uint8_t)M.md(*zq + (int)d - *xq); break;
      case OP_CNOT: {
        const int a = *xq, b = *zt;
        *xt = (uint8_t)M.md(*xt + a);
        *zq = (uint8_t)M.md(*zq + (int)d - b);
        break;
      }
      case OP_CNOT_INV: {
        const int a = *xq, b = *zt;
        *xt = (uint8_t)M.md(*xt + (int)d - a);
        *zq = (uint8_t)M.md(*zq + b);
        break;
      }
      case FOP_CZ:  // z_t += x_c, then z_c += x_t (in this order for c == t)
        *zt = (uint8_t)M.md(*zt + *xq);
        *zq = (uint8_t)M.md(*zq + *xt);
        break;
      case FOP_CZ_INV:
        *zt = (uint8_t)M.md(*zt + (int)d - *xq);
        *zq = (uint8_t)M.md(*zq + (int)d - *xt);
        break;
      case FOP_SWAP: {
        const uint8_t a = *xq, b = *xt, c = *zq, e = *zt;
        *xq = b;
        *xt = a;
        *zq = e;
        *zt = c;
        break;
      }
      case OP_M:
      case FOP_MX:
      case OP_RESET: {
        if ((int)k >= nmeas) {
          if (lane == 0) atomicCAS(status, DEV_OK, DEV_SLOT_TOO_SMALL);
          return;
        }
        const uint8_t rv = __ldg(fd.ref + k);
        uint8_t r;
        if (op == OP_RESET) {
          r = rv;  // the reference value, not frame-adjusted (sdim/program.py:146-155)
          *xq = 0;
        } else {
          if (op == FOP_MX) {
            const int a = *xq, b = *zq;
            *xq = (uint8_t)b;
            *zq = (uint8_t)M.neg(a);
          }
          r = (uint8_t)(M.md((rv & 0x7f) + *xq) | (rv & 0x80));
        }
        *zq = (uint8_t)mulshift(fr.word(seed, shot, (uint32_t)n + k, kDomainFrame), d);
        myrec[k & (kFrameRecWindow - 1)] = r;
        if ((k & (kFrameRecWindow - 1)) == kFrameRecWindow - 1 || (int)k == nmeas - 1) {
          const int k0 = (int)(k & ~(uint32_t)(kFrameRecWindow - 1));
          flush_frame_records(rec, gout, nmeas, rows, k0, (int)k + 1 - k0, lane);
        }
        ++k;
        break;
      }
      case OP_N1D:
      case OP_N1F:
      case OP_N1P: {
        const uint32_t coin = coins.word(seed, shot, j, 1u);
        if (active && coin >= w.y) {
          const int2 ab = noise_choice(op, (int)d, seed, shot, j);
          *xq = (uint8_t)M.md(*xq + ab.x);
          *zq = (uint8_t)M.md(*zq + ab.y);
        }
        ++j;
        break;
      }
      case OP_N1OFF: ++j; break;
      default: break;  // X, X_INV, Z, Z_INV leave the frame unchanged
    }
  }
}

template <int DD>
cudaError_t set_frame_smem(int optin) {
  return set_dynamic_smem(k_frame_pass<DD>, optin);
}

}  // namespace

size_t frame_smem_bytes(int n) { return round16((size_t)64 * n + 32 * kFrameRecStride); }

cudaError_t frame_set_smem(int optin) {
  cudaError_t e;
  if ((e = set_frame_smem<2>(optin)) != cudaSuccess) return e;
  if ((e = set_frame_smem<3>(optin)) != cudaSuccess) return e;
  if ((e = set_frame_smem<5>(optin)) != cudaSuccess) return e;
  if ((e = set_frame_smem<7>(optin)) != cudaSuccess) return e;
  return set_frame_smem<0>(optin);
}

bool launch_frame_pass(int grid, size_t smem, cudaStream_t s, const FrameDesc& fd, int* status) {
  switch (fd.d) {
    case 2: k_frame_pass<2><<<grid, 32, smem, s>>>(fd, status); return true;
    case 3: k_frame_pass<3><<<grid, 32, smem, s>>>(fd, status); return true;
    case 5: k_frame_pass<5><<<grid, 32, smem, s>>>(fd, status); return true;
    case 7: k_frame_pass<7><<<grid, 32, smem, s>>>(fd, status); return true;
    default: k_frame_pass<0><<<grid, 32, smem, s>>>(fd, status); return true;
  }
}

}  // namespace sdim
