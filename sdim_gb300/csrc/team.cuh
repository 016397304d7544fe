// Thread teams: the threads that share one tableau slot.  WarpTeam is one
// warp (up to 32 slots per CTA); CtaTeam is a whole CTA (one slot per CTA,
// for programs with many qudits).  Both expose the same strided-loop index,
// barrier and reductions, so one engine source serves both.
#pragma once
#include <climits>
#include "common.cuh"

namespace sdim {

// Shared-memory ints a CtaTeam's reductions use (add3: three partial sums per
// warp of a CTA of up to 1024 threads, and the three results).
constexpr int kTeamRedInts = 3 * 32 + 8;

struct WarpTeam {
  int t;
  __device__ WarpTeam() : t(threadIdx.x & 31) {}
  __device__ __forceinline__ int size() const { return 32; }
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ int min(int v) const { return __reduce_min_sync(0xffffffffu, v); }
  __device__ __forceinline__ int add(int v) const { return __reduce_add_sync(0xffffffffu, v); }
  // Three sums at once.
  __device__ __forceinline__ void add3(int& a, int& b, int& c) const {
    a = __reduce_add_sync(0xffffffffu, a);
    b = __reduce_add_sync(0xffffffffu, b);
    c = __reduce_add_sync(0xffffffffu, c);
  }
  __device__ __forceinline__ unsigned bxor(unsigned v) const { return __reduce_xor_sync(0xffffffffu, v); }
  __device__ __forceinline__ bool any(bool b) const { return __any_sync(0xffffffffu, b); }
  __device__ __forceinline__ bool leader() const { return t == 0; }
};

// red: kTeamRedInts ints of shared memory owned by the team.
struct CtaTeam {
  int t, nt;
  int* red;
  __device__ CtaTeam(int* red_) : t(threadIdx.x), nt(blockDim.x), red(red_) {}
  __device__ __forceinline__ int size() const { return nt; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ bool leader() const { return t == 0; }
  __device__ __forceinline__ bool any(bool b) const { return __syncthreads_or(b) != 0; }
  template <class Op>
  __device__ __forceinline__ int reduce(int v, int ident, Op op) const {
    const int lane = t & 31, w = t >> 5, nw = (nt + 31) >> 5;
    for (int off = 16; off > 0; off >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
      int x = lane < nw ? red[lane] : ident;
      for (int off = 16; off > 0; off >>= 1) x = op(x, __shfl_xor_sync(0xffffffffu, x, off));
      if (lane == 0) red[32] = x;
    }
    __syncthreads();
    const int r = red[32];
    __syncthreads();
    return r;
  }
  __device__ __forceinline__ int min(int v) const {
    return reduce(v, INT_MAX, [](int a, int b) { return a < b ? a : b; });
  }
  __device__ __forceinline__ int add(int v) const {
    return reduce(v, 0, [](int a, int b) { return a + b; });
  }
  // Three sums over the CTA in the barriers of one (three sums one after the
  // other take three times as many): per-warp partials in red[3 w + i], the
  // totals in red[96 + i].
  __device__ __forceinline__ void add3(int& a, int& b, int& c) const {
    const int lane = t & 31, w = t >> 5, nw = (nt + 31) >> 5;
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, off);
      b += __shfl_xor_sync(0xffffffffu, b, off);
      c += __shfl_xor_sync(0xffffffffu, c, off);
    }
    if (lane == 0) {
      red[3 * w] = a;
      red[3 * w + 1] = b;
      red[3 * w + 2] = c;
    }
    __syncthreads();
    if (w == 0) {
      int x = lane < nw ? red[3 * lane] : 0, y = lane < nw ? red[3 * lane + 1] : 0,
          z = lane < nw ? red[3 * lane + 2] : 0;
      for (int off = 16; off > 0; off >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, off);
        y += __shfl_xor_sync(0xffffffffu, y, off);
        z += __shfl_xor_sync(0xffffffffu, z, off);
      }
      if (lane == 0) {
        red[96] = x;
        red[97] = y;
        red[98] = z;
      }
    }
    __syncthreads();
    a = red[96];
    b = red[97];
    c = red[98];
    __syncthreads();
  }
  __device__ __forceinline__ unsigned bxor(unsigned v) const {
    return (unsigned)reduce((int)v, 0, [](int a, int b) { return a ^ b; });
  }
};

// A CtaTeam whose x / z region streams from global memory when it does not
// fit in shared memory (the odd-d trace engine's single-CTA x / z pass): the
// rank-1 update keeps more rows in flight for it.
struct StreamCtaTeam : CtaTeam {
  __device__ explicit StreamCtaTeam(int* red_) : CtaTeam(red_) {}
};

}  // namespace sdim
