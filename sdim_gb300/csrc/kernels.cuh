// Shot driver and kernels, templated over the tableau engine.
//
// run_shot() is Program._simulate_tableau's inner loop for one shot
// (sdim/program.py:308-351): fresh tableau, every instruction in order,
// measurement records in program order, RESET corrections
// (sdim/program.py:335-339).  N1 applies X^a Z^b from the noise stream.
#pragma once
#include "common.cuh"
#include "engine_bits.cuh"
#include "group_bits.cuh"
#include "group_u8.cuh"
#include "engine_u8.cuh"

namespace sdim {

constexpr uint32_t kOpMask = 0x7fu;
constexpr uint32_t kOpEnd = 0x80u;  // last device op of a user instruction

enum SnapMode : int { SNAP_NONE = 0, SNAP_EVERY_INSTRUCTION = 1, SNAP_AT_MEASUREMENT = 2, SNAP_FINAL = 3 };

template <class E, bool SNAP>
__device__ __forceinline__ void run_shot(const CircuitDesc& c, long long shot_local, uint8_t* slot,
                                         int lane, int8_t* snap, int snap_mode, int* status) {
  E eng(slot, c.n, c.d);
  eng.init(lane);
  const long long shot = c.shot0 + shot_local;
  uint8_t* out = c.out + shot_local * (long long)c.nmeas;
  const int n = c.n, d = c.d;
  const size_t tb = 4 * (size_t)n * n + 2 * (size_t)n;
  uint32_t mord = 0, nord = 0;
  CoinCache coins;
  long long user_ins = 0;
  uint2 w = (c.nops > 0) ? __ldg(c.ops) : make_uint2(0u, 0u);
  for (int i = 0; i < c.nops; ++i) {
    const uint2 cur = w;
    if (i + 1 < c.nops) w = __ldg(c.ops + i + 1);  // prefetch the next word
    const uint32_t op = cur.x & kOpMask;
    const int q = (int)(cur.x >> 8);
    if (q >= n) {
      if (lane == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      return;
    }
    switch (op) {
      case OP_NOP: break;
      case OP_X: eng.pauli(lane, q, d - 1, 0); break;
      case OP_X_INV: eng.pauli(lane, q, 1, 0); break;
      case OP_Z: eng.pauli(lane, q, 0, 1); break;
      case OP_Z_INV: eng.pauli(lane, q, 0, d - 1); break;
      case OP_H: eng.h(lane, q); break;
      case OP_H_INV: eng.h_inv(lane, q); break;
      case OP_P: eng.p(lane, q, false); break;
      case OP_P_INV: eng.p(lane, q, true); break;
      case OP_CNOT:
      case OP_CNOT_INV: {
        const int t = (int)cur.y;
        if (t >= n) {
          if (lane == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
          return;
        }
        eng.cnot(lane, q, t, op == OP_CNOT_INV);
        break;
      }
      case OP_M:
      case OP_RESET: {
        int det = 0;
        const int m = eng.measure(lane, q, c.seed, shot, mord, &det);
        if (SNAP && snap_mode == SNAP_AT_MEASUREMENT) eng.export_tableau(lane, snap + (size_t)mord * tb);
        if (op == OP_RESET) eng.reset_fix(lane, q, m);
        if (lane == 0 && (int)mord < c.nmeas) out[mord] = (uint8_t)(m | (det << 7));
        ++mord;
        break;
      }
      case OP_N1D:
      case OP_N1F:
      case OP_N1P: {
        if (coins.coin(c.seed, shot, nord) >= cur.y) {
          const int2 ab = noise_choice(op, d, c.seed, shot, nord);
          eng.pauli(lane, q, ab.x ? d - ab.x : 0, ab.y);
        }
        ++nord;
        break;
      }
      case OP_N1OFF: ++nord; break;
      default:
        if (lane == 0) atomicCAS(status, DEV_OK, DEV_BAD_OPCODE);
        return;
    }
    if (SNAP && snap_mode == SNAP_EVERY_INSTRUCTION && (cur.x & kOpEnd)) {
      eng.export_tableau(lane, snap + (size_t)user_ins * tb);
      ++user_ins;
    }
  }
  if (SNAP && snap_mode == SNAP_FINAL) eng.export_tableau(lane, snap);
  __syncwarp();
}

// One group of up to 32 shots of one program on one team.  Thread t < 32
// owns shot t's scalar work (coins, outcomes, records); the engine spreads
// per-shot vector work over (shot, chunk) pairs.  snap_lane >= 0 exports that
// shot's tableau according to snap_mode.
template <class G, bool SNAP>
__device__ __forceinline__ void run_tgroup(const CircuitDesc& c, long long group, G& eng, int8_t* snap,
                                           int snap_mode, int snap_lane, int* status) {
  const int t = eng.tm.t;
  const int s = t & 31;
  const long long base = group * 32;
  const long long left = (long long)c.nshots - base;
  const int nact = left >= 32 ? 32 : (int)left;
  eng.init(nact);
  const bool active = t < 32 && s < nact;
  const long long shot = c.shot0 + base + s;
  uint8_t* out = c.out + (active ? base + s : 0) * (long long)c.nmeas;
  const int n = c.n, d = c.d;
  const size_t tb = 4 * (size_t)n * n + 2 * (size_t)n;
  uint32_t mord = 0, nord = 0;
  CoinCache coins;
  long long user_ins = 0;
  uint2 w = (c.nops > 0) ? __ldg(c.ops) : make_uint2(0u, 0u);
  for (int i = 0; i < c.nops; ++i) {
    const uint2 cur = w;
    if (i + 1 < c.nops) w = __ldg(c.ops + i + 1);
    const uint32_t op = cur.x & kOpMask;
    const int q = (int)(cur.x >> 8);
    if (q >= n) {
      if (t == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
      return;
    }
    switch (op) {
      case OP_NOP: break;
      case OP_X: eng.pauli(q, d - 1, 0); break;
      case OP_X_INV: eng.pauli(q, 1, 0); break;
      case OP_Z: eng.pauli(q, 0, 1); break;
      case OP_Z_INV: eng.pauli(q, 0, d - 1); break;
      case OP_H: eng.h(q); break;
      case OP_H_INV: eng.h_inv(q); break;
      case OP_P: eng.p(q, false); break;
      case OP_P_INV: eng.p(q, true); break;
      case OP_CNOT:
      case OP_CNOT_INV: {
        const int tq = (int)cur.y;
        if (tq >= n) {
          if (t == 0) atomicCAS(status, DEV_OK, DEV_BAD_QUDIT);
          return;
        }
        eng.cnot(q, tq, op == OP_CNOT_INV);
        break;
      }
      case OP_M:
      case OP_RESET: {
        const int det = eng.measure(q, c.seed, c.shot0 + base, mord);
        if (SNAP && snap_mode == SNAP_AT_MEASUREMENT) eng.export_shot(snap_lane, snap + (size_t)mord * tb);
        const int m = (t < 32) ? eng.shot_m[s] : 0;
        if (op == OP_RESET) eng.reset_fix(q);
        if (active && (int)mord < c.nmeas) out[mord] = (uint8_t)(m | (det << 7));
        ++mord;
        break;
      }
      case OP_N1D:
      case OP_N1F:
      case OP_N1P: {
        const bool fire = active && coins.coin(c.seed, shot, nord) >= cur.y;
        if (eng.tm.any(fire)) {
          if (t < 32) {
            int2 ab = make_int2(0, 0);
            if (fire) ab = noise_choice(op, d, c.seed, shot, nord);
            eng.set_shot_ab(s, ab.x ? d - ab.x : 0, ab.y);
          }
          eng.shot_pauli(q);
        }
        ++nord;
        break;
      }
      case OP_N1OFF: ++nord; break;
      default:
        if (t == 0) atomicCAS(status, DEV_OK, DEV_BAD_OPCODE);
        return;
    }
    if (SNAP && snap_mode == SNAP_EVERY_INSTRUCTION && (cur.x & kOpEnd)) {
      eng.export_shot(snap_lane, snap + (size_t)user_ins * tb);
      ++user_ins;
    }
  }
  if (SNAP && snap_mode == SNAP_FINAL) eng.export_shot(snap_lane, snap);
  eng.tm.sync();
}

template <class G>
__device__ __forceinline__ int find_desc(const CircuitDesc* descs, int ncirc, long long it) {
  int lo = 0, hi = ncirc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (descs[mid].item_begin <= it) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Group slots: a hot region (hot_bytes, always shared memory) and an x / z
// region (xz_bytes) in shared memory right after it when xz_in_smem, else in
// global memory at gxz + slot * xz_bytes.

// Persistent shot-group kernel, one warp per group: items are
// (program, group of 32 shots); each warp owns one slot.
template <class G>
__global__ void __launch_bounds__(G::kWarpBlockMax) k_group_warp(const CircuitDesc* __restrict__ descs, int ncirc,
                                                     long long total_items, unsigned long long* __restrict__ counter,
                                                     uint8_t* gxz, size_t xz_bytes, size_t hot_bytes, int xz_in_smem,
                                                     int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  uint8_t* hot = smem + (size_t)warp * (hot_bytes + (xz_in_smem ? xz_bytes : 0));
  uint8_t* xz = xz_in_smem ? hot + hot_bytes : gxz + ((size_t)blockIdx.x * wpb + warp) * xz_bytes;
  for (;;) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(counter, 1ull);
    it = __shfl_sync(0xffffffffu, it, 0);
    if ((long long)it >= total_items) break;
    const int ci = find_desc<G>(descs, ncirc, (long long)it);
    const CircuitDesc c = descs[ci];
    G eng(xz, hot, c.n, c.d, WarpTeam());
    run_tgroup<G, false>(c, (long long)it - c.item_begin, eng, nullptr, SNAP_NONE, 0, status);
    if (*(volatile int*)status != DEV_OK) break;
  }
}

// Persistent shot-group kernel, one CTA per group (programs with many
// qudits): the whole CTA shares one slot.
template <class G>
__global__ void __launch_bounds__(512) k_group_cta(const CircuitDesc* __restrict__ descs, int ncirc,
                                                   long long total_items, unsigned long long* __restrict__ counter,
                                                   uint8_t* gxz, size_t xz_bytes, size_t hot_bytes, int xz_in_smem,
                                                   int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[kTeamRedInts];
  __shared__ long long item;
  uint8_t* hot = smem;
  uint8_t* xz = xz_in_smem ? smem + hot_bytes : gxz + (size_t)blockIdx.x * xz_bytes;
  for (;;) {
    if (threadIdx.x == 0) item = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const long long it = item;
    __syncthreads();
    if (it >= total_items) break;
    const int ci = find_desc<G>(descs, ncirc, it);
    const CircuitDesc c = descs[ci];
    G eng(xz, hot, c.n, c.d, CtaTeam(red));
    run_tgroup<G, false>(c, it - c.item_begin, eng, nullptr, SNAP_NONE, 0, status);
    __syncthreads();
    if (*(volatile int*)status != DEV_OK) break;
  }
}

// One group with the tableau of shot (group * 32 + snap_lane) exported;
// CTA-team engines run with blockDim threads, warp-team engines with 32.
template <class G, bool CTA>
__global__ void __launch_bounds__(512) k_group_snapshot(const CircuitDesc* __restrict__ desc, long long group,
                                                        uint8_t* gxz, size_t xz_bytes, size_t hot_bytes,
                                                        int xz_in_smem, int8_t* snap, int snap_mode, int snap_lane,
                                                        int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int red[kTeamRedInts];
  const CircuitDesc c = *desc;
  uint8_t* hot = smem;
  uint8_t* xz = xz_in_smem ? smem + hot_bytes : gxz;
  (void)xz_bytes;
  if constexpr (CTA) {
    G eng(xz, hot, c.n, c.d, CtaTeam(red));
    run_tgroup<G, true>(c, group, eng, snap, snap_mode, snap_lane, status);
  } else {
    G eng(xz, hot, c.n, c.d, WarpTeam());
    run_tgroup<G, true>(c, group, eng, snap, snap_mode, snap_lane, status);
  }
}

// Persistent batched kernel: every warp owns one tableau slot (shared memory
// when smem_slots != 0, else a global-memory slot) and pulls (circuit, shot)
// items from a device work queue until it is empty.
template <class E>
__global__ void __launch_bounds__(1024) k_persistent(const CircuitDesc* __restrict__ descs, int ncirc,
                                                     long long total_items,
                                                     unsigned long long* __restrict__ counter,
                                                     uint8_t* gslots, size_t slot_bytes,
                                                     int smem_slots, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  uint8_t* slot = smem_slots ? smem + (size_t)warp * slot_bytes
                             : gslots + ((size_t)blockIdx.x * wpb + warp) * slot_bytes;
  for (;;) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(counter, 1ull);
    it = __shfl_sync(0xffffffffu, it, 0);
    if ((long long)it >= total_items) break;
    int lo = 0, hi = ncirc - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (descs[mid].item_begin <= (long long)it) lo = mid; else hi = mid - 1;
    }
    const CircuitDesc c = descs[lo];
    run_shot<E, false>(c, (long long)it - c.item_begin, slot, lane, nullptr, SNAP_NONE, status);
    if (*(volatile int*)status != DEV_OK) break;
  }
}

// One shot, one warp: the plain per-shot form (one launch per shot).
template <class E>
__global__ void __launch_bounds__(32) k_single(const CircuitDesc* __restrict__ desc, long long shot_local,
                                               uint8_t* gslot, int smem_slot, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const CircuitDesc c = *desc;
  run_shot<E, false>(c, shot_local, smem_slot ? smem : gslot, threadIdx.x & 31, nullptr, SNAP_NONE,
                     status);
}

// One shot with tableau export (record_tableau / per-instruction parity).
template <class E>
__global__ void __launch_bounds__(32) k_snapshot(const CircuitDesc* __restrict__ desc, long long shot_local,
                                                 uint8_t* gslot, int smem_slot, int8_t* snap,
                                                 int snap_mode, int* status) {
  extern __shared__ __align__(16) uint8_t smem[];
  const CircuitDesc c = *desc;
  run_shot<E, true>(c, shot_local, smem_slot ? smem : gslot, threadIdx.x & 31, snap, snap_mode, status);
}

}  // namespace sdim
