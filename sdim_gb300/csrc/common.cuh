// Shared definitions of the GB300 tableau engine: device opcodes, the packed
// instruction word, per-circuit descriptors and the Philox4x32-10 stream.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sdim {

// Device opcodes.  Values 1-10, 14 and 16 keep the reference's gate ids
// (sdim/gatedata.py:55-102, sdim/program.py:13-32).  CZ, CZ_INV, SWAP and
// M_X are expanded by the host encoder into the H/H_INV/CNOT sequences the
// reference itself applies (sdim/tableau/tableau_gates.py:229-329), and N1
// is split by channel.
enum DevOp : uint32_t {
  OP_NOP = 0,
  OP_X = 1,
  OP_X_INV = 2,
  OP_Z = 3,
  OP_Z_INV = 4,
  OP_H = 5,
  OP_H_INV = 6,
  OP_P = 7,
  OP_P_INV = 8,
  OP_CNOT = 9,
  OP_CNOT_INV = 10,
  OP_M = 14,
  OP_RESET = 16,
  OP_N1D = 17,   // depolarizing: X^a Z^b, (a,b) != (0,0)
  OP_N1F = 18,   // flip: X^a, a != 0
  OP_N1P = 19,   // phase: Z^b, b != 0
  OP_N1OFF = 20,  // N1 whose coin never fires (prob 0): only advances the noise ordinal
  OP_GROUP = 21,  // layered odd-d x / z streams only: y gates on pairwise disjoint qudits follow
  OP_RUN = 22     // layered odd-d x / z streams only: a run of gates (y words) follows
};

// Instruction word: x = opcode | qudit << 8; y = target qudit (two-qudit
// gates) or the N1 coin threshold (identity iff philox word0 < threshold).
__host__ __device__ inline uint32_t op_code(uint2 w) { return w.x & 0xffu; }
__host__ __device__ inline uint32_t op_qudit(uint2 w) { return w.x >> 8; }

// One circuit of a batch, resident on the device.
struct CircuitDesc {
  const uint2* ops;        // device instruction stream
  uint8_t* out;            // nshots x nmeas records: value | deterministic << 7
  unsigned long long seed;
  long long shot0;         // global index of the first shot (Philox counter)
  long long item_begin;    // first work-queue item of this circuit
  int nops;
  int n;                   // qudits
  int d;                   // prime dimension
  int nmeas;               // records per shot
  int nshots;
  int slot;                // tableau slot layout id (engine specific)
};

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds of two
// 32x32->64-bit multiplies with a Weyl key schedule.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Stream block for (seed, shot, ordinal, domain); domain 0 = measurement
// outcome, 1 = N1 noise.
__device__ __forceinline__ uint4 stream_block(unsigned long long seed, long long shot,
                                              uint32_t ordinal, uint32_t domain) {
  const unsigned long long s = (unsigned long long)shot;
  return philox4x32_10(make_uint4(ordinal, (uint32_t)s, (uint32_t)(s >> 32), domain),
                       make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

// Multiply-shift map of a 32-bit word onto [0, m).
__device__ __forceinline__ int mulshift(uint32_t w, uint32_t m) { return (int)__umulhi(w, m); }

// N1 coins: the coin of N1 ordinal j is word (j & 3) of the domain-1 block
// with counter ordinal j >> 2, so one Philox block serves four consecutive
// N1 instructions.  The cache holds the last block.
struct CoinCache {
  uint4 blk;
  uint32_t id;
  __device__ CoinCache() : blk(make_uint4(0u, 0u, 0u, 0u)), id(0xffffffffu) {}
  __device__ __forceinline__ uint32_t coin(unsigned long long seed, long long shot, uint32_t ordinal) {
    if ((ordinal >> 2) != id) {
      id = ordinal >> 2;
      blk = stream_block(seed, shot, id, 1u);
    }
    const uint32_t j = ordinal & 3u;
    return j == 0 ? blk.x : j == 1 ? blk.y : j == 2 ? blk.z : blk.w;
  }
};

// Exponents (a, b) of X^a Z^b for an N1 whose coin fired: word 0 of the
// domain-2 block (seed, shot, ordinal).  Channel draws follow the reference's
// frame-sampler draws (sdim/program.py:486-497): 'd' r in [1, d^2) with
// a = r % d, b = r / d; 'f' a in [1, d); 'p' b in [1, d).
__device__ __forceinline__ int2 noise_choice(uint32_t op, int d, unsigned long long seed, long long shot,
                                             uint32_t ordinal) {
  const uint4 w = stream_block(seed, shot, ordinal, 2u);
  if (op == OP_N1D) {
    const int r = 1 + mulshift(w.x, (uint32_t)(d * d - 1));
    return make_int2(r % d, r / d);
  }
  if (op == OP_N1F) return make_int2(1 + mulshift(w.x, (uint32_t)(d - 1)), 0);
  return make_int2(0, 1 + mulshift(w.x, (uint32_t)(d - 1)));
}

// Error codes written to the device status word.
enum DevStatus : int {
  DEV_OK = 0,
  DEV_BAD_OPCODE = 1,
  DEV_BAD_QUDIT = 2,
  DEV_SLOT_TOO_SMALL = 3
};

}  // namespace sdim
