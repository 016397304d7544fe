// Trace engine for d = 2: the shot-independent part of a program (x / z
// blocks and the common phase c) runs once per program; every shot then
// replays only its own phase deltas from a trace of what those read.  This
// header is what the host side sees: the per-program descriptor and the two
// launchers (k_trace.cu).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sdim {

// Trace of one program, written by the x / z pass, read by the phase pass.
//   mhdr[k] (measurement k, M or RESET in program order):
//     x = bit 0 deterministic, bit 1 RESET
//     y = pivot generator p (random measurements)
//     z = number of N1 ordinals before the measurement
//     w = common outcome phase aph_c (deterministic measurements)
//   mrow[k][0][tw]: factor words -- random: x_q over the 2n generators with
//     bit p cleared; deterministic: the destabilizer half of x_q (Wn words)
//   mrow[k][1][tw]: z_q after the measurement (RESET only)
//   nrow[j][0][tw], nrow[j][1][tw]: x_q and z_q at N1 ordinal j
// Rows are tw words (a power of two >= 2 Wn), zero past 2 Wn.  From the
// program's blob (built by the host encoder, see append_schedule in abi.cu):
// the layered schedule the x / z pass walks (steps, lops, wins), the N1
// coin thresholds nthr[j] (padded to a multiple of 64 ordinals with
// 0xffffffff) and nhdr[j] = (threshold, opcode).  masks, when not null,
// holds the fired Paulis of every shot as word pairs, pair c * nshots + s:
// bit i of the first word = N1 ordinal 32 c + i of shot s applied X^a with
// a odd, of the second = Z^b with b odd (written by the coin pass), and
// cmap its chunk map: bit i of word w * nshots + s set when pair (32 w + i)
// of shot s is not zero (bits at or past nchunk are undefined).
struct TraceDesc {
  CircuitDesc c;  // item_begin counts the phase pass's groups of 32 spl shots
  const uint4* steps;
  const uint4* lops;
  const uint4* wins;
  const uint32_t* nthr;
  const uint2* nhdr;
  uint4* mhdr;
  uint32_t* mrow;
  uint32_t* nrow;
  uint32_t* masks;
  uint32_t* cmap;
  uint32_t* cols;        // record columns (trace_cols.cuh), null when the phase pass replays
  // nsnap slots of 2 n wn words: the stabilizer halves of x (n rows of wn
  // words), then of z, at a run of deterministic measurements; their headers
  // carry flag 4 and the slot until the header pass adds the cross term
  uint32_t* snap;
  int nsnap;
  long long coin_begin;  // first coin-pass item of this program
  int nsteps;
  int nwins;
  int nm;      // measurements (M and RESET)
  int nn1;     // N1 ordinals
  int nchunk;  // 32-ordinal chunks of fire masks (those before the last measurement)
  int tw;      // words per trace row
  int wn;      // words per generator half
  int spl;     // shots per lane of the phase pass (item_begin counts groups of 32 spl)
  int nw;      // words per record column (a power of two >= 2)
  int nused;   // N1 ordinals before the last measurement
};

__host__ __device__ inline size_t round_up(size_t b, size_t a) { return (b + a - 1) / a * a; }

// Byte offsets of the trace arrays inside one program's trace (each array
// 256-byte aligned); o[3] is the total.
__host__ __device__ inline void trace_offsets(int nm, int nn1, int tw, size_t o[4]) {
  o[0] = 0;                                                  // mhdr
  o[1] = o[0] + round_up((size_t)nm * 16, 256);              // mrow
  o[2] = o[1] + round_up((size_t)nm * 8 * tw, 256);          // nrow
  o[3] = o[2] + round_up((size_t)nn1 * 8 * tw, 256);
}

__host__ __device__ inline size_t trace_bytes(int nm, int nn1, int tw) {
  size_t o[4];
  trace_offsets(nm, nn1, tw, o);
  return o[3];
}

// Chunks of 32 N1 ordinals of one shot's fire mask.
constexpr int kCoinChunk = 32;
// Chunks one coin-pass thread fills (one byte of the chunk map).
constexpr int kCoinChunksPerItem = 8;

// Bytes of the fire masks and of the chunk map of one program (each
// 256-byte aligned).
__host__ __device__ inline size_t coin_mask_bytes(long long nchunk, long long nshots) {
  return round_up((size_t)nchunk * (size_t)nshots * 8, 256);
}
__host__ __device__ inline size_t coin_map_bytes(long long nchunk, long long nshots) {
  return round_up((size_t)((nchunk + 31) / 32) * (size_t)nshots * 4, 256);
}

// Trace of one odd-d program (layout in trace_u8.cuh); N1 coins are drawn in
// its phase pass.
// Instructions the odd-d x / z passes stage in shared memory at a time.
constexpr int kOpWindow = 512;

// Gates in one OP_GROUP of a layered odd-d stream (abi.cu: append_layers_u8).
constexpr int kGateGroup = 8;

struct TraceDescU8 {
  CircuitDesc c;  // item_begin counts 32-shot groups of the phase pass
  uint4* mhdr;
  uint8_t* mrow;
  uint8_t* nrow;
  uint2* nhdr;  // N1 ordinal j: (coin threshold, opcode), 0xffffffff for probability 0
  int nm, nn1;
  int sw;         // bytes per trace row
  uint8_t* dsum;  // cluster x / z pass: per measurement its deterministic slice sums (cluster_det_bytes)
  const uint2* lay;  // the cluster x / z pass's layered instruction stream (OP_GROUP), or null: c.ops
  int nlay;
};

__host__ __device__ inline int trace_row_bytes_u8(int n) { return (int)round_up((size_t)2 * n, 16); }

__host__ __device__ inline void trace_offsets_u8(int nm, int nn1, int sw, size_t o[5]) {
  o[0] = 0;                                                // mhdr
  o[1] = o[0] + round_up((size_t)nm * 16, 256);            // mrow
  o[2] = o[1] + round_up((size_t)nm * 2 * sw, 256);        // nrow
  o[3] = o[2] + round_up((size_t)nn1 * 2 * sw, 256);       // nhdr
  o[4] = o[3] + round_up((size_t)nn1 * 8, 256);
}

// Widest trace row the phase pass has an instance for (n <= 2048).  Rows of
// up to 32 words (n <= 512) keep two shots per lane from kPhasePairMinShots
// shots on; wider rows keep one.
constexpr int kTraceMaxWords = 128;
constexpr int kPhasePairMaxWords = 32;

// Words per trace row for n qudits, 0 when n is too large for the phase pass.
__host__ __device__ inline int trace_words(int n) {
  const int w2 = 2 * ((n + 31) >> 5);
  int tw = 2;
  while (tw < w2) tw <<= 1;
  return tw <= kTraceMaxWords ? tw : 0;
}

// Threads of the x / z pass (one CTA per program): 256 or 512.
constexpr int kTracePassThreads = 512;

// Threads of a phase-pass block (one warp: one 32-shot group).
constexpr int kPhaseThreads = 32;

// Schedule window the x / z pass stages in shared memory: steps and ops.
constexpr int kTraceWinSteps = 512;
constexpr int kTraceWinOps = 2048;
inline size_t trace_pass_window_bytes() { return (size_t)16 * (kTraceWinSteps + kTraceWinOps); }


// Shared-memory bytes of one x / z pass CTA (hot part, x / z part).
size_t trace_pass_hot_bytes(int n);
size_t trace_pass_xz_bytes(int n);
cudaError_t trace_set_smem(int optin);

// x / z pass: one CTA of `threads` (256 or 512) per program, x / z in
// shared memory when xz_in_smem, else at gxz + blockIdx.x * xz_bytes.
void launch_trace_pass(int threads, int grid, size_t smem, cudaStream_t s, const TraceDesc* descs, int ndesc,
                       uint8_t* gxz, size_t xz_bytes, size_t hot_bytes, int xz_in_smem, int* status);

// Philox4x32-10 throughput probe: grid blocks of 256 threads, each drawing
// iters x 8 blocks keyed by seeds[thread % 256]; results folded into sink[256].
void launch_philox_probe(int grid, cudaStream_t s, const unsigned long long* seeds, int iters, uint4* sink);

// Coin pass: the fire masks of every program of descs with masks (items:
// (chunk group, shot) pairs numbered through coin_begin).
void launch_coin_pass(int grid, int block, size_t smem, cudaStream_t s, const TraceDesc* descs, int ndesc,
                      long long total);

// Dynamic shared memory every coin-pass block requests (and leaves unused):
// with a few x / z CTAs running alongside, those claim the rest of their SM's
// shared memory so that no coin block lands beside them.
constexpr size_t kCoinFenceSmem = 8192;

// Phase pass: spl (1 or 2) shots per lane, one warp per group of 32 spl
// shots (item_begin counts those groups); every program of descs has trace
// rows of tw words.  Returns false for an unsupported tw.
bool launch_phase_pass(int tw, int spl, int grid, int block, cudaStream_t s, const TraceDesc* descs, int ndesc,
                       long long total_groups, int* status);

// From this many shots in one phase-pass launch, lanes carry two shots each:
// with 152 SMs that still leaves 8 single-warp blocks per SM.
constexpr long long kPhasePairMinShots = 152LL * 64 * 8;

// Record columns (trace_cols.cuh): one program per run, trace rows of up to
// kColumnMaxWords words (n <= 512) and up to 32 x kColumnMaxRecordWords
// measurements; column_count(nm, nused) columns of nw words each.
constexpr int kColumnMaxWords = 32;
constexpr int kColumnMaxRecordWords = 32;
__host__ __device__ inline long long column_count(int nm, int nused) { return 1LL + nm + 2LL * nused; }
// Words per record column for nm measurements: a power of two >= 2.
inline int column_words(int nm) {
  int w = 2;
  while (32 * w < nm) w <<= 1;
  return w;
}
// Header pass: one warp per measurement of descs[0]; completes the headers
// of deterministic measurements whose cross terms were left to it.
void launch_header_pass(int grid, cudaStream_t s, const TraceDesc* descs, const int* status);
// Device memory the deterministic snapshots of one program may take.
constexpr size_t kSnapBudget = (size_t)64 << 20;

// Fewest shots for which a run takes the record columns by default (one
// 32-shot group per SM and scheduler); SDIM_FLAG_COLUMNS takes them at any
// shot count.
constexpr long long kColumnMinShots = 152LL * 32 * 4;
// Warps of a column-pass block (32 columns each).
constexpr int kColumnWarps = 4;
// Column pass: one block per 32 kColumnWarps columns of descs[0].
bool launch_column_pass(int tw, int grid, cudaStream_t s, const TraceDesc* descs, const int* status);
// Record pass: one single-warp block per 32-shot group of descs[0], groups
// g0 .. g0 + groups.
bool launch_record_pass(int nw, long long g0, int grid, cudaStream_t s, const TraceDesc* descs, long long groups,
                        const int* status);


// Odd-d trace engine (k_trace_u8.cu).  variant: 0, 1, 2 for d = 3, 5, 7, 3
// for any other odd prime.
int trace_u8_variant(int d);
cudaError_t trace_u8_set_smem(int optin);
size_t trace_u8_hot_bytes(int n);
size_t trace_u8_xz_bytes(int n);
size_t trace_u8_phase_smem(int n);
// x / z pass on single CTAs; queue (may be null): a zeroed counter from which
// the CTAs take programs dynamically (the x / z regions in global memory at
// gxz + blockIdx.x * xzb).
void launch_trace_u8_xz(int variant, int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd,
                        uint8_t* gxz, size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status);
// x / z pass on CTA pairs (trace_split_u8.cuh): `pairs` clusters of two,
// the instruction window at trace_u8_split_smem(nmax),
// smem = that + trace_u8_window_bytes().
size_t trace_u8_split_smem(int n);
// Shared memory of the instruction window both odd-d x / z passes keep after
// their tableau.
size_t trace_u8_window_bytes();
void launch_trace_u8_split(int variant, int pairs, size_t smem, size_t scratch_off, cudaStream_t s,
                           const TraceDescU8* d, int nd, int* status);
// x / z pass on clusters of kTraceClusterCtas CTAs (trace_cluster_u8.cuh).
// Each CTA holds trace_u8_cluster_xz(n) bytes of columns: in its shared
// memory after trace_u8_cluster_hot(nmax) bytes (in_smem), else at gxz +
// blockIdx.x * xzb; the instruction window follows in shared memory.
constexpr int kTraceClusterCtas = 8;
size_t trace_u8_cluster_hot(int n);
size_t trace_u8_cluster_xz(int n);
void launch_trace_u8_cluster(int variant, int clusters, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd,
                             uint8_t* gxz, size_t xzb, size_t hot, int in_smem, int* status);
// Each program's deterministic slice sums: trace_u8_cluster_det(n) bytes per
// measurement at TraceDescU8::dsum.  After the cluster x / z pass of programs
// d[0, nd), with at most maxnm measurements each, the deterministic-header
// pass writes their deterministic outcomes' common phases.
size_t trace_u8_cluster_det(int n);
void launch_cluster_det_headers(int maxnm, cudaStream_t s, const TraceDescU8* d, int nd, int* status);
void launch_trace_u8_phase(int variant, int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d,
                           int nd, long long total, int* status);

// x / z pass for d = 3 on bit planes (k_trace_p3.cu): one CTA of block (64
// to 512, or 1024) threads per program, x / z in shared memory after the hot part when
// in_smem, else at gxz + blockIdx.x * xzb with programs taken from queue;
// the instruction window (trace_u8_window_bytes) follows in shared memory.
// Writes the same trace as the byte-residue passes.
size_t trace_p3_hot_bytes(int n, int threads);
size_t trace_p3_xz_bytes(int n);
cudaError_t trace_p3_set_smem(int optin);
void launch_trace_p3(int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* d, int nd, uint8_t* gxz,
                     size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status);

// x / z pass for d = 5 and 7 on 4-bit residue lanes (k_trace_n4.cu), in the
// same form as the d = 3 bit-plane pass.
size_t trace_n4_hot_bytes(int n, int d, int threads);
size_t trace_n4_xz_bytes(int n);
cudaError_t trace_n4_set_smem(int optin);
void launch_trace_n4(int d, int grid, int block, size_t smem, cudaStream_t s, const TraceDescU8* dsc, int nd,
                     uint8_t* gxz, size_t xzb, size_t hot, int in_smem, unsigned* queue, int* status);

}  // namespace sdim
