// C ABI of the GB300 tableau engine: context, program encoder, launch
// planner and the plain / persistent / snapshot launches.  The kernels live
// in k_pershot.cu and k_group.cu behind the launch table of variants.cuh.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <climits>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/sdim_gb300.h"
#include "frame.cuh"
#include "kernels.cuh"
#include "trace.cuh"
#include "variants.cuh"

using namespace sdim;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

}  // namespace

// Descriptor staging of a run captured into a CUDA graph (sdim_graph_create).
// In the uncaptured first run (sizing) the descriptor uploads only add up
// their bytes.  In the captured run each descriptor array is copied into
// pinned host memory that the graph's copy node reads at every replay, and
// the byte offsets of every descriptor's seed and shot0 are noted with the
// batch index of its job, for sdim_graph_launch to rewrite.
struct GraphCapture {
  bool sizing = true;
  size_t need = 0;
  uint8_t* host = nullptr;
  size_t cap = 0, used = 0;
  std::vector<std::pair<size_t, int>> seed_at, shot0_at;  // (offset in host, job index)
};

struct sdim_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t last_stream = nullptr;  // stream of the last launch (sdim_sync / sdim_query)
  int num_sms = 0;
  int smem_optin = 0;
  int smem_per_sm = 0;    // shared memory of one SM
  int smem_reserved = 0;  // shared memory the system keeps per block
  int64_t l2_bytes = 0;
  int64_t gmem_bytes = 0;
  size_t gmem_slot_budget = (size_t)8 << 30;
  std::string err;
  DevBuf descs, counters, status, gslots, out, snap, arena, tdescs, trace, masks, tdescs_u8, trace_u8, xz_u8;
  DevBuf gslots_xz;  // d = 2 x / z pass tableaux in global memory (gslots: the shot-group engines')
  DevBuf cols;       // record columns of a d = 2 trace program (trace_cols.cuh)
  DevBuf dsnap;      // its x / z pass's deterministic snapshots (TraceDesc::snap)
  DevBuf cdet;       // deterministic slice sums of the odd-d cluster x / z passes (TraceDescU8::dsum)
  cudaStream_t aux = nullptr;                      // coin pass, concurrent with the x / z pass
  cudaStream_t grp = nullptr;                      // shot-group engines of a batch with trace programs
  // sdim_run's device-to-host copy of the records, when the record pass can
  // feed it in chunks (launch_trace_jobs copies each chunk as it is written)
  static constexpr int kD2HChunks = 4;
  cudaStream_t cps = nullptr;
  cudaEvent_t ev_rec[kD2HChunks] = {};
  cudaEvent_t ev_cps = nullptr;
  uint8_t* d2h_dst = nullptr;        // host records of the pending sdim_run
  const uint8_t* d2h_src = nullptr;  // their device buffer
  bool d2h_done = false;             // the copies are enqueued on cps
  cudaEvent_t ev_gf = nullptr, ev_gj = nullptr;    // fork to and join from grp
  cudaEvent_t ev_g0 = nullptr, ev_g1 = nullptr;    // shot-group engines' span on grp (SDIM_FLAG_TIME)
  static constexpr int kXzStreams = 3;
  cudaStream_t xzs[kXzStreams] = {};               // odd-d x / z passes of different runs, concurrently
  cudaEvent_t ev_xzf = nullptr, ev_xzj[kXzStreams] = {};
  DevBuf xz_queue;                                 // program counters of the dynamic x / z passes
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void* staging = nullptr;  // pinned host staging of sdim_run_tables
  size_t staging_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_xz = nullptr, ev_phase = nullptr;  // trace engine stage ends (SDIM_FLAG_TIME)
  cudaEvent_t ev_xzo = nullptr;                      // end of the x / z passes alone
  cudaEvent_t ev_c0 = nullptr, ev_c1 = nullptr;      // coin pass start and end (on aux)
  bool timing_pending = false;
  bool stages_recorded = false;  // ev_xz / ev_phase belong to the pending span
  bool coin_recorded = false;    // ev_c0 / ev_c1 belong to the pending span
  bool group_recorded = false;   // ev_g0 / ev_g1 belong to the pending span
  double group_ms = 0.0;         // shot-group engines on their own stream
  double last_ms = 0.0;
  double stage_ms[3] = {0.0, 0.0, 0.0};  // x / z passes, phase passes, other engines
  double pass_ms[2] = {0.0, 0.0};        // x / z passes alone, coin pass alone
  int smem_attr_set[V_COUNT] = {};
  bool trace_smem_set = false;
  bool frame_smem_set = false;
  int trace_threads = kTracePassThreads;  // x / z pass CTA size (SDIM_TRACE_PASS_THREADS: 256 or 512)
  GraphCapture* capture = nullptr;  // set while sdim_graph_create runs on its private context
  sdim_circuit* xz_pending = nullptr;  // circuit whose kept trace the current call writes (SDIM_FLAG_REUSE_XZ)
  bool pend_trace = false, pend_cols = false;  // what of it the call writes: the trace, the columns
  cudaEvent_t ev_cols = nullptr;               // end of the column pass (SDIM_FLAG_TIME)
  bool cols_recorded = false;
  double col_ms = 0.0;                         // column pass alone
  unsigned long long reallocs = 0;  // device buffers moved by ensure()
};

// A batch run captured into a CUDA graph.  It owns a private context, so the
// device buffers its nodes point into move only when the graph is destroyed.
struct sdim_graph {
  sdim_ctx* own = nullptr;
  GraphCapture cap;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;  // end of the last replay
  bool launched = false;
  int njobs = 0;
};

// Where the trace schedule of a program sits in its blob (uint2 words).
struct TraceSchedule {
  int64_t steps_off = -1, lops_off = -1, wins_off = -1, nthr_off = -1, nhdr_off = -1;
  int nsteps = 0, nwins = 0;
  int nn1_used = 0;  // N1 ordinals before the last measurement (the only ones a record can see)
};

struct sdim_circuit {
  int device = 0;
  int n = 0, d = 0, nmeas = 0;
  int nn1 = 0;        // N1 instructions (noise ordinals)
  int64_t nops_user = 0;
  int nops = 0;
  int variant = 0;    // per-shot engine (plain form, per-shot snapshots)
  int gvariant = 0;   // shot-group engine for batched runs
  int gblock = 32;    // threads of one group team
  uint2* h_ops = nullptr;  // pinned host copy of the blob: instruction words, then the trace schedule
  uint2* d_ops = nullptr;  // device copy of the same blob
  int64_t blob_words = 0;  // uint2 words of the blob
  const uint4* d_steps = nullptr;  // trace schedule (d = 2, n <= 2048), inside the blob
  const uint4* d_lops = nullptr;
  const uint4* d_wins = nullptr;
  const uint32_t* d_nthr = nullptr;  // N1 coin thresholds, padded to a multiple of 64 with 0xffffffff
  const uint2* d_nhdr = nullptr;     // N1 (threshold, opcode)
  int nsteps = 0, nwins = 0, nn1_used = 0;
  int64_t fops_off = 0;  // frame instruction stream (frame.cuh), inside the blob
  int nfops = 0;
  const uint2* d_lay = nullptr;  // odd d: the layered x / z stream (append_layers_u8), inside the blob
  int nlay = 0;
  // d = 2 x / z trace kept on the device for SDIM_FLAG_REUSE_XZ: written by a
  // run with the flag, valid once that synchronous run has ended without a
  // device error, then read by the later runs with the flag instead of
  // running the x / z pass again (it depends only on the program)
  DevBuf xz_trace;
  bool xz_trace_valid = false;
  DevBuf xz_cols;  // its record columns (trace_cols.cuh), kept the same way
  bool xz_cols_valid = false;
};

namespace {

int fail(sdim_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_fail(sdim_ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(ctx, SDIM_ECUDA, m);
}

#define CK(call)                                             \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

int ensure(sdim_ctx* ctx, DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return SDIM_OK;
  // grow geometrically: a reallocation (cudaFree) waits for the device
  size_t cap = std::max(std::max(bytes, (size_t)256), b.cap + b.cap / 2);
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  ++ctx->reallocs;
  cudaError_t e = cudaMalloc(&b.p, cap);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, SDIM_ENOMEM, std::string("device allocation of ") + std::to_string(cap) +
                                      " bytes failed: " + cudaGetErrorString(e));
  }
  b.cap = cap;
  return SDIM_OK;
}

bool is_prime(int d) {
  if (d < 2) return false;
  for (int k = 2; k * k <= d; ++k)
    if (d % k == 0) return false;
  return true;
}

int variant_for(int d) {
  switch (d) {
    case 2: return V_BITS;
    case 3: return V_U8_3;
    case 5: return V_U8_5;
    case 7: return V_U8_7;
    default: return V_U8_GEN;
  }
}

// Programs with at least this many qudits run one group per CTA: their
// measurements touch n x 2n residues, which one warp would walk alone.
constexpr int kCtaTeamQudits = 160;

int group_variant_for(int d, int n, unsigned flags) {
  bool cta = n >= kCtaTeamQudits;
  if (flags & SDIM_FLAG_TEAM_WARP) cta = false;
  if (flags & SDIM_FLAG_TEAM_CTA) cta = true;
  switch (d) {
    case 2: return cta ? V_GBITS_C : V_GBITS_W;
    case 3: return cta ? V_GU8_3_C : V_GU8_3_W;
    case 5: return cta ? V_GU8_5_C : V_GU8_5_W;
    case 7: return cta ? V_GU8_7_C : V_GU8_7_W;
    default: return cta ? V_GU8_GEN_C : V_GU8_GEN_W;
  }
}

// threads of a CTA team: a power of two near n, 64 to 512
int cta_block_for(int n) {
  int b = 64;
  while (b < n && b < 512) b <<= 1;
  return b;
}

// shared memory a block may use for slots
size_t smem_usable(const sdim_ctx* ctx) { return (size_t)(ctx->smem_optin - kStaticSmemReserve); }

int set_smem_attr(sdim_ctx* ctx, int variant) {
  if (ctx->smem_attr_set[variant]) return SDIM_OK;
  const cudaError_t e = variant_ops(variant).set_smem(ctx->smem_optin);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaFuncSetAttribute");
  ctx->smem_attr_set[variant] = 1;
  return SDIM_OK;
}

// Where the slots of one launch live and how many there are.
struct Plan {
  bool in_smem;         // big part of each slot in shared memory
  int team_threads;     // 32 for warp teams
  int slots_per_block;
  int blocks;
  size_t hot, big;      // bytes of the two parts of a slot
  size_t smem_per_block;
};

Plan plan_launch(const sdim_ctx* ctx, int variant, size_t hot, size_t big, long long items, int cta_block,
                 bool force_gmem) {
  const VariantOps& ops = variant_ops(variant);
  const size_t usable = smem_usable(ctx);
  Plan p;
  p.hot = hot;
  p.big = big;
  p.in_smem = !force_gmem && hot + big <= usable;
  p.team_threads = ops.cta ? cta_block : 32;
  const size_t per_slot_smem = hot + (p.in_smem ? big : 0);
  if (ops.cta) {
    p.slots_per_block = 1;
  } else {
    const int max_slots = ops.max_block / 32;
    p.slots_per_block = per_slot_smem ? (int)std::min<size_t>(max_slots, usable / per_slot_smem) : 8;
    if (p.slots_per_block < 1) p.slots_per_block = 1;
    if (!p.in_smem && !ops.group) p.slots_per_block = 4;  // per-shot tableaux in global memory
    // spread the items over every SM before stacking more warps on one
    const long long per_sm = (items + ctx->num_sms - 1) / ctx->num_sms;
    if (per_sm < p.slots_per_block) p.slots_per_block = (int)std::max<long long>(1, per_sm);
  }
  const int block = p.team_threads * p.slots_per_block;
  p.smem_per_block = per_slot_smem * p.slots_per_block;
  const int occ = ops.occupancy(block, p.smem_per_block);
  long long blocks = (long long)ctx->num_sms * occ;
  const long long need = (items + p.slots_per_block - 1) / p.slots_per_block;
  blocks = std::min(blocks, need);
  if (!p.in_smem) {
    const long long by_budget = (long long)(ctx->gmem_slot_budget / (big * p.slots_per_block));
    blocks = std::min(blocks, std::max<long long>(1, by_budget));
  }
  p.blocks = (int)std::max<long long>(1, blocks);
  return p;
}

int read_status(sdim_ctx* ctx) {
  int st = 0;
  CK(cudaMemcpy(&st, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (st == DEV_OK) return SDIM_OK;
  const char* why = st == DEV_BAD_OPCODE ? "bad opcode" : st == DEV_BAD_QUDIT ? "qudit index out of range"
                                                                                 : "slot too small";
  return fail(ctx, SDIM_EDEVICE, std::string("device reported: ") + why);
}

// Kernel times of the last SDIM_FLAG_TIME call: the whole span and its stages.
int collect_times(sdim_ctx* ctx) {
  float all = 0.f, a = 0.f, b = 0.f, c = 0.f, xo = 0.f, co = 0.f;
  CK(cudaEventElapsedTime(&all, ctx->ev0, ctx->ev1));
  if (ctx->stages_recorded) {
    CK(cudaEventElapsedTime(&a, ctx->ev0, ctx->ev_xz));
    CK(cudaEventElapsedTime(&b, ctx->ev_xz, ctx->ev_phase));
    CK(cudaEventElapsedTime(&c, ctx->ev_phase, ctx->ev1));
    CK(cudaEventElapsedTime(&xo, ctx->ev0, ctx->ev_xzo));
  } else {
    c = all;
  }
  if (ctx->coin_recorded) CK(cudaEventElapsedTime(&co, ctx->ev_c0, ctx->ev_c1));
  if (ctx->group_recorded) CK(cudaEventElapsedTime(&c, ctx->ev_g0, ctx->ev_g1));  // on their own stream
  float cm = 0.f;
  if (ctx->cols_recorded) CK(cudaEventElapsedTime(&cm, ctx->ev_xzo, ctx->ev_cols));
  ctx->col_ms = cm;
  ctx->group_ms = ctx->group_recorded ? c : 0.0;
  ctx->cols_recorded = false;
  ctx->pass_ms[0] = xo;
  ctx->pass_ms[1] = co;
  ctx->stages_recorded = false;
  ctx->coin_recorded = false;
  ctx->group_recorded = false;
  ctx->last_ms = all;
  ctx->stage_ms[0] = a;
  ctx->stage_ms[1] = b;
  ctx->stage_ms[2] = c;
  ctx->timing_pending = false;
  return SDIM_OK;
}

// The end of a synchronous call: a kept x / z trace that it wrote
// (SDIM_FLAG_REUSE_XZ) becomes valid when the call ended without an error.
int settle_xz(sdim_ctx* ctx, int rc) {
  if (ctx->xz_pending && rc == SDIM_OK) {
    if (ctx->pend_trace) ctx->xz_pending->xz_trace_valid = true;
    if (ctx->pend_cols) ctx->xz_pending->xz_cols_valid = true;
  }
  ctx->xz_pending = nullptr;
  ctx->pend_trace = ctx->pend_cols = false;
  return rc;
}

int finish(sdim_ctx* ctx, cudaStream_t s, unsigned flags) {
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->timing_pending = true;
  }
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return cuda_fail(ctx, le, "kernel launch");
  if (flags & SDIM_FLAG_ASYNC) {
    ctx->xz_pending = nullptr;  // not checked, so a trace written now is not kept valid
    ctx->pend_trace = ctx->pend_cols = false;
    return SDIM_OK;
  }
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    const int trc = collect_times(ctx);
    if (trc != SDIM_OK) return trc;
  }
  return settle_xz(ctx, read_status(ctx));
}

// With SDIM_FLAG_DIRECT_HOST: the device address through which the kernels
// can write the host buffer p directly (page-locked memory: cudaHostAlloc,
// cudaMallocHost, cudaHostRegister), or null for pageable memory.  Records
// written this way reach the host with the kernels' own stores, so no
// device-to-host copy follows.  Without the flag (null) they are staged in
// device memory and copied down, which measured faster for the d = 2 trace
// engine's record runs (0.56 against 1.16 ms for 38.5 MB of records).
uint8_t* mapped_host(void* p, unsigned flags) {
  if (!p || !(flags & SDIM_FLAG_DIRECT_HOST)) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost && a.devicePointer ? static_cast<uint8_t*>(a.devicePointer) : nullptr;
}

struct Job {
  const sdim_circuit* c;
  uint64_t seed;
  int64_t shot0, nshots;
  uint8_t* out_dev;
  int index = -1;  // position in the caller's batch (graph capture: whose seed a descriptor holds)
};

// Host -> device copy of `count` descriptors of `each` bytes, each holding a
// CircuitDesc at byte `cdesc_off`; job_index(k) is the batch index of
// descriptor k.  Outside a graph capture this is one cudaMemcpyAsync.
template <class JobIndex>
int upload_descs(sdim_ctx* ctx, void* dst, const void* src, size_t each, size_t count, size_t cdesc_off,
                 JobIndex job_index, cudaStream_t s) {
  const size_t bytes = each * count;
  GraphCapture* g = ctx->capture;
  if (g && !g->sizing) {
    if (g->used + bytes > g->cap) return fail(ctx, SDIM_ECUDA, "graph descriptor staging overflow");
    const size_t off = g->used;
    std::memcpy(g->host + off, src, bytes);
    g->used += (bytes + 255) & ~(size_t)255;
    for (size_t k = 0; k < count; ++k) {
      const size_t base = off + k * each + cdesc_off;
      g->seed_at.emplace_back(base + offsetof(CircuitDesc, seed), job_index(k));
      g->shot0_at.emplace_back(base + offsetof(CircuitDesc, shot0), job_index(k));
    }
    CK(cudaMemcpyAsync(dst, g->host + off, bytes, cudaMemcpyHostToDevice, s));
    return SDIM_OK;
  }
  if (g) g->need += (bytes + 255) & ~(size_t)255;
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  return SDIM_OK;
}

// Engine used for a job: the shot-group engine for batched runs (unless
// SDIM_FLAG_PER_SHOT; SDIM_FLAG_TEAM_* override the team kind), the
// per-shot engine for the plain form.
int job_variant(const sdim_circuit* c, unsigned flags) {
  if (flags & (SDIM_FLAG_PLAIN | SDIM_FLAG_PER_SHOT)) return c->variant;
  if (flags & (SDIM_FLAG_TEAM_WARP | SDIM_FLAG_TEAM_CTA)) return group_variant_for(c->d, c->n, flags);
  return c->gvariant;
}

// Below this many shots a program runs on the shot-group engine: one x / z
// pass per program plus a phase pass only pays once there are several 32-shot
// groups to share it, and in a batch of small programs the group engine's
// single persistent launch keeps every SM busy.
constexpr int64_t kTraceMinShots = 128;

// From this many qudits the trace engines take a program at any shot count:
// its x / z pass dominates, and the shot-group engine repeats it for every
// 32 shots where the trace engine runs it once.
constexpr int kTraceMinQudits = 160;

// Jobs for the trace engine: d = 2, batched form, trace rows of at most
// kTraceMaxWords words (n <= 2048) and kTraceMinShots shots or
// kTraceMinQudits qudits, unless SDIM_FLAG_TRACE (any shot count) or a flag
// that names another engine.
bool use_trace(const Job& j, unsigned flags) {
  if (flags & (SDIM_FLAG_PLAIN | SDIM_FLAG_PER_SHOT | SDIM_FLAG_TEAM_WARP | SDIM_FLAG_TEAM_CTA |
               SDIM_FLAG_NO_TRACE))
    return false;
  if (j.c->d != 2 || trace_words(j.c->n) == 0 || !j.c->d_steps || j.nshots <= 0) return false;
  return (flags & SDIM_FLAG_TRACE) || j.nshots >= kTraceMinShots || j.c->n >= kTraceMinQudits;
}

// Odd-d programs above this many qudits stay on the shot-group engine (the
// phase pass keeps 32 shots' deltas in shared memory).
constexpr int kTraceU8MaxQudits = 2048;

// Jobs for the odd-d trace engine: same rule with d odd.
// The odd-d x / z pass form of a program of n qudits in a run with
// `programs` odd-d trace programs: 0, one CTA with the tableau in shared
// memory when it fits.  Otherwise, in a batch with programs enough to fill
// the SMs (num_sms / 2 or more), for throughput: 1, a CTA pair splitting the
// generator columns (trace_split_u8.cuh) when that fits, else 2, one CTA
// with the tableau in global memory.  In a smaller batch, for latency: a
// cluster of kTraceClusterCtas CTAs (trace_cluster_u8.cuh) with its columns
// in shared memory (3) or global memory (4).  For d = 3 (unless
// SDIM_FLAG_U8_XZ, SDIM_FLAG_SPLIT_XZ or SDIM_FLAG_CLUSTER_XZ names a byte
// form) in a batch of num_sms / 2 or more odd-d trace programs (or with
// SDIM_FLAG_PACKED_XZ) one CTA on the bit-plane tableau (trace_p3.cuh), in
// shared memory (5) up to n = 448 on GB300, else in a global-memory slot (6).
// For d = 5 and 7 likewise on the 4-bit-lane tableau (trace_n4.cuh): shared
// memory (7) up to n = 320, else a global-memory slot (8).  A cluster shares each
// measurement's fixed cost (a cluster barrier, pivot search, candidate
// broadcast) among 8 SMs, so it finishes one program sooner but a full batch
// later.
// Threads of a packed odd-d x / z pass CTA for programs of up to n qudits:
// about one per qudit (64 to 512) in a batch, where more warps would only
// spend issue slots walking the instruction stream; 1024 for a few programs
// of 128+ qudits, whose rank-1 updates then spread over more row groups.
int packed_threads(int n, bool few) {
  if (few && n >= 128) return 1024;
  return std::max(64, std::min(kTracePassThreads, (n + 31) & ~31));
}

int odd_xz_mode(int n, int d, long long programs, unsigned flags, size_t optin, int num_sms) {
  const size_t win = trace_u8_window_bytes();
  const bool force_gmem = flags & SDIM_FLAG_FORCE_GMEM;
  const bool few = programs * 2 < (long long)num_sms;
  const bool single = trace_u8_hot_bytes(n) + trace_u8_xz_bytes(n) + win + 4096 <= optin;
  // packed tableaux for batches (throughput: a quarter or half of the bytes);
  // for a few programs (latency) only where the byte tableau would sit in one
  // CTA and n >= 128.  On GB300, lone programs: d = 5, n = 180 1.27 ms packed
  // against 1.46 on one byte CTA, d = 3, n = 200 1.32 against 1.66; but
  // d = 5, n = 256 4.32 against 3.16 on the byte cluster (2.17 once it took
  // one cluster barrier a measurement), d = 7, n = 600 11.5 against 5.6 on
  // the streamed cluster, PR1 (n = 32) 0.31 against 0.26 (0.24 since)
  const bool packed = (d == 3 || d == 5 || d == 7) &&
                      !(flags & (SDIM_FLAG_U8_XZ | SDIM_FLAG_SPLIT_XZ | SDIM_FLAG_CLUSTER_XZ)) &&
                      (!few || (flags & SDIM_FLAG_PACKED_XZ) || (single && n >= 128));
  const int th = packed_threads(n, few);
  if (packed && d == 3)
    return !force_gmem && trace_p3_hot_bytes(n, th) + trace_p3_xz_bytes(n) + win + 4096 <= optin ? 5 : 6;
  if (packed)
    return !force_gmem && trace_n4_hot_bytes(n, d, th) + trace_n4_xz_bytes(n) + win + 4096 <= optin ? 7 : 8;
  const bool pair = trace_u8_split_smem(n) + win + 4096 <= optin;
  const bool cl_smem = trace_u8_cluster_hot(n) + trace_u8_cluster_xz(n) + win + 4096 <= optin;
  if (flags & SDIM_FLAG_CLUSTER_XZ) return cl_smem && !force_gmem ? 3 : 4;
  if (force_gmem) return 2;
  if (pair && (flags & SDIM_FLAG_SPLIT_XZ)) return 1;
  if (single) return 0;
  if (few) return cl_smem ? 3 : 4;
  return pair ? 1 : 2;
}

bool use_trace_u8(const Job& j, unsigned flags) {
  if (flags & (SDIM_FLAG_PLAIN | SDIM_FLAG_PER_SHOT | SDIM_FLAG_TEAM_WARP | SDIM_FLAG_TEAM_CTA |
               SDIM_FLAG_NO_TRACE))
    return false;
  if (j.c->d == 2 || j.c->n > kTraceU8MaxQudits || j.nshots <= 0) return false;
  return (flags & SDIM_FLAG_TRACE) || j.nshots >= kTraceMinShots || j.c->n >= kTraceMinQudits;
}

// Trace-engine launches: the x / z pass of every program (d = 2 jobs, then
// odd-d jobs per variant of d), the coin pass of the d = 2 jobs alongside on
// the second stream, then the phase passes (d = 2 per trace-row width, odd
// d per variant).  d = 2 programs are ordered by n, largest first, which
// orders the row widths; odd-d programs by (variant, n), largest first.
int launch_trace_jobs(sdim_ctx* ctx, std::vector<Job> jobs, std::vector<Job> ujobs, cudaStream_t s, unsigned flags,
                      int* status) {
  const bool timed = flags & SDIM_FLAG_TIME;
  if (jobs.empty() && ujobs.empty()) {
    if (timed) {
      CK(cudaEventRecord(ctx->ev_xzo, s));
      CK(cudaEventRecord(ctx->ev_xz, s));
      CK(cudaEventRecord(ctx->ev_phase, s));
      ctx->stages_recorded = true;
    }
    return SDIM_OK;
  }
  const bool force_gmem = flags & SDIM_FLAG_FORCE_GMEM;
  int rc;
  if (!ctx->trace_smem_set) {
    cudaError_t e = trace_set_smem(ctx->smem_optin);
    if (e == cudaSuccess) e = trace_u8_set_smem(ctx->smem_optin);
    if (e == cudaSuccess) e = trace_p3_set_smem(ctx->smem_optin);
    if (e == cudaSuccess) e = trace_n4_set_smem(ctx->smem_optin);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaFuncSetAttribute");
    ctx->trace_smem_set = true;
  }
  // ---- d = 2 descriptors
  // largest first: the x / z passes of a batch start with the longest ones
  std::stable_sort(jobs.begin(), jobs.end(), [](const Job& a, const Job& b) { return a.c->n > b.c->n; });
  const size_t k = jobs.size();
  std::vector<TraceDesc> hd(k);
  long long coins = 0;
  TraceDesc* dd = nullptr;
  // SDIM_FLAG_REUSE_XZ, one d = 2 program: its trace lives in the circuit's
  // own buffer, and a valid one is replayed without the x / z pass
  sdim_circuit* keep = (flags & SDIM_FLAG_REUSE_XZ) && k == 1 && !ctx->capture
                           ? const_cast<sdim_circuit*>(jobs[0].c) : nullptr;
  const bool skip_xz = keep && keep->xz_trace_valid;
  if (keep && !skip_xz) {
    rc = ensure(ctx, keep->xz_trace, trace_bytes(keep->nmeas, keep->nn1, trace_words(keep->n)));
    if (rc != SDIM_OK) return rc;
    keep->xz_cols_valid = false;  // columns of the trace about to be rewritten
    ctx->xz_pending = keep;
    ctx->pend_trace = true;
  }
  // record columns instead of the phase replay (trace_cols.cuh): one program,
  // fires known from the coin pass, enough shots to pay for the column pass
  // (or SDIM_FLAG_COLUMNS); SDIM_FLAG_PHASE_REPLAY keeps the replay
  bool colform = false, skip_cols = false;
  int cnw = 0;
  long long ncols = 0;
  if (k == 1 && !(flags & SDIM_FLAG_PHASE_REPLAY)) {
    const sdim_circuit* c0 = jobs[0].c;
    ncols = column_count(c0->nmeas, c0->nn1_used);
    cnw = column_words(c0->nmeas);
    const bool masked = c0->nn1_used == 0 || !(flags & SDIM_FLAG_NO_COIN_PASS);
    const bool fits = trace_words(c0->n) <= kColumnMaxWords && c0->nmeas >= 1 && cnw <= kColumnMaxRecordWords;
    const bool pays = (flags & SDIM_FLAG_COLUMNS) || jobs[0].nshots >= std::max<long long>(ncols, kColumnMinShots);
    colform = fits && masked && pays;
  }
  if (k) {
    std::vector<size_t> off(k);
    size_t total = 0;
    for (size_t i = 0; i < k; ++i) {
      off[i] = total;
      total += trace_bytes(jobs[i].c->nmeas, jobs[i].c->nn1, trace_words(jobs[i].c->n));
    }
    if (!keep && (rc = ensure(ctx, ctx->trace, std::max<size_t>(total, 256))) != SDIM_OK) return rc;
    if ((rc = ensure(ctx, ctx->tdescs, sizeof(TraceDesc) * k)) != SDIM_OK) return rc;
    // fire masks: a word pair per 32 N1 ordinals per shot and the chunk map,
    // within a budget
    constexpr size_t kMaskBudget = (size_t)1 << 30;
    std::vector<size_t> moff(k, SIZE_MAX);
    size_t mtotal = 0;
    for (size_t i = 0; i < k; ++i) {
      const long long nchunk = ((long long)jobs[i].c->nn1_used + kCoinChunk - 1) / kCoinChunk;
      const size_t b = coin_mask_bytes(nchunk, jobs[i].nshots) + coin_map_bytes(nchunk, jobs[i].nshots);
      if (nchunk && mtotal + b <= kMaskBudget && !(flags & SDIM_FLAG_NO_COIN_PASS)) {
        moff[i] = mtotal;
        mtotal += b;
      }
    }
    if (mtotal && (rc = ensure(ctx, ctx->masks, mtotal)) != SDIM_OK) return rc;
    // shots per lane of each phase-pass launch (one per trace-row width)
    std::vector<int> spl(k, 1);
    for (size_t b = 0; b < k;) {
      const int tw = trace_words(jobs[b].c->n);
      size_t e = b;
      long long shots = 0;
      while (e < k && trace_words(jobs[e].c->n) == tw) shots += jobs[e++].nshots;
      // two shots per lane from kPhasePairMinShots (four measured slower on
      // the L = 7 surface step: 0.31 against 0.20 ms, the lanes' registers
      // leave five warps per SM); SDIM_FLAG_LANE_SHOTS_1 keeps one
      const int sp = shots >= kPhasePairMinShots && tw <= kPhasePairMaxWords && !(flags & SDIM_FLAG_LANE_SHOTS_1)
                         ? 2 : 1;
      for (size_t i = b; i < e; ++i) spl[i] = sp;
      b = e;
    }
    if (colform) spl[0] = 1;  // the record pass: one shot per lane
    long long groups = 0;
    for (size_t i = 0; i < k; ++i) {
      const Job& j = jobs[i];
      const int tw = trace_words(j.c->n);
      if (i > 0 && tw != trace_words(jobs[i - 1].c->n)) groups = 0;  // item numbers restart per phase launch
      TraceDesc& td = hd[i];
      std::memset(&td, 0, sizeof(td));
      td.c.ops = j.c->d_ops;
      td.c.out = j.out_dev;
      td.c.seed = j.seed;
      td.c.shot0 = j.shot0;
      td.c.item_begin = groups;
      td.c.nops = j.c->nops;
      td.c.n = j.c->n;
      td.c.d = j.c->d;
      td.c.nmeas = j.c->nmeas;
      td.c.nshots = (int)j.nshots;
      groups += (j.nshots + 32 * spl[i] - 1) / (32 * spl[i]);
      td.spl = spl[i];
      uint8_t* b = keep ? static_cast<uint8_t*>(keep->xz_trace.p) : static_cast<uint8_t*>(ctx->trace.p) + off[i];
      size_t o[4];
      trace_offsets(j.c->nmeas, j.c->nn1, tw, o);
      td.steps = j.c->d_steps;
      td.lops = j.c->d_lops;
      td.wins = j.c->d_wins;
      td.nthr = j.c->d_nthr;
      td.nhdr = j.c->d_nhdr;
      td.nsteps = j.c->nsteps;
      td.nwins = j.c->nwins;
      td.mhdr = reinterpret_cast<uint4*>(b + o[0]);
      td.mrow = reinterpret_cast<uint32_t*>(b + o[1]);
      td.nrow = reinterpret_cast<uint32_t*>(b + o[2]);
      td.coin_begin = coins;
      if (moff[i] != SIZE_MAX) {
        td.masks = reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(ctx->masks.p) + moff[i]);
        td.nchunk = (j.c->nn1_used + kCoinChunk - 1) / kCoinChunk;
        td.cmap = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(td.masks) +
                                              coin_mask_bytes(td.nchunk, j.nshots));
        coins += (long long)((td.nchunk + kCoinChunksPerItem - 1) / kCoinChunksPerItem) * j.nshots;
      }
      td.nm = j.c->nmeas;
      td.nn1 = j.c->nn1;
      td.tw = tw;
      td.wn = (j.c->n + 31) >> 5;
      td.nused = j.c->nn1_used;
    }
    if (k == 1 && !skip_xz && jobs[0].c->nmeas > 0) {
      // one program: the x / z pass leaves the deterministic cross terms to
      // the header pass, a snapshot per run of deterministic measurements
      const sdim_circuit* c0 = jobs[0].c;
      const size_t per = (size_t)8 * c0->n * ((c0->n + 31) >> 5);
      const long long ns = std::min<long long>(c0->nmeas, (long long)(kSnapBudget / per));
      if (ns > 0) {
        if ((rc = ensure(ctx, ctx->dsnap, (size_t)ns * per)) != SDIM_OK) return rc;
        hd[0].snap = static_cast<uint32_t*>(ctx->dsnap.p);
        hd[0].nsnap = (int)ns;
      }
    }
    if (colform) {
      // the fire masks must be there unless the program has no N1 before its
      // last measurement (a mask budget overflow falls back to the replay)
      if (hd[0].nused > 0 && !hd[0].masks) colform = false;
    }
    if (colform) {
      const size_t cbytes = std::max<size_t>((size_t)ncols * (size_t)cnw * 4, 256);
      DevBuf& cb = keep ? keep->xz_cols : ctx->cols;
      skip_cols = keep && skip_xz && keep->xz_cols_valid;
      if (!skip_cols) {
        if ((rc = ensure(ctx, cb, cbytes)) != SDIM_OK) return rc;
        if (keep) {
          ctx->xz_pending = keep;
          ctx->pend_cols = true;
        }
      }
      hd[0].cols = static_cast<uint32_t*>(cb.p);
      hd[0].nw = cnw;
    }
    dd = static_cast<TraceDesc*>(ctx->tdescs.p);
    if ((rc = upload_descs(ctx, dd, hd.data(), sizeof(TraceDesc), k, offsetof(TraceDesc, c),
                           [&](size_t i) { return jobs[i].index; }, s)) != SDIM_OK)
      return rc;
  }
  // ---- odd-d descriptors
  std::stable_sort(ujobs.begin(), ujobs.end(), [](const Job& a, const Job& b) {
    const int va = trace_u8_variant(a.c->d), vb = trace_u8_variant(b.c->d);
    return va != vb ? va < vb : a.c->n > b.c->n;
  });
  const size_t ku = ujobs.size();
  std::vector<TraceDescU8> hu(ku);
  TraceDescU8* du = nullptr;
  if (ku) {
    // per program its trace, and for a cluster x / z pass (odd_xz_mode 3, 4)
    // its deterministic slice sums
    std::vector<size_t> off(ku), doff(ku, SIZE_MAX);
    std::vector<int> xmode(ku);
    size_t total = 0, dtotal = 0;
    for (size_t i = 0; i < ku; ++i) {
      const Job& j = ujobs[i];
      size_t o[5];
      trace_offsets_u8(j.c->nmeas, j.c->nn1, trace_row_bytes_u8(j.c->n), o);
      off[i] = total;
      total += o[4];
      const int mode = odd_xz_mode(j.c->n, j.c->d, (long long)ku, flags, (size_t)ctx->smem_optin, ctx->num_sms);
      xmode[i] = mode;
      if (mode == 3 || mode == 4) {
        doff[i] = dtotal;
        dtotal += round_up((size_t)j.c->nmeas * trace_u8_cluster_det(j.c->n), 256);
      }
    }
    if ((rc = ensure(ctx, ctx->trace_u8, std::max<size_t>(total, 256))) != SDIM_OK) return rc;
    if (dtotal && (rc = ensure(ctx, ctx->cdet, dtotal)) != SDIM_OK) return rc;
    if ((rc = ensure(ctx, ctx->tdescs_u8, sizeof(TraceDescU8) * ku)) != SDIM_OK) return rc;
    long long groups = 0;
    for (size_t i = 0; i < ku; ++i) {
      const Job& j = ujobs[i];
      if (i > 0 && trace_u8_variant(j.c->d) != trace_u8_variant(ujobs[i - 1].c->d)) groups = 0;
      TraceDescU8& td = hu[i];
      std::memset(&td, 0, sizeof(td));
      td.c.ops = j.c->d_ops;
      td.c.out = j.out_dev;
      td.c.seed = j.seed;
      td.c.shot0 = j.shot0;
      td.c.item_begin = groups;
      td.c.nops = j.c->nops;
      td.c.n = j.c->n;
      td.c.d = j.c->d;
      td.c.nmeas = j.c->nmeas;
      td.c.nshots = (int)j.nshots;
      groups += (j.nshots + 31) / 32;
      td.sw = trace_row_bytes_u8(j.c->n);
      size_t o[5];
      trace_offsets_u8(j.c->nmeas, j.c->nn1, td.sw, o);
      uint8_t* b = static_cast<uint8_t*>(ctx->trace_u8.p) + off[i];
      td.mhdr = reinterpret_cast<uint4*>(b + o[0]);
      td.mrow = b + o[1];
      td.nrow = b + o[2];
      td.nhdr = reinterpret_cast<uint2*>(b + o[3]);
      td.nm = j.c->nmeas;
      td.nn1 = j.c->nn1;
      td.dsum = doff[i] == SIZE_MAX ? nullptr : static_cast<uint8_t*>(ctx->cdet.p) + doff[i];
      // the cluster walks the layered stream (gate groups); the other forms
      // the instructions as written.  On GB300: oddd5's cluster x / z pass
      // 2.17 ms layered against 2.21, PR1's single CTA 0.257 against 0.241
      const int xm = xmode[i];
      if ((xm == 3 || xm == 4) && j.c->d_lay && !(flags & SDIM_FLAG_UNLAYERED)) {
        td.lay = j.c->d_lay;
        td.nlay = j.c->nlay;
      }
    }
    du = static_cast<TraceDescU8*>(ctx->tdescs_u8.p);
    if ((rc = upload_descs(ctx, du, hu.data(), sizeof(TraceDescU8), ku, offsetof(TraceDescU8, c),
                           [&](size_t i) { return ujobs[i].index; }, s)) != SDIM_OK)
      return rc;
  }
  if (coins) CK(cudaEventRecord(ctx->ev_fork, s));
  // odd d: the x / z pass form of each program (odd_xz_mode)
  const size_t optin = (size_t)ctx->smem_optin;
  const size_t win = trace_u8_window_bytes();
  auto xz_mode = [&](int n, int d) { return odd_xz_mode(n, d, (long long)ku, flags, optin, ctx->num_sms); };
  // clusters of a mode-4 run: one per kTraceClusterCtas SMs, each CTA alone
  // on its SM, so the programs in flight keep their columns in L2
  auto stream_clusters = [&](size_t programs) {
    return std::min<size_t>(programs, (size_t)std::max(1, ctx->num_sms / kTraceClusterCtas));
  };
  // runs of programs with one (variant, mode); with several runs each goes
  // on its own stream so that one run's tail overlaps the next run
  struct Run { size_t b, e; int v, mode; size_t slot_off; };
  std::vector<Run> runs;
  size_t slot_total = 0;
  for (size_t b = 0; b < ku;) {
    const int v = trace_u8_variant(hu[b].c.d);
    const int mode = xz_mode(hu[b].c.n, hu[b].c.d);
    size_t e = b;
    while (e < ku && trace_u8_variant(hu[e].c.d) == v && xz_mode(hu[e].c.n, hu[e].c.d) == mode) ++e;
    runs.push_back(Run{b, e, v, mode, slot_total});
    if (mode == 2) {
      const size_t grid = std::min<size_t>(e - b, 2 * (size_t)ctx->num_sms);
      slot_total += trace_u8_xz_bytes(hu[b].c.n) * grid;
    } else if (mode == 6) {
      const size_t grid = std::min<size_t>(e - b, 2 * (size_t)ctx->num_sms);
      slot_total += trace_p3_xz_bytes(hu[b].c.n) * grid;
    } else if (mode == 8) {
      const size_t grid = std::min<size_t>(e - b, 2 * (size_t)ctx->num_sms);
      slot_total += trace_n4_xz_bytes(hu[b].c.n) * grid;
    } else if (mode == 4) {
      slot_total += trace_u8_cluster_xz(hu[b].c.n) * kTraceClusterCtas * stream_clusters(e - b);
    }
    b = e;
  }
  if (slot_total && (rc = ensure(ctx, ctx->xz_u8, slot_total)) != SDIM_OK) return rc;
  if (!runs.empty()) {
    if ((rc = ensure(ctx, ctx->xz_queue, sizeof(unsigned) * runs.size())) != SDIM_OK) return rc;
    CK(cudaMemsetAsync(ctx->xz_queue.p, 0, sizeof(unsigned) * runs.size(), s));
  }
  // the odd-d runs go on streams of their own when there are several, or when
  // the d = 2 x / z passes run on s: all x / z passes of the batch start
  // together (the uneven batch: x / z stage 295 -> 229 ms)
  const bool d2_xz = k && !skip_xz;
  const bool fan = runs.size() > 1 || (d2_xz && !runs.empty());
  if (fan) CK(cudaEventRecord(ctx->ev_xzf, s));
  // ---- x / z passes: one CTA per program (none when a kept trace is valid)
  if (d2_xz) {
    const int nmax = jobs[0].c->n;
    const size_t hot = trace_pass_hot_bytes(nmax), xz = trace_pass_xz_bytes(nmax);
    // after the tableau: the schedule window; about 3.2 KB of static shared memory besides
    const size_t win = trace_pass_window_bytes();
    const bool in_smem = !force_gmem && hot + xz + win + 4096 <= (size_t)ctx->smem_optin;
    int grid = (int)std::min<size_t>(k, 65535);
    if (!in_smem) {
      grid = std::min(grid, 2 * ctx->num_sms);
      if ((rc = ensure(ctx, ctx->gslots_xz, xz * (size_t)grid)) != SDIM_OK) return rc;
    }
    size_t smem = hot + (in_smem ? xz : 0) + win;
    if (coins && grid <= ctx->num_sms / 8) {
      // shared-memory fence: a few x / z CTAs claim enough shared memory that
      // no coin-pass block fits beside them, so the coin warps do not take
      // the issue slots of the latency-bound x / z pass on its SM
      const long long fence = (long long)ctx->smem_per_sm - 2LL * ctx->smem_reserved - (long long)kCoinFenceSmem + 16;
      const long long cap = (long long)ctx->smem_optin - 4096;  // room for the kernel's static arrays
      smem = std::max<size_t>(smem, (size_t)std::max(0LL, std::min(fence, cap)));
    }
    launch_trace_pass(ctx->trace_threads, grid, smem, s, dd, (int)k, static_cast<uint8_t*>(ctx->gslots_xz.p), xz, hot,
                      in_smem ? 1 : 0, status);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "trace pass launch");
  }
  bool used[sdim_ctx::kXzStreams] = {};
  for (size_t r = 0; r < runs.size(); ++r) {
    const Run& run = runs[r];
    const size_t b = run.b, e = run.e;
    const int v = run.v, mode = run.mode;
    cudaStream_t rs = s;
    if (fan) {
      const int si = (int)(r % sdim_ctx::kXzStreams);
      rs = ctx->xzs[si];
      if (!used[si]) CK(cudaStreamWaitEvent(rs, ctx->ev_xzf, 0));
      used[si] = true;
    }
    const int nmax = hu[b].c.n;
    if (mode >= 7) {
      // d = 5, 7 on 4-bit lanes: one CTA per program, largest first
      const bool in_smem = mode == 7;
      const int dd = hu[b].c.d;
      const int block = packed_threads(nmax, 2 * (long long)ku < ctx->num_sms);
      const size_t hot = trace_n4_hot_bytes(nmax, dd, block), xz = trace_n4_xz_bytes(nmax);
      int grid = (int)std::min<size_t>(e - b, 65535);
      if (!in_smem) grid = std::min(grid, 2 * ctx->num_sms);
      unsigned* queue = in_smem ? nullptr : static_cast<unsigned*>(ctx->xz_queue.p) + r;
      launch_trace_n4(dd, grid, block, hot + (in_smem ? xz : 0) + win, rs, du + b, (int)(e - b),
                      static_cast<uint8_t*>(ctx->xz_u8.p) + run.slot_off, xz, hot, in_smem ? 1 : 0, queue, status);
    } else if (mode >= 5) {
      // d = 3 on bit planes: one CTA per program, largest first
      const bool in_smem = mode == 5;
      const int block = packed_threads(nmax, 2 * (long long)ku < ctx->num_sms);
      const size_t hot = trace_p3_hot_bytes(nmax, block), xz = trace_p3_xz_bytes(nmax);
      int grid = (int)std::min<size_t>(e - b, 65535);
      if (!in_smem) grid = std::min(grid, 2 * ctx->num_sms);
      unsigned* queue = in_smem ? nullptr : static_cast<unsigned*>(ctx->xz_queue.p) + r;
      launch_trace_p3(grid, block, hot + (in_smem ? xz : 0) + win, rs, du + b, (int)(e - b),
                      static_cast<uint8_t*>(ctx->xz_u8.p) + run.slot_off, xz, hot, in_smem ? 1 : 0, queue, status);
    } else if (mode == 1) {
      launch_trace_u8_split(v, (int)std::min<size_t>(e - b, 32768), trace_u8_split_smem(nmax) + win,
                            trace_u8_split_smem(nmax), rs, du + b, (int)(e - b), status);
    } else if (mode >= 3) {
      const bool in_smem = mode == 3;
      const size_t hot = trace_u8_cluster_hot(nmax), xz = trace_u8_cluster_xz(nmax);
      size_t smem = hot + (in_smem ? xz : 0) + win;
      // streamed columns: more than half an SM's shared memory keeps one CTA per SM
      if (!in_smem) smem = std::max(smem, (size_t)ctx->smem_per_sm / 2);
      const size_t clusters = in_smem ? std::min<size_t>(e - b, 65535 / kTraceClusterCtas) : stream_clusters(e - b);
      launch_trace_u8_cluster(v, (int)clusters, smem, rs, du + b, (int)(e - b),
                              static_cast<uint8_t*>(ctx->xz_u8.p) + run.slot_off, xz, hot, in_smem ? 1 : 0, status);
      int maxnm = 0;
      for (size_t i = b; i < e; ++i) maxnm = std::max(maxnm, hu[i].nm);
      launch_cluster_det_headers(maxnm, rs, du + b, (int)(e - b), status);
    } else {
      const size_t hot = trace_u8_hot_bytes(nmax), xz = trace_u8_xz_bytes(nmax);
      const bool in_smem = mode == 0;
      int grid = (int)std::min<size_t>(e - b, 65535);
      if (!in_smem) grid = std::min(grid, 2 * ctx->num_sms);
      // about two generator columns per thread: 64 to kTracePassThreads threads
      const int block = std::max(64, std::min(kTracePassThreads, (nmax + 31) & ~31));
      unsigned* queue = in_smem ? nullptr : static_cast<unsigned*>(ctx->xz_queue.p) + r;
      launch_trace_u8_xz(v, grid, block, hot + (in_smem ? xz : 0) + win, rs, du + b, (int)(e - b),
                         static_cast<uint8_t*>(ctx->xz_u8.p) + run.slot_off, xz, hot, in_smem ? 1 : 0, queue, status);
    }
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "odd-d trace pass launch");
  }
  for (int i = 0; i < sdim_ctx::kXzStreams; ++i)
    if (used[i]) {
      CK(cudaEventRecord(ctx->ev_xzj[i], ctx->xzs[i]));
      CK(cudaStreamWaitEvent(s, ctx->ev_xzj[i], 0));
    }
  if (timed) CK(cudaEventRecord(ctx->ev_xzo, s));
  // ---- header and column passes: after the x / z pass, beside the rest of
  // the coin pass.  (On a stream of the highest priority their blocks shared
  // SMs with the coin pass's and the latency-bound column pass took twice as
  // long: 0.389 against 0.370 ms on the L = 7 step.)
  if (k == 1 && d2_xz && hd[0].snap) {
    launch_header_pass((jobs[0].c->nmeas + 3) / 4, s, dd, status);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "header pass launch");
  }
  if (colform && !skip_cols) {
    if (!launch_column_pass(hd[0].tw, (int)((ncols + 32 * kColumnWarps - 1) / (32 * kColumnWarps)), s, dd, status))
      return fail(ctx, SDIM_EINVAL, "no column pass for trace rows of " + std::to_string(hd[0].tw) + " words");
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "column pass launch");
    if (timed) {
      CK(cudaEventRecord(ctx->ev_cols, s));
      ctx->cols_recorded = true;
    }
  }
  // ---- coin pass on the second stream, alongside the x / z passes (independent work)
  if (coins) {
    CK(cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0));
    const int block = 256;
    const long long grid = (coins + block - 1) / block;
    if (grid > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one coin pass");
    if (timed) CK(cudaEventRecord(ctx->ev_c0, ctx->aux));
    launch_coin_pass((int)grid, block, kCoinFenceSmem, ctx->aux, dd, (int)k, coins);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "coin pass launch");
    if (timed) {
      CK(cudaEventRecord(ctx->ev_c1, ctx->aux));
      ctx->coin_recorded = true;
    }
    CK(cudaEventRecord(ctx->ev_join, ctx->aux));
    CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
  }
  if (timed) CK(cudaEventRecord(ctx->ev_xz, s));
  // ---- phase passes (the record pass for record columns)
  if (colform) {
    const long long groups = (jobs[0].nshots + 31) / 32;
    if (groups > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one record pass");
    // sdim_run with host records: the record pass in chunks of shots, each
    // chunk's rows copied down on a copy stream while the next is written
    const int K = sdim_ctx::kD2HChunks;
    const bool pipe = ctx->d2h_dst && !ctx->capture && jobs[0].out_dev == ctx->d2h_src && groups >= 8LL * K;
    const long long per = pipe ? (groups + K - 1) / K : groups;
    const size_t rowb = (size_t)jobs[0].c->nmeas;
    for (long long g0 = 0, c = 0; g0 < groups; g0 += per, ++c) {
      const long long gn = std::min(per, groups - g0);
      if (!launch_record_pass(cnw, g0, (int)gn, s, dd, gn, status))
        return fail(ctx, SDIM_EINVAL, "no record pass for columns of " + std::to_string(cnw) + " words");
      if (pipe) {
        const long long r0 = 32 * g0, rn = std::min(32 * gn, jobs[0].nshots - r0);
        CK(cudaEventRecord(ctx->ev_rec[c], s));
        CK(cudaStreamWaitEvent(ctx->cps, ctx->ev_rec[c], 0));
        CK(cudaMemcpyAsync(ctx->d2h_dst + (size_t)r0 * rowb, ctx->d2h_src + (size_t)r0 * rowb, (size_t)rn * rowb,
                           cudaMemcpyDeviceToHost, ctx->cps));
      }
    }
    if (pipe) ctx->d2h_done = true;
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "record pass launch");
  }
  for (size_t b = colform ? k : 0; b < k;) {
    const int tw = hd[b].tw, sp = hd[b].spl;
    size_t e = b;
    long long items = 0;
    while (e < k && hd[e].tw == tw) {
      items = hd[e].c.item_begin + (hd[e].c.nshots + 32 * sp - 1) / (32 * sp);
      ++e;
    }
    const int warps = kPhaseThreads / 32;
    const long long grid = (items + warps - 1) / warps;
    if (grid > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one phase pass");
    if (!launch_phase_pass(tw, sp, (int)grid, 32 * warps, s, dd + b, (int)(e - b), items, status))
      return fail(ctx, SDIM_EINVAL, "no phase pass for trace rows of " + std::to_string(tw) + " words");
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "phase pass launch");
    b = e;
  }
  for (size_t b = 0; b < ku;) {
    const int v = trace_u8_variant(hu[b].c.d);
    size_t e = b;
    long long items = 0;
    while (e < ku && trace_u8_variant(hu[e].c.d) == v) {
      items = hu[e].c.item_begin + (hu[e].c.nshots + 31) / 32;
      ++e;
    }
    const int nmax = hu[b].c.n;
    // (shot, chunk) threads: about 64 generators per thread, 32 to 512 threads
    const int nch = std::max(1, std::min(16, (2 * nmax + 63) / 64));
    if (items > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one phase pass");
    launch_trace_u8_phase(v, (int)items, 32 * nch, trace_u8_phase_smem(nmax), s, du + b, (int)(e - b), items,
                          status);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "odd-d phase pass launch");
    b = e;
  }
  if (timed) {
    CK(cudaEventRecord(ctx->ev_phase, s));
    ctx->stages_recorded = true;
  }
  return SDIM_OK;
}

// Launches every job, grouped by engine variant: one persistent launch per
// variant (or one single-warp launch per shot with SDIM_FLAG_PLAIN).  Work
// items are shots for per-shot engines and 32-shot groups for group engines;
// inside a variant the most expensive programs are queued first.  d = 2 jobs
// with enough shots go to the trace engine first (use_trace).
int launch_jobs(sdim_ctx* ctx, std::vector<Job>& all_jobs, cudaStream_t s, unsigned flags) {
  const bool plain = flags & SDIM_FLAG_PLAIN;
  const bool force_gmem = flags & SDIM_FLAG_FORCE_GMEM;
  ctx->last_stream = s;
  ctx->xz_pending = nullptr;
  ctx->pend_trace = ctx->pend_cols = false;
  std::vector<Job> jobs, tjobs, ujobs;
  for (const Job& j : all_jobs) (use_trace(j, flags) ? tjobs : use_trace_u8(j, flags) ? ujobs : jobs).push_back(j);
  int rc;
  if ((rc = ensure(ctx, ctx->status, sizeof(int))) != SDIM_OK) return rc;
  if ((rc = ensure(ctx, ctx->counters, sizeof(unsigned long long) * V_COUNT)) != SDIM_OK) return rc;
  if ((rc = ensure(ctx, ctx->descs, sizeof(CircuitDesc) * std::max<size_t>(jobs.size(), 1))) != SDIM_OK)
    return rc;
  std::vector<int> var(jobs.size());
  for (size_t i = 0; i < jobs.size(); ++i) var[i] = job_variant(jobs[i].c, flags);
  std::vector<int> order(jobs.size());
  for (size_t i = 0; i < jobs.size(); ++i) order[i] = (int)i;
  auto cost = [&](const Job& j) { return (double)j.c->nops * (double)j.c->n * (double)j.c->n; };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (var[a] != var[b]) return var[a] < var[b];
    return cost(jobs[a]) > cost(jobs[b]);
  });
  std::vector<CircuitDesc> hd(jobs.size());
  struct Group { int variant, begin, end; long long items; size_t hot, big; int block; };
  std::vector<Group> groups;
  for (size_t k = 0; k < order.size(); ++k) {
    const Job& j = jobs[order[k]];
    const int v = var[order[k]];
    const VariantOps& ops = variant_ops(v);
    if (groups.empty() || groups.back().variant != v) groups.push_back(Group{v, (int)k, (int)k, 0, 0, 0, 32});
    Group& g = groups.back();
    CircuitDesc& dsc = hd[k];
    std::memset(&dsc, 0, sizeof(dsc));
    dsc.ops = j.c->d_ops;
    dsc.out = j.out_dev;
    dsc.seed = j.seed;
    dsc.shot0 = j.shot0;
    dsc.item_begin = g.items;
    dsc.nops = j.c->nops;
    dsc.n = j.c->n;
    dsc.d = j.c->d;
    dsc.nmeas = j.c->nmeas;
    dsc.nshots = (int)j.nshots;
    g.items += ops.group ? (j.nshots + 31) / 32 : j.nshots;
    g.hot = std::max(g.hot, ops.hot_bytes(j.c->n));
    g.big = std::max(g.big, ops.big_bytes(j.c->n));
    g.block = std::max(g.block, ops.cta ? cta_block_for(j.c->n) : 32);
    g.end = (int)k + 1;
  }
  CircuitDesc* ddesc = static_cast<CircuitDesc*>(ctx->descs.p);
  if (!hd.empty() && (rc = upload_descs(ctx, ddesc, hd.data(), sizeof(CircuitDesc), hd.size(), 0,
                                        [&](size_t k) { return jobs[order[k]].index; }, s)) != SDIM_OK)
    return rc;
  CK(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), s));
  CK(cudaMemsetAsync(ctx->counters.p, 0, sizeof(unsigned long long) * V_COUNT, s));
  if (flags & SDIM_FLAG_TIME) CK(cudaEventRecord(ctx->ev0, s));
  int* status = static_cast<int*>(ctx->status.p);
  // with trace programs in the batch the shot-group engines run on a stream
  // of their own, beside the trace engines (the uneven batch: their 23 ms
  // overlap the x / z passes); they are launched after them, so the x / z
  // CTAs are dispatched first
  bool side = false;
  for (const Group& g : groups) side |= !plain && g.items > 0 && (!tjobs.empty() || !ujobs.empty());
  cudaStream_t gs = s;
  if (side) {
    CK(cudaEventRecord(ctx->ev_gf, s));
    CK(cudaStreamWaitEvent(ctx->grp, ctx->ev_gf, 0));
    gs = ctx->grp;
  }
  if ((rc = launch_trace_jobs(ctx, tjobs, ujobs, s, flags, status)) != SDIM_OK) return rc;
  if (side && (flags & SDIM_FLAG_TIME)) CK(cudaEventRecord(ctx->ev_g0, gs));
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const Group& g = groups[gi];
    if (g.items == 0) continue;
    if ((rc = set_smem_attr(ctx, g.variant)) != SDIM_OK) return rc;
    const VariantOps& ops = variant_ops(g.variant);
    if (plain) {
      const bool sm = !force_gmem && g.big <= smem_usable(ctx);
      if (!sm && (rc = ensure(ctx, ctx->gslots, g.big)) != SDIM_OK) return rc;
      for (int k = g.begin; k < g.end; ++k)
        for (long long sh = 0; sh < hd[k].nshots; ++sh)
          ops.single(sm ? g.big : 0, s, ddesc + k, sh, static_cast<uint8_t*>(ctx->gslots.p), sm ? 1 : 0, status);
    } else {
      const Plan p = plan_launch(ctx, g.variant, g.hot, g.big, g.items, g.block, force_gmem);
      if (!p.in_smem && (rc = ensure(ctx, ctx->gslots, p.big * p.slots_per_block * (size_t)p.blocks)) != SDIM_OK)
        return rc;
      unsigned long long* counter = static_cast<unsigned long long*>(ctx->counters.p) + g.variant;
      ops.persistent(dim3(p.blocks), dim3(p.team_threads * p.slots_per_block), p.smem_per_block, gs,
                     ddesc + g.begin, g.end - g.begin, g.items, counter, static_cast<uint8_t*>(ctx->gslots.p),
                     p.big, p.hot, p.in_smem ? 1 : 0, status);
    }
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "kernel launch");
  }
  if (side) {
    if (flags & SDIM_FLAG_TIME) {
      CK(cudaEventRecord(ctx->ev_g1, gs));
      ctx->group_recorded = true;
    }
    CK(cudaEventRecord(ctx->ev_gj, gs));
    CK(cudaStreamWaitEvent(s, ctx->ev_gj, 0));
  }
  return SDIM_OK;
}

// Shared-memory read bandwidth probe: every thread streams 16-byte words out
// of a 32 KB shared buffer; the xor keeps the loads live.
__global__ void __launch_bounds__(1024) k_smem_probe(int iters, uint4* sink) {
  __shared__ uint4 buf[2048];
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) buf[i] = make_uint4(i, i + 1, i + 2, i + 3);
  __syncthreads();
  uint4 acc = make_uint4(0, 0, 0, 0);
  int idx = threadIdx.x;
  for (int it = 0; it < iters; ++it) {
    const uint4 v = buf[idx & 2047];
    acc.x ^= v.x; acc.y ^= v.y; acc.z ^= v.z; acc.w ^= v.w;
    idx += blockDim.x + 1;
  }
  if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9e3779b9u) sink[blockIdx.x] = acc;
}

// L2 read-write bandwidth probe: every pass reads and rewrites each 16-byte
// word of a buffer that fits in L2, as the rank-1 update of columns held in
// L2 does; four words in flight per thread.
__global__ void __launch_bounds__(512) k_l2_probe(uint4* buf, size_t words, int passes) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int p = 0; p < passes; ++p) {
    size_t i = t0;
    for (; i + 3 * stride < words; i += 4 * stride) {
      uint4 v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = buf[i + j * stride];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        v[j].x ^= 1u;
        buf[i + j * stride] = v[j];
      }
    }
    for (; i < words; i += stride) {
      uint4 v = buf[i];
      v.x ^= 1u;
      buf[i] = v;
    }
  }
}

// Op-table rows (gate id, qudit, target, channel) -> device instruction
// words appended to dev (sdim/program.py:13-32 dispatch table, with CZ /
// CZ_INV / SWAP / M_X expanded as sdim/tableau/tableau_gates.py:229-329 does).
int encode_rows(sdim_ctx* ctx, const int32_t* ops, int64_t nops, const double* noise_prob, int n, int d,
                std::vector<uint2>& dev, int& nmeas, int& nn1) {
  if (n < 1) return fail(ctx, SDIM_EINVAL, "Number of qudits must be greater than 0");
  if (d < 2) return fail(ctx, SDIM_EINVAL, "Dimension must be greater than 1");
  if (!is_prime(d)) return fail(ctx, SDIM_EUNSUPPORTED, "composite dimension: only prime d has a tableau path here");
  if (d > 127) return fail(ctx, SDIM_EUNSUPPORTED, "dimension above 127 is not supported");
  if (n > (1 << 20)) return fail(ctx, SDIM_EINVAL, "too many qudits");
  dev.reserve(dev.size() + (size_t)nops + 8);
  nmeas = 0;
  nn1 = 0;
  auto emit = [&](uint32_t op, int q, uint32_t y) { dev.push_back(make_uint2(op | ((uint32_t)q << 8), y)); };
  for (int64_t i = 0; i < nops; ++i) {
    const int id = ops[4 * i], q = ops[4 * i + 1], t = ops[4 * i + 2], ch = ops[4 * i + 3];
    if (id < 0 || id > 17) return fail(ctx, SDIM_EINVAL, "Invalid gate value " + std::to_string(id));
    if (q < 0 || q >= n)
      return fail(ctx, SDIM_EINVAL, "qudit index " + std::to_string(q) + " out of range at instruction " +
                                        std::to_string(i));
    const bool two = id >= 9 && id <= 13;
    if (two && (t < 0 || t >= n))
      return fail(ctx, SDIM_EINVAL, "target index " + std::to_string(t) + " out of range at instruction " +
                                        std::to_string(i));
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
      case 11:  // CZ = H_INV(t) CNOT(c,t) H(t)   (tableau_gates.py:229-244)
        emit(OP_H_INV, t, 0); emit(OP_CNOT, q, t); emit(OP_H, t, 0);
        break;
      case 12:  // CZ_INV = H_INV(t) CNOT_INV(c,t) H(t)   (tableau_gates.py:246-261)
        emit(OP_H_INV, t, 0); emit(OP_CNOT_INV, q, t); emit(OP_H, t, 0);
        break;
      case 13:  // SWAP, prime-d sequence (tableau_gates.py:320-328)
        emit(OP_CNOT, q, t); emit(OP_H, q, 0); emit(OP_H, t, 0);
        emit(OP_CNOT, q, t); emit(OP_H, q, 0); emit(OP_H, t, 0);
        emit(OP_CNOT, q, t); emit(OP_H, t, 0); emit(OP_H, t, 0);
        break;
      case 14: emit(OP_M, q, 0); ++nmeas; break;
      case 15:  // M_X = H_INV then measure (tableau_gates.py:280-296)
        emit(OP_H_INV, q, 0); emit(OP_M, q, 0); ++nmeas;
        break;
      case 16: emit(OP_RESET, q, 0); ++nmeas; break;
      case 17: {
        const double p = noise_prob ? noise_prob[i] : 0.01;
        if (!(p == p)) return fail(ctx, SDIM_EINVAL, "noise probability is NaN");
        if (ch < 1 || ch > 3) return fail(ctx, SDIM_EINVAL, "Must specify a valid noise channel.");
        const double thr = std::floor((1.0 - p) * 4294967296.0);
        ++nn1;
        if (thr >= 4294967296.0) {
          emit(OP_N1OFF, q, 0);
        } else {
          const uint32_t th = thr <= 0.0 ? 0u : (uint32_t)thr;
          emit(ch == 1 ? OP_N1D : ch == 2 ? OP_N1F : OP_N1P, q, th);
        }
        break;
      }
    }
    dev.back().x |= kOpEnd;
  }
  if (dev.size() > (size_t)0x7fffffff) return fail(ctx, SDIM_EINVAL, "program too long");
  return SDIM_OK;
}

// Layered instruction stream of an odd-d program for the cluster x / z pass
// (trace_cluster_u8.cuh), appended to dev: the program's
// instructions, with each run of gates between two measurements, RESETs or
// N1 reordered into layers -- every gate goes one layer after the last gate
// that shares a qudit with it, so a layer's gates act on pairwise disjoint
// qudits -- and each layer cut into groups of up to kGateGroup gates, a
// group being the header {OP_GROUP, count} and its gates.  Gates on disjoint
// qudits commute and their phase terms add, so a thread applies a group to
// its column with all operands loaded first.  Each run starts with
// {OP_RUN, words}, so that warps holding no column pass it in one step.  No
// group straddles a window of kOpWindow words (NOPs pad the window's end).
// Gates on out-of-range qudits stay single, for the walker's own check.
void append_layers_u8(std::vector<uint2>& dev, size_t op_begin, size_t nops, int n, int64_t& off, int& count) {
  std::vector<uint2> out;
  std::vector<std::vector<uint2>> layers;
  std::vector<int> level(std::max(n, 1), -1);
  std::vector<int> touched;
  auto put_group = [&](const uint2* g, int cnt) {
    const size_t pos = out.size() % (size_t)kOpWindow;
    if (pos + (size_t)cnt + 1 > (size_t)kOpWindow)
      out.insert(out.end(), (size_t)kOpWindow - pos, make_uint2(OP_NOP, 0u));
    out.push_back(make_uint2(OP_GROUP, (uint32_t)cnt));
    out.insert(out.end(), g, g + cnt);
  };
  auto flush = [&]() {
    if (layers.empty()) return;
    const size_t head = out.size();  // {OP_RUN, words of the run}
    out.push_back(make_uint2(OP_RUN, 0u));
    for (const auto& l : layers)
      for (size_t a = 0; a < l.size(); a += kGateGroup) {
        const int cnt = (int)std::min<size_t>(kGateGroup, l.size() - a);
        if (cnt == 1)
          out.push_back(l[a]);
        else
          put_group(l.data() + a, cnt);
      }
    out[head].y = (uint32_t)(out.size() - head - 1);
    layers.clear();
    for (int q : touched) level[q] = -1;
    touched.clear();
  };
  for (size_t i = op_begin; i < op_begin + nops; ++i) {
    const uint2 w = dev[i];
    const uint32_t op = w.x & kOpMask;
    if (op == OP_NOP) continue;
    const bool gate = op >= OP_X && op <= OP_CNOT_INV;
    const bool two = op == OP_CNOT || op == OP_CNOT_INV;
    const int q = (int)(w.x >> 8), t = (int)w.y;
    if (!gate || q >= n || (two && t >= n)) {
      flush();
      out.push_back(w);
      continue;
    }
    int lv = level[q] + 1;
    if (two) lv = std::max(lv, level[t] + 1);
    if (lv == (int)layers.size()) layers.emplace_back();
    layers[lv].push_back(make_uint2(w.x & ~kOpEnd, w.y));
    if (level[q] < 0) touched.push_back(q);
    level[q] = lv;
    if (two) {
      if (level[t] < 0) touched.push_back(t);
      level[t] = lv;
    }
  }
  flush();
  off = (int64_t)dev.size();
  count = (int)out.size();
  dev.insert(dev.end(), out.begin(), out.end());
}

// Layered schedule of a d = 2 program for the trace engine's x / z pass,
// appended to dev after the instruction words (16-byte aligned):
//   steps[s] = {kind, first, count, 0}: kind 0 is a gate layer -- ops on
//     pairwise disjoint qudits with at most one P / P_INV, the only ops
//     whose common-phase update is not a plain xor -- and kind 1 a block of
//     consecutive M / RESET, with the N1 between them (an N1 only reads its
//     rows, so it can wait for the measurements around it);
//   lops[i] = {instruction word, y, ordinal (measurement index of M /
//     RESET, noise ordinal of N1), N1 ordinals before it (M / RESET)};
//   wins[i] = {first step, steps, first op, ops}: windows of at most
//     win_steps steps and win_ops ops that the pass stages in shared memory
//     (a longer step is a window of its own, read in place).
// Between two measurements only ops that share a qudit (or two P's) are
// ordered, so each op goes one level after the last op it follows.
void append_schedule(std::vector<uint2>& dev, size_t op_begin, size_t nops, int n, int win_steps, int win_ops,
                     TraceSchedule& out) {
  std::vector<uint4> steps, lops, wins;
  std::vector<std::vector<uint4>> layers;
  std::vector<int> last(n, -1), gen(n, -1);
  // where the last op on each qudit sits when it is a gate (layer, position,
  // slot 2 or 3 of its entry: z for the first qudit, w for a CNOT target), or
  // layer -1: an N1 that follows reads the gate's columns, so it rides on the
  // gate's tasks (the slot holds its ordinal + 1) instead of taking a layer
  struct GateSlot { int layer, pos, slot; };
  std::vector<GateSlot> lgate(n, GateSlot{-1, 0, 0});
  int window = 0, last_p = -1;
  bool in_block = false;
  uint32_t mord = 0, nord = 0;
  auto flush = [&]() {
    for (auto& l : layers) {
      steps.push_back(make_uint4(0u, (uint32_t)lops.size(), (uint32_t)l.size(), 0u));
      lops.insert(lops.end(), l.begin(), l.end());
    }
    layers.clear();
    ++window;
    last_p = -1;
  };
  auto level = [&](int q) { return gen[q] == window ? last[q] : -1; };
  for (size_t i = op_begin; i < op_begin + nops; ++i) {
    const uint2 w = dev[i];
    const uint32_t op = w.x & kOpMask;
    const int q = (int)(w.x >> 8);
    if (op == OP_NOP) continue;
    const bool noise = op == OP_N1D || op == OP_N1F || op == OP_N1P || op == OP_N1OFF;
    if (op == OP_M || op == OP_RESET) {
      if (!layers.empty()) {
        flush();
        in_block = false;
      }
      if (!in_block) {
        steps.push_back(make_uint4(1u, (uint32_t)lops.size(), 0u, 0u));
        in_block = true;
        ++window;
      }
      lops.push_back(make_uint4(w.x, w.y, mord++, nord));
      ++steps.back().z;
      continue;
    }
    if (noise && in_block) {
      lops.push_back(make_uint4(w.x, w.y, nord++, mord));  // w: the next measurement's ordinal
      ++steps.back().z;
      continue;
    }
    in_block = false;
    if (noise && gen[q] == window && lgate[q].layer >= 0) {
      uint4& g = layers[lgate[q].layer][lgate[q].pos];
      uint32_t& slot = lgate[q].slot == 2 ? g.z : g.w;
      if (slot == 0u) {
        slot = nord++ + 1u;
        continue;
      }
    }
    const bool two = op == OP_CNOT || op == OP_CNOT_INV;
    const bool is_p = op == OP_P || op == OP_P_INV;
    int lv = level(q) + 1;
    if (two) lv = std::max(lv, level((int)w.y) + 1);
    if (is_p) lv = std::max(lv, last_p + 1);
    if (lv == (int)layers.size()) layers.emplace_back();
    const int pos = (int)layers[lv].size();
    layers[lv].push_back(make_uint4(w.x, w.y, noise ? nord++ : 0u, 0u));
    last[q] = lv;
    gen[q] = window;
    lgate[q] = noise ? GateSlot{-1, 0, 0} : GateSlot{lv, pos, 2};
    if (two) {
      last[w.y] = lv;
      gen[w.y] = window;
      lgate[w.y] = GateSlot{lv, pos, 3};
    }
    if (is_p) last_p = lv;
  }
  if (!layers.empty()) flush();
  for (size_t s = 0; s < steps.size();) {
    if (steps[s].z > (uint32_t)win_ops) {
      wins.push_back(make_uint4((uint32_t)s, 1u, steps[s].y, steps[s].z));
      ++s;
      continue;
    }
    size_t e = s;
    uint32_t cnt = 0;
    while (e < steps.size() && e - s < (size_t)win_steps && cnt + steps[e].z <= (uint32_t)win_ops)
      cnt += steps[e++].z;
    wins.push_back(make_uint4((uint32_t)s, (uint32_t)(e - s), steps[s].y, cnt));
    s = e;
  }
  if (dev.size() & 1) dev.push_back(make_uint2(0u, 0u));
  auto put = [&](const std::vector<uint4>& v) {
    const int64_t off = (int64_t)dev.size();
    for (const uint4& x : v) {
      dev.push_back(make_uint2(x.x, x.y));
      dev.push_back(make_uint2(x.z, x.w));
    }
    return off;
  };
  out.steps_off = put(steps);
  out.lops_off = put(lops);
  out.wins_off = put(wins);
  out.nsteps = (int)steps.size();
  out.nwins = (int)wins.size();
  // N1 coin thresholds (dense, 64-ordinal padded, 16-byte aligned) and (threshold, opcode) pairs
  std::vector<uint32_t> thr;
  std::vector<uint2> hdr;
  int used = 0;
  for (size_t i = op_begin; i < op_begin + nops; ++i) {
    const uint32_t op = dev[i].x & kOpMask;
    if (op == OP_M || op == OP_RESET) used = (int)thr.size();
    if (op == OP_N1D || op == OP_N1F || op == OP_N1P || op == OP_N1OFF) {
      const uint32_t t = op == OP_N1OFF ? 0xffffffffu : dev[i].y;
      thr.push_back(t);
      hdr.push_back(make_uint2(t, op));
    }
  }
  out.nn1_used = used;
  while (thr.size() % 64) thr.push_back(0xffffffffu);
  out.nthr_off = (int64_t)dev.size();
  for (size_t i = 0; i < thr.size(); i += 2) dev.push_back(make_uint2(thr[i], thr[i + 1]));
  out.nhdr_off = (int64_t)dev.size();
  dev.insert(dev.end(), hdr.begin(), hdr.end());
  if (dev.size() & 1) dev.push_back(make_uint2(0u, 0u));
}

// Frame instruction stream (frame.cuh) of rows already checked by
// encode_rows, appended to dev: one word per instruction other than the
// identity (sdim/program.py:479-480 leaves I out of the frame walk).
void append_frame_ops(const int32_t* ops, int64_t nops, const double* noise_prob, std::vector<uint2>& dev,
                      int64_t& off, int& count) {
  off = (int64_t)dev.size();
  for (int64_t i = 0; i < nops; ++i) {
    const int id = ops[4 * i], q = ops[4 * i + 1], t = ops[4 * i + 2], ch = ops[4 * i + 3];
    if (id == 0) continue;
    uint32_t code = (uint32_t)id, y = 0;
    if (id >= 9 && id <= 13) y = (uint32_t)t;
    if (id == 17) {
      const double p = noise_prob ? noise_prob[i] : 0.01;
      const double thr = std::floor((1.0 - p) * 4294967296.0);
      if (thr >= 4294967296.0) {
        code = OP_N1OFF;
      } else {
        code = ch == 1 ? OP_N1D : ch == 2 ? OP_N1F : OP_N1P;
        y = thr <= 0.0 ? 0u : (uint32_t)thr;
      }
    }
    dev.push_back(make_uint2(code | ((uint32_t)q << 8), y));
  }
  count = (int)((int64_t)dev.size() - off);
}

}  // namespace

extern "C" {

int sdim_program_words(const int32_t* ops, int64_t nops, const double* noise_prob, int32_t n, int32_t d,
                       int32_t layered, uint32_t* out, int64_t cap, int64_t* count) {
  if ((nops > 0 && !ops) || nops < 0 || !count || (cap > 0 && !out) || cap < 0) return SDIM_EINVAL;
  std::vector<uint2> dev;
  int nmeas = 0, nn1 = 0;
  const int rc = encode_rows(nullptr, ops, nops, noise_prob, n, d, dev, nmeas, nn1);
  if (rc != SDIM_OK) return rc;
  size_t first = 0, len = dev.size();
  if (layered) {
    if (d == 2) return SDIM_EINVAL;
    int64_t off = 0;
    int cnt = 0;
    append_layers_u8(dev, 0, dev.size(), n, off, cnt);
    first = (size_t)off;
    len = (size_t)cnt;
  }
  *count = (int64_t)len;
  if ((int64_t)len > cap) return SDIM_ENOMEM;
  for (size_t k = 0; k < len; ++k) {
    out[2 * k] = dev[first + k].x;
    out[2 * k + 1] = dev[first + k].y;
  }
  return SDIM_OK;
}

int sdim_trace_xz_mode(int32_t n, int32_t d, int64_t odd_trace_programs, unsigned flags, int32_t smem_optin,
                       int32_t num_sms) {
  if (n < 1 || n > kTraceU8MaxQudits || d < 3 || !(d & 1) || odd_trace_programs < 0 || smem_optin <= 0 ||
      num_sms <= 0)
    return SDIM_EINVAL;
  return odd_xz_mode(n, d, (long long)odd_trace_programs, flags, (size_t)smem_optin, num_sms);
}

int sdim_probe_smem_bandwidth(sdim_ctx* ctx, double* gbs) {
  if (!ctx || !gbs) return fail(ctx, SDIM_EINVAL, "null argument");
  CK(cudaSetDevice(ctx->device));
  int rc = ensure(ctx, ctx->snap, sizeof(uint4) * 8 * ctx->num_sms);
  if (rc != SDIM_OK) return rc;
  const int blocks = 2 * ctx->num_sms, threads = 1024, iters = 4096;
  uint4* sink = static_cast<uint4*>(ctx->snap.p);
  k_smem_probe<<<blocks, threads, 0, ctx->stream>>>(64, sink);  // warm-up
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  k_smem_probe<<<blocks, threads, 0, ctx->stream>>>(iters, sink);
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *gbs = (double)blocks * threads * iters * 16.0 / (ms * 1e-3) / 1e9;
  return SDIM_OK;
}

int sdim_probe_l2_bandwidth(sdim_ctx* ctx, double* gbs) {
  if (!ctx || !gbs) return fail(ctx, SDIM_EINVAL, "null argument");
  CK(cudaSetDevice(ctx->device));
  const size_t bytes = (size_t)48 << 20;  // well inside the 129 MB L2
  int rc = ensure(ctx, ctx->snap, bytes);
  if (rc != SDIM_OK) return rc;
  uint4* buf = static_cast<uint4*>(ctx->snap.p);
  const size_t words = bytes / sizeof(uint4);
  const int blocks = 2 * ctx->num_sms, threads = 512, passes = 40;
  CK(cudaMemsetAsync(buf, 0, bytes, ctx->stream));
  k_l2_probe<<<blocks, threads, 0, ctx->stream>>>(buf, words, 2);  // warm-up: the buffer into L2
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  k_l2_probe<<<blocks, threads, 0, ctx->stream>>>(buf, words, passes);
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *gbs = 2.0 * (double)bytes * passes / (ms * 1e-3) / 1e9;
  return SDIM_OK;
}

int sdim_probe_philox_rate(sdim_ctx* ctx, double* blocks_per_s) {
  if (!ctx || !blocks_per_s) return fail(ctx, SDIM_EINVAL, "null argument");
  CK(cudaSetDevice(ctx->device));
  int rc = ensure(ctx, ctx->snap, 256 * sizeof(unsigned long long) + 256 * sizeof(uint4));
  if (rc != SDIM_OK) return rc;
  unsigned long long seeds[256];
  for (int i = 0; i < 256; ++i) seeds[i] = 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
  unsigned long long* dseeds = static_cast<unsigned long long*>(ctx->snap.p);
  uint4* sink = reinterpret_cast<uint4*>(dseeds + 256);
  CK(cudaMemcpyAsync(dseeds, seeds, sizeof(seeds), cudaMemcpyHostToDevice, ctx->stream));
  const int grid = 8 * ctx->num_sms, iters = 256;
  launch_philox_probe(grid, ctx->stream, dseeds, 8, sink);  // warm-up
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  launch_philox_probe(grid, ctx->stream, dseeds, iters, sink);
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaGetLastError());
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *blocks_per_s = (double)grid * 256.0 * iters * 8.0 / (ms * 1e-3);
  return SDIM_OK;
}

int sdim_ctx_create(int device, sdim_ctx** out) {
  if (!out) return SDIM_EINVAL;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return SDIM_ECUDA;
  }
  if (device < 0 || device >= count) return SDIM_EINVAL;
  sdim_ctx* ctx = new sdim_ctx();
  ctx->device = device;
  cudaSetDevice(device);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
      cudaEventCreate(&ctx->ev_xz) != cudaSuccess || cudaEventCreate(&ctx->ev_phase) != cudaSuccess ||
      cudaEventCreate(&ctx->ev_xzo) != cudaSuccess || cudaEventCreate(&ctx->ev_c0) != cudaSuccess ||
      cudaEventCreate(&ctx->ev_c1) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_xzf, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->grp, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_gf, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_gj, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&ctx->ev_g0) != cudaSuccess || cudaEventCreate(&ctx->ev_g1) != cudaSuccess ||
      cudaEventCreate(&ctx->ev_cols) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->cps, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_cps, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return SDIM_ECUDA;
  }
  for (int i = 0; i < sdim_ctx::kD2HChunks; ++i)
    if (cudaEventCreateWithFlags(&ctx->ev_rec[i], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      delete ctx;
      return SDIM_ECUDA;
    }
  for (int i = 0; i < sdim_ctx::kXzStreams; ++i)
    if (cudaStreamCreateWithFlags(&ctx->xzs[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_xzj[i], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      delete ctx;
      return SDIM_ECUDA;
    }
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
  ctx->smem_per_sm = (int)prop.sharedMemPerMultiprocessor;
  ctx->smem_reserved = (int)prop.reservedSharedMemPerBlock;
  ctx->l2_bytes = prop.l2CacheSize;
  ctx->gmem_bytes = (int64_t)prop.totalGlobalMem;
  ctx->gmem_slot_budget = std::min<size_t>((size_t)8 << 30, (size_t)(prop.totalGlobalMem / 8));
  if (const char* v = std::getenv("SDIM_TRACE_PASS_THREADS")) ctx->trace_threads = std::atoi(v) >= 512 ? 512 : 256;
  *out = ctx;
  return SDIM_OK;
}

int sdim_ctx_destroy(sdim_ctx* ctx) {
  if (!ctx) return SDIM_EINVAL;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaStreamSynchronize(ctx->aux);
  cudaStreamSynchronize(ctx->grp);
  cudaStreamSynchronize(ctx->cps);
  for (int i = 0; i < sdim_ctx::kXzStreams; ++i) cudaStreamSynchronize(ctx->xzs[i]);
  DevBuf* bufs[] = {&ctx->descs, &ctx->counters, &ctx->status, &ctx->gslots, &ctx->out, &ctx->snap, &ctx->arena,
                    &ctx->tdescs, &ctx->trace, &ctx->masks, &ctx->tdescs_u8, &ctx->trace_u8, &ctx->xz_u8,
                    &ctx->xz_queue, &ctx->gslots_xz, &ctx->cols, &ctx->dsnap, &ctx->cdet};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  if (ctx->staging) cudaFreeHost(ctx->staging);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  cudaEventDestroy(ctx->ev_xz);
  cudaEventDestroy(ctx->ev_phase);
  cudaEventDestroy(ctx->ev_xzo);
  cudaEventDestroy(ctx->ev_c0);
  cudaEventDestroy(ctx->ev_c1);
  cudaEventDestroy(ctx->ev_fork);
  cudaEventDestroy(ctx->ev_join);
  cudaEventDestroy(ctx->ev_xzf);
  cudaEventDestroy(ctx->ev_gf);
  cudaEventDestroy(ctx->ev_gj);
  cudaEventDestroy(ctx->ev_g0);
  cudaEventDestroy(ctx->ev_g1);
  cudaEventDestroy(ctx->ev_cols);
  for (int i = 0; i < sdim_ctx::kD2HChunks; ++i) cudaEventDestroy(ctx->ev_rec[i]);
  cudaEventDestroy(ctx->ev_cps);
  cudaStreamDestroy(ctx->cps);
  cudaStreamDestroy(ctx->grp);
  for (int i = 0; i < sdim_ctx::kXzStreams; ++i) {
    cudaEventDestroy(ctx->ev_xzj[i]);
    cudaStreamDestroy(ctx->xzs[i]);
  }
  cudaStreamDestroy(ctx->aux);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SDIM_OK;
}

const char* sdim_last_error(const sdim_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int sdim_device_info(sdim_ctx* ctx, int64_t info[4]) {
  if (!ctx || !info) return SDIM_EINVAL;
  info[0] = ctx->num_sms;
  info[1] = ctx->smem_optin;
  info[2] = ctx->l2_bytes;
  info[3] = ctx->gmem_bytes;
  return SDIM_OK;
}

int sdim_memory_info(sdim_ctx* ctx, int64_t info[3]) {
  if (!ctx || !info) return SDIM_EINVAL;
  CK(cudaSetDevice(ctx->device));
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  info[0] = (int64_t)free_b;
  info[1] = (int64_t)total_b;
  const DevBuf* bufs[] = {&ctx->descs, &ctx->counters, &ctx->status, &ctx->gslots, &ctx->out, &ctx->snap,
                          &ctx->arena, &ctx->tdescs, &ctx->trace, &ctx->masks, &ctx->tdescs_u8, &ctx->trace_u8,
                          &ctx->xz_u8, &ctx->xz_queue, &ctx->gslots_xz, &ctx->cols, &ctx->dsnap, &ctx->cdet};
  int64_t held = 0;
  for (const DevBuf* b : bufs) held += (int64_t)b->cap;
  info[2] = held;
  return SDIM_OK;
}

int sdim_program_bytes(const sdim_circuit* c, int64_t nshots, int64_t out[2]) {
  if (!c || !out || nshots < 0) return SDIM_EINVAL;
  const VariantOps& g = variant_ops(c->gvariant);
  out[0] = (int64_t)nshots * c->nmeas;                   // records
  out[1] = (int64_t)(g.hot_bytes(c->n) + g.big_bytes(c->n));  // one group slot
  const int tw = c->d == 2 ? trace_words(c->n) : 0;
  if (tw) out[1] += (int64_t)trace_bytes(c->nmeas, c->nn1, tw);
  return SDIM_OK;
}

int sdim_encode_circuit(sdim_ctx* ctx, const int32_t* ops, int64_t nops, const double* noise_prob, int n, int d,
                        sdim_circuit** out) {
  if (!ctx || !out || (nops > 0 && !ops) || nops < 0) return fail(ctx, SDIM_EINVAL, "null argument");
  *out = nullptr;
  std::vector<uint2> dev;
  int nmeas = 0, nn1 = 0;
  const int rc = encode_rows(ctx, ops, nops, noise_prob, n, d, dev, nmeas, nn1);
  if (rc != SDIM_OK) return rc;
  const size_t ndev = dev.size();
  TraceSchedule sch;
  if (d == 2 && trace_words(n)) append_schedule(dev, 0, ndev, n, kTraceWinSteps, kTraceWinOps, sch);
  int64_t lay_off = -1;
  int nlay = 0;
  if (d != 2) append_layers_u8(dev, 0, ndev, n, lay_off, nlay);
  int64_t fops_off = 0;
  int nfops = 0;
  append_frame_ops(ops, nops, noise_prob, dev, fops_off, nfops);
  cudaSetDevice(ctx->device);
  sdim_circuit* c = new sdim_circuit();
  c->device = ctx->device;
  c->n = n;
  c->d = d;
  c->nmeas = nmeas;
  c->nn1 = nn1;
  c->nops_user = nops;
  c->nops = (int)ndev;
  c->blob_words = (int64_t)dev.size();
  c->variant = variant_for(d);
  c->gvariant = group_variant_for(d, n, 0);
  c->gblock = variant_ops(c->gvariant).cta ? cta_block_for(n) : 32;
  const size_t bytes = std::max<size_t>(dev.size(), 1) * sizeof(uint2);
  cudaError_t e = cudaMallocHost(&c->h_ops, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_ops, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (c->h_ops) cudaFreeHost(c->h_ops);
    delete c;
    return fail(ctx, SDIM_ENOMEM, "circuit allocation failed");
  }
  if (!dev.empty()) std::memcpy(c->h_ops, dev.data(), dev.size() * sizeof(uint2));
  e = cudaMemcpy(c->d_ops, c->h_ops, dev.size() * sizeof(uint2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(c->d_ops);
    cudaFreeHost(c->h_ops);
    delete c;
    return cuda_fail(ctx, e, "circuit upload");
  }
  if (sch.steps_off >= 0) {
    c->d_steps = reinterpret_cast<const uint4*>(c->d_ops + sch.steps_off);
    c->d_lops = reinterpret_cast<const uint4*>(c->d_ops + sch.lops_off);
    c->d_wins = reinterpret_cast<const uint4*>(c->d_ops + sch.wins_off);
    c->d_nthr = reinterpret_cast<const uint32_t*>(c->d_ops + sch.nthr_off);
    c->d_nhdr = c->d_ops + sch.nhdr_off;
    c->nsteps = sch.nsteps;
    c->nwins = sch.nwins;
    c->nn1_used = sch.nn1_used;
  }
  if (lay_off >= 0) {
    c->d_lay = c->d_ops + lay_off;
    c->nlay = nlay;
  }
  c->fops_off = fops_off;
  c->nfops = nfops;
  *out = c;
  return SDIM_OK;
}

int sdim_circuit_destroy(sdim_circuit* c) {
  if (!c) return SDIM_EINVAL;
  cudaSetDevice(c->device);
  if (c->d_ops) cudaFree(c->d_ops);
  if (c->h_ops) cudaFreeHost(c->h_ops);
  if (c->xz_trace.p) cudaFree(c->xz_trace.p);
  if (c->xz_cols.p) cudaFree(c->xz_cols.p);
  delete c;
  return SDIM_OK;
}

int sdim_circuit_info(const sdim_circuit* c, int64_t info[8]) {
  if (!c || !info) return SDIM_EINVAL;
  const VariantOps& g = variant_ops(c->gvariant);
  info[0] = c->n;
  info[1] = c->d;
  info[2] = c->nmeas;
  info[3] = c->nops_user;
  info[4] = c->nops;
  info[5] = c->d == 2 ? 1 : 0;
  info[6] = (int64_t)variant_ops(c->variant).big_bytes(c->n);
  info[7] = (int64_t)(g.hot_bytes(c->n) + g.big_bytes(c->n));
  return SDIM_OK;
}

int sdim_circuit_kept(const sdim_circuit* c, int32_t out[2]) {
  if (!c || !out) return SDIM_EINVAL;
  out[0] = c->xz_trace_valid ? 1 : 0;
  out[1] = c->xz_cols_valid ? 1 : 0;
  return SDIM_OK;
}

int sdim_run_device(sdim_ctx* ctx, const sdim_circuit* c, uint64_t seed, int64_t shot0, int64_t nshots,
                    uint8_t* out_dev, void* stream, unsigned flags) {
  if (!ctx || !c || nshots < 0 || (nshots > 0 && c->nmeas > 0 && !out_dev))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_run_device");
  if (nshots > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one call");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  std::vector<Job> jobs{Job{c, seed, shot0, nshots, out_dev}};
  int rc = launch_jobs(ctx, jobs, s, flags);
  if (rc != SDIM_OK) return rc;
  return finish(ctx, s, flags);
}

int sdim_run(sdim_ctx* ctx, const sdim_circuit* c, uint64_t seed, int64_t shot0, int64_t nshots, uint8_t* out,
             unsigned flags) {
  if (flags & SDIM_FLAG_OUT_DEVICE) return sdim_run_device(ctx, c, seed, shot0, nshots, out, nullptr, flags);
  if (!ctx || !c || nshots < 0 || (nshots > 0 && c->nmeas > 0 && !out))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_run");
  if (nshots > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one call");
  CK(cudaSetDevice(ctx->device));
  const size_t bytes = (size_t)nshots * c->nmeas;
  uint8_t* direct = bytes ? mapped_host(out, flags) : nullptr;
  int rc = direct ? SDIM_OK : ensure(ctx, ctx->out, std::max<size_t>(bytes, 1));
  if (rc != SDIM_OK) return rc;
  // host -> device: the program's instruction stream; device -> host: records
  // (written into page-locked host memory by the kernels, else copied down)
  CK(cudaMemcpyAsync(c->d_ops, c->h_ops, (size_t)c->blob_words * sizeof(uint2), cudaMemcpyHostToDevice,
                     ctx->stream));
  std::vector<Job> jobs{Job{c, seed, shot0, nshots, direct ? direct : static_cast<uint8_t*>(ctx->out.p)}};
  ctx->d2h_done = false;
  if (bytes && !direct) {
    ctx->d2h_dst = out;
    ctx->d2h_src = static_cast<uint8_t*>(ctx->out.p);
  }
  rc = launch_jobs(ctx, jobs, ctx->stream, flags & ~SDIM_FLAG_ASYNC);
  ctx->d2h_dst = nullptr;
  ctx->d2h_src = nullptr;
  if (rc != SDIM_OK) {
    cudaStreamSynchronize(ctx->cps);  // no copy outlives the call
    return rc;
  }
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->timing_pending = true;
  }
  if (ctx->d2h_done) {  // the record pass's chunks are being copied on cps
    CK(cudaEventRecord(ctx->ev_cps, ctx->cps));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_cps, 0));
  } else if (bytes && !direct) {
    CK(cudaMemcpyAsync(out, ctx->out.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->timing_pending) {
    const int trc = collect_times(ctx);
    if (trc != SDIM_OK) return trc;
  }
  return settle_xz(ctx, read_status(ctx));
}

int sdim_frame_run(sdim_ctx* ctx, const sdim_circuit* c, const sdim_circuit* ref, uint64_t seed, int64_t nshots,
                   uint8_t* out, unsigned flags) {
  if (!ctx || !c || !ref || nshots < 0 || (nshots > 0 && c->nmeas > 0 && !out))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_frame_run");
  if (c->n != ref->n || c->d != ref->d || c->nmeas != ref->nmeas)
    return fail(ctx, SDIM_EINVAL, "the reference-shot program does not match the frame program");
  if (nshots > 0x7fffffffLL) return fail(ctx, SDIM_EINVAL, "too many shots in one call");
  if (nshots == 0) return SDIM_OK;
  CK(cudaSetDevice(ctx->device));
  const size_t smem = frame_smem_bytes(c->n);
  if (nshots > 1 && smem > (size_t)ctx->smem_optin)
    return fail(ctx, SDIM_EUNSUPPORTED, "too many qudits for the frame sampler's shared-memory frames");
  if (!ctx->frame_smem_set) {
    const cudaError_t e = frame_set_smem(ctx->smem_optin);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaFuncSetAttribute");
    ctx->frame_smem_set = true;
  }
  const bool dev_out = flags & SDIM_FLAG_OUT_DEVICE;
  const size_t bytes = (size_t)nshots * c->nmeas;
  int rc;
  uint8_t* dst = out;
  if (!dev_out) {
    if ((rc = ensure(ctx, ctx->out, std::max<size_t>(bytes, 1))) != SDIM_OK) return rc;
    dst = static_cast<uint8_t*>(ctx->out.p);
    // host -> device: both instruction streams
    CK(cudaMemcpyAsync(ref->d_ops, ref->h_ops, (size_t)ref->blob_words * sizeof(uint2), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(c->d_ops, c->h_ops, (size_t)c->blob_words * sizeof(uint2), cudaMemcpyHostToDevice,
                       ctx->stream));
  }
  cudaStream_t s = ctx->stream;
  // shot 0: the noiseless tableau shot, into row 0, on the trace engines
  // (one x / z pass) where they take the program: the shot-group engine
  // spends a whole group's latency on a single shot
  std::vector<Job> jobs{Job{ref, seed, 0, 1, dst}};
  if ((rc = launch_jobs(ctx, jobs, s, (flags & ~SDIM_FLAG_ASYNC) | SDIM_FLAG_TRACE)) != SDIM_OK) return rc;
  // shots 1 .. nshots - 1: frames against row 0
  if (nshots > 1 && c->nmeas > 0) {
    FrameDesc fd;
    fd.ops = c->d_ops + c->fops_off;
    fd.ref = dst;
    fd.out = dst + c->nmeas;
    fd.seed = seed;
    fd.shot0 = 1;
    fd.nops = c->nfops;
    fd.n = c->n;
    fd.d = c->d;
    fd.nmeas = c->nmeas;
    fd.nshots = (int)(nshots - 1);
    const long long grid = (nshots - 1 + 31) / 32;
    launch_frame_pass((int)grid, smem, s, fd, static_cast<int*>(ctx->status.p));
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "frame pass launch");
  }
  if (dev_out) return finish(ctx, s, flags & ~SDIM_FLAG_ASYNC);
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->timing_pending = true;
  }
  if (bytes) CK(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    const int trc = collect_times(ctx);
    if (trc != SDIM_OK) return trc;
  }
  return settle_xz(ctx, read_status(ctx));
}

int sdim_run_batch(sdim_ctx* ctx, int ncirc, const sdim_circuit* const* circs, const uint64_t* seeds,
                   const int64_t* shot0, const int64_t* nshots, uint8_t* const* outs, void* stream,
                   unsigned flags) {
  if (!ctx || ncirc < 0 || (ncirc > 0 && (!circs || !seeds || !shot0 || !nshots || !outs)))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_run_batch");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  const bool on_dev = flags & SDIM_FLAG_OUT_DEVICE;
  std::vector<Job> jobs;
  jobs.reserve(ncirc);
  size_t total = 0;
  std::vector<size_t> offs(ncirc);
  for (int i = 0; i < ncirc; ++i) {
    if (!circs[i] || nshots[i] < 0 || nshots[i] > 0x7fffffffLL)
      return fail(ctx, SDIM_EINVAL, "bad circuit or shot count at batch index " + std::to_string(i));
    if (nshots[i] > 0 && circs[i]->nmeas > 0 && !outs[i])
      return fail(ctx, SDIM_EINVAL, "null output at batch index " + std::to_string(i));
    offs[i] = total;
    total += (size_t)nshots[i] * circs[i]->nmeas;
  }
  int rc;
  // host outputs in page-locked memory are written by the kernels directly
  std::vector<uint8_t*> direct(ncirc, nullptr);
  bool staged = false;
  for (int i = 0; i < ncirc && !on_dev; ++i) {
    if ((size_t)nshots[i] * circs[i]->nmeas == 0) continue;
    direct[i] = mapped_host(outs[i], flags);
    staged |= !direct[i];
  }
  if (staged && (rc = ensure(ctx, ctx->out, std::max<size_t>(total, 1))) != SDIM_OK) return rc;
  for (int i = 0; i < ncirc; ++i) {
    uint8_t* o = on_dev ? outs[i] : direct[i] ? direct[i] : static_cast<uint8_t*>(ctx->out.p) + offs[i];
    jobs.push_back(Job{circs[i], seeds[i], shot0[i], nshots[i], o});
  }
  rc = launch_jobs(ctx, jobs, s, flags);
  if (rc != SDIM_OK) return rc;
  if (on_dev) return finish(ctx, s, flags);
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->timing_pending = true;
  }
  for (int i = 0; i < ncirc; ++i) {
    const size_t b = (size_t)nshots[i] * circs[i]->nmeas;
    if (b && !direct[i])
      CK(cudaMemcpyAsync(outs[i], static_cast<uint8_t*>(ctx->out.p) + offs[i], b, cudaMemcpyDeviceToHost, s));
  }
  if (flags & SDIM_FLAG_ASYNC) {
    // the caller keeps the (pinned) host buffers alive until sdim_query / sdim_sync
    ctx->last_stream = s;
    return SDIM_OK;
  }
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    const int trc = collect_times(ctx);
    if (trc != SDIM_OK) return trc;
  }
  return settle_xz(ctx, read_status(ctx));
}

int sdim_graph_create(sdim_ctx* parent, int ncirc, const sdim_circuit* const* circs, const uint64_t* seeds,
                      const int64_t* shot0, const int64_t* nshots, uint8_t* const* outs_dev, unsigned flags,
                      sdim_graph** out) {
  sdim_ctx* ctx = parent;
  if (!ctx || !out || ncirc < 0 || (ncirc > 0 && (!circs || !seeds || !shot0 || !nshots || !outs_dev)))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_graph_create");
  *out = nullptr;
  if (flags & SDIM_FLAG_PLAIN) return fail(ctx, SDIM_EINVAL, "the plain form (one launch per shot) is not captured");
  std::vector<Job> jobs;
  jobs.reserve(ncirc);
  for (int i = 0; i < ncirc; ++i) {
    if (!circs[i] || nshots[i] < 0 || nshots[i] > 0x7fffffffLL)
      return fail(ctx, SDIM_EINVAL, "bad circuit or shot count at batch index " + std::to_string(i));
    if (circs[i]->device != ctx->device)
      return fail(ctx, SDIM_EINVAL, "circuit at batch index " + std::to_string(i) + " lives on another device");
    if (nshots[i] > 0 && circs[i]->nmeas > 0 && !outs_dev[i])
      return fail(ctx, SDIM_EINVAL, "null output at batch index " + std::to_string(i));
    jobs.push_back(Job{circs[i], seeds[i], shot0[i], nshots[i], outs_dev[i], i});
  }
  CK(cudaSetDevice(ctx->device));
  sdim_graph* g = new sdim_graph();
  g->njobs = ncirc;
  int rc = sdim_ctx_create(ctx->device, &g->own);
  if (rc != SDIM_OK) {
    delete g;
    return fail(ctx, rc, "graph: context creation failed");
  }
  auto bail = [&](int code) {
    const std::string why = "graph: " + g->own->err;
    g->own->capture = nullptr;
    sdim_graph_destroy(g);
    return fail(parent, code, why);
  };
  ctx = g->own;
  const unsigned f = (flags & ~(SDIM_FLAG_TIME | SDIM_FLAG_ASYNC)) | SDIM_FLAG_OUT_DEVICE;
  // 1. the run, uncaptured: checks the programs, sizes every device buffer
  //    and the descriptor staging, sets the kernels' shared-memory limits
  ctx->capture = &g->cap;
  rc = launch_jobs(ctx, jobs, ctx->stream, f);
  if (rc == SDIM_OK) rc = finish(ctx, ctx->stream, f);
  if (rc != SDIM_OK) return bail(rc);
  if (g->cap.need) {
    void* h = nullptr;
    if (cudaMallocHost(&h, g->cap.need) != cudaSuccess) {
      cudaGetLastError();
      fail(ctx, SDIM_ENOMEM, "pinned descriptor staging");
      return bail(SDIM_ENOMEM);
    }
    g->cap.host = static_cast<uint8_t*>(h);
    g->cap.cap = g->cap.need;
  }
  g->cap.sizing = false;
  // 2. the same run, captured: buffers are already large enough, so nothing
  //    is allocated and every node points at memory that stays put
  const unsigned long long moved = ctx->reallocs;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaStreamBeginCapture"));
  rc = launch_jobs(ctx, jobs, ctx->stream, f);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &graph);
  ctx->capture = nullptr;
  g->graph = graph;
  if (rc != SDIM_OK) return bail(rc);
  if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaStreamEndCapture"));
  if (ctx->reallocs != moved) {
    fail(ctx, SDIM_ECUDA, "a device buffer moved during capture");
    return bail(SDIM_ECUDA);
  }
  e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaGraphInstantiate"));
  *out = g;
  return SDIM_OK;
}

int sdim_graph_launch(sdim_graph* g, const uint64_t* seeds, const int64_t* shot0, void* stream) {
  if (!g || !g->exec) return SDIM_EINVAL;
  sdim_ctx* ctx = g->own;
  CK(cudaSetDevice(ctx->device));
  if (seeds || shot0) {
    // the last replay's copy node may not have read the staging yet
    if (g->launched) CK(cudaEventSynchronize(g->done));
    if (seeds)
      for (const auto& a : g->cap.seed_at) std::memcpy(g->cap.host + a.first, &seeds[a.second], sizeof(uint64_t));
    if (shot0)
      for (const auto& a : g->cap.shot0_at) std::memcpy(g->cap.host + a.first, &shot0[a.second], sizeof(int64_t));
  }
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  CK(cudaGraphLaunch(g->exec, s));
  CK(cudaEventRecord(g->done, s));
  g->launched = true;
  return SDIM_OK;
}

int sdim_graph_sync(sdim_graph* g) {
  if (!g) return SDIM_EINVAL;
  sdim_ctx* ctx = g->own;
  CK(cudaSetDevice(ctx->device));
  if (!g->launched) return SDIM_OK;
  CK(cudaEventSynchronize(g->done));
  return read_status(ctx);
}

int sdim_graph_info(const sdim_graph* g, int64_t info[3]) {
  if (!g || !info || !g->graph) return SDIM_EINVAL;
  size_t count = 0;
  if (cudaGraphGetNodes(g->graph, nullptr, &count) != cudaSuccess) return SDIM_ECUDA;
  std::vector<cudaGraphNode_t> nodes(count);
  if (count && cudaGraphGetNodes(g->graph, nodes.data(), &count) != cudaSuccess) return SDIM_ECUDA;
  int64_t kernels = 0;
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) != cudaSuccess) return SDIM_ECUDA;
    kernels += t == cudaGraphNodeTypeKernel;
  }
  info[0] = (int64_t)count;
  info[1] = kernels;
  info[2] = (int64_t)g->cap.cap;
  return SDIM_OK;
}

const char* sdim_graph_last_error(const sdim_graph* g) { return g ? g->own->err.c_str() : "null graph"; }

int sdim_graph_destroy(sdim_graph* g) {
  if (!g) return SDIM_EINVAL;
  if (g->own) {
    cudaSetDevice(g->own->device);
    if (g->launched) cudaEventSynchronize(g->done);
  }
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->done) cudaEventDestroy(g->done);
  if (g->cap.host) cudaFreeHost(g->cap.host);
  if (g->own) sdim_ctx_destroy(g->own);
  delete g;
  return SDIM_OK;
}

int sdim_run_tables(sdim_ctx* ctx, int ncirc, const int32_t* rows, const int64_t* row_begin,
                    const double* noise_prob, const int32_t* n, const int32_t* d, const uint64_t* seeds,
                    const int64_t* shot0, const int64_t* nshots, uint8_t* const* outs, void* stream,
                    unsigned flags) {
  if (!ctx || ncirc < 0 || (ncirc > 0 && (!rows || !row_begin || !n || !d || !seeds || !shot0 || !nshots || !outs)))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_run_tables");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  std::vector<uint2> dev;
  std::vector<size_t> op_off(ncirc);
  std::vector<TraceSchedule> sch(ncirc);
  std::vector<int64_t> lay_off(ncirc, -1);
  std::vector<int> nlay(ncirc, 0);
  // layered streams only serve the cluster x / z pass, which a batch takes
  // only with fewer than num_sms / 2 odd-d programs (odd_xz_mode); larger
  // batches skip building them (SDIM_FLAG_CLUSTER_XZ then walks the
  // instructions as written)
  int odd = 0;
  for (int i = 0; i < ncirc; ++i) odd += d[i] != 2 ? 1 : 0;
  const bool layered = 2 * odd < ctx->num_sms;
  std::vector<sdim_circuit> circs(ncirc);
  int rc;
  for (int i = 0; i < ncirc; ++i) {
    op_off[i] = dev.size();
    int nmeas = 0, nn1 = 0;
    const int64_t r0 = row_begin[i], r1 = row_begin[i + 1];
    if (r1 < r0) return fail(ctx, SDIM_EINVAL, "row offsets must not decrease");
    rc = encode_rows(ctx, rows + 4 * r0, r1 - r0, noise_prob ? noise_prob + r0 : nullptr, n[i], d[i], dev, nmeas, nn1);
    if (rc != SDIM_OK) return rc;
    sdim_circuit& c = circs[i];
    c.device = ctx->device;
    c.n = n[i];
    c.d = d[i];
    c.nmeas = nmeas;
    c.nn1 = nn1;
    c.nops_user = r1 - r0;
    c.nops = (int)(dev.size() - op_off[i]);
    if (d[i] == 2 && trace_words(n[i]))
      append_schedule(dev, op_off[i], (size_t)c.nops, n[i], kTraceWinSteps, kTraceWinOps, sch[i]);
    if (d[i] != 2 && layered) append_layers_u8(dev, op_off[i], (size_t)c.nops, n[i], lay_off[i], nlay[i]);
    c.variant = variant_for(d[i]);
    c.gvariant = group_variant_for(d[i], n[i], 0);
    c.gblock = variant_ops(c.gvariant).cta ? cta_block_for(n[i]) : 32;
  }
  // instruction streams: pinned staging -> device arena, both owned by the context
  const size_t ob = std::max<size_t>(dev.size(), 1) * sizeof(uint2);
  if ((rc = ensure(ctx, ctx->arena, ob)) != SDIM_OK) return rc;
  if (ctx->staging_cap < ob) {
    const size_t cap = std::max(ob, ctx->staging_cap + ctx->staging_cap / 2);
    if (ctx->staging) cudaFreeHost(ctx->staging);
    ctx->staging = nullptr;
    ctx->staging_cap = 0;
    if (cudaMallocHost(&ctx->staging, cap) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, SDIM_ENOMEM, "pinned staging allocation failed");
    }
    ctx->staging_cap = cap;
  }
  if (!dev.empty()) std::memcpy(ctx->staging, dev.data(), dev.size() * sizeof(uint2));
  CK(cudaMemcpyAsync(ctx->arena.p, ctx->staging, dev.size() * sizeof(uint2), cudaMemcpyHostToDevice, s));
  uint2* base = static_cast<uint2*>(ctx->arena.p);
  for (int i = 0; i < ncirc; ++i) {
    circs[i].d_ops = base + op_off[i];
    if (sch[i].steps_off >= 0) {
      circs[i].d_steps = reinterpret_cast<const uint4*>(base + sch[i].steps_off);
      circs[i].d_lops = reinterpret_cast<const uint4*>(base + sch[i].lops_off);
      circs[i].d_wins = reinterpret_cast<const uint4*>(base + sch[i].wins_off);
      circs[i].d_nthr = reinterpret_cast<const uint32_t*>(base + sch[i].nthr_off);
      circs[i].d_nhdr = base + sch[i].nhdr_off;
      circs[i].nsteps = sch[i].nsteps;
      circs[i].nwins = sch[i].nwins;
      circs[i].nn1_used = sch[i].nn1_used;
    }
    if (lay_off[i] >= 0) {
      circs[i].d_lay = base + lay_off[i];
      circs[i].nlay = nlay[i];
    }
  }
  const bool on_dev = flags & SDIM_FLAG_OUT_DEVICE;
  std::vector<size_t> offs(ncirc);
  size_t total = 0;
  for (int i = 0; i < ncirc; ++i) {
    if (nshots[i] < 0 || nshots[i] > 0x7fffffffLL)
      return fail(ctx, SDIM_EINVAL, "bad shot count at index " + std::to_string(i));
    if (nshots[i] > 0 && circs[i].nmeas > 0 && !outs[i])
      return fail(ctx, SDIM_EINVAL, "null output at index " + std::to_string(i));
    offs[i] = total;
    total += (size_t)nshots[i] * circs[i].nmeas;
  }
  // host outputs in page-locked memory are written by the kernels directly
  std::vector<uint8_t*> direct(ncirc, nullptr);
  bool staged = false;
  for (int i = 0; i < ncirc && !on_dev; ++i) {
    if ((size_t)nshots[i] * circs[i].nmeas == 0) continue;
    direct[i] = mapped_host(outs[i], flags);
    staged |= !direct[i];
  }
  if (staged && (rc = ensure(ctx, ctx->out, std::max<size_t>(total, 1))) != SDIM_OK) return rc;
  std::vector<Job> jobs;
  jobs.reserve(ncirc);
  for (int i = 0; i < ncirc; ++i)
    jobs.push_back(Job{&circs[i], seeds[i], shot0[i], nshots[i],
                       on_dev ? outs[i] : direct[i] ? direct[i] : static_cast<uint8_t*>(ctx->out.p) + offs[i]});
  rc = launch_jobs(ctx, jobs, s, flags);
  if (rc != SDIM_OK) return rc;
  if (on_dev) return finish(ctx, s, flags);
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->timing_pending = true;
  }
  for (int i = 0; i < ncirc; ++i) {
    const size_t b = (size_t)nshots[i] * circs[i].nmeas;
    if (b && !direct[i])
      CK(cudaMemcpyAsync(outs[i], static_cast<uint8_t*>(ctx->out.p) + offs[i], b, cudaMemcpyDeviceToHost, s));
  }
  if (flags & SDIM_FLAG_ASYNC) return SDIM_OK;
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    const int trc = collect_times(ctx);
    if (trc != SDIM_OK) return trc;
  }
  return read_status(ctx);
}

int sdim_query(sdim_ctx* ctx) {
  if (!ctx) return SDIM_EINVAL;
  CK(cudaSetDevice(ctx->device));
  const cudaError_t e = cudaStreamQuery(ctx->last_stream ? ctx->last_stream : ctx->stream);
  if (e == cudaErrorNotReady) return 0;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamQuery");
  return 1;
}

int sdim_host_alloc(size_t bytes, void** out) {
  if (!out) return SDIM_EINVAL;
  *out = nullptr;
  if (cudaMallocHost(out, std::max<size_t>(bytes, 1)) != cudaSuccess) {
    cudaGetLastError();
    return SDIM_ENOMEM;
  }
  return SDIM_OK;
}

int sdim_host_free(void* p) {
  if (p && cudaFreeHost(p) != cudaSuccess) {
    cudaGetLastError();
    return SDIM_ECUDA;
  }
  return SDIM_OK;
}

int sdim_sync(sdim_ctx* ctx) {
  if (!ctx) return SDIM_EINVAL;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->last_stream ? ctx->last_stream : ctx->stream));
  if (ctx->timing_pending) {
    const int trc = collect_times(ctx);
    if (trc != SDIM_OK) return trc;
  }
  return ctx->status.p ? read_status(ctx) : SDIM_OK;
}

double sdim_last_kernel_ms(const sdim_ctx* ctx) { return ctx ? ctx->last_ms : -1.0; }

int sdim_last_stage_ms(const sdim_ctx* ctx, double out[3]) {
  if (!ctx || !out) return SDIM_EINVAL;
  for (int i = 0; i < 3; ++i) out[i] = ctx->stage_ms[i];
  return SDIM_OK;
}

int sdim_last_pass_ms(const sdim_ctx* ctx, double out[2]) {
  if (!ctx || !out) return SDIM_EINVAL;
  out[0] = ctx->pass_ms[0];
  out[1] = ctx->pass_ms[1];
  return SDIM_OK;
}

int sdim_last_passes_ms(const sdim_ctx* ctx, double* out, int n) {
  if (!ctx || (!out && n > 0) || n < 0) return SDIM_EINVAL;
  const double v[4] = {ctx->pass_ms[0], ctx->pass_ms[1], ctx->col_ms, ctx->group_ms};
  for (int i = 0; i < n && i < 4; ++i) out[i] = v[i];
  for (int i = 4; i < n; ++i) out[i] = 0.0;
  return SDIM_OK;
}

int sdim_snapshot(sdim_ctx* ctx, const sdim_circuit* c, uint64_t seed, int64_t shot, int mode, int8_t* out,
                  uint8_t* records_out, unsigned flags) {
  if (!ctx || !c || !out || shot < 0 ||
      (mode != SDIM_SNAP_EVERY_INSTRUCTION && mode != SDIM_SNAP_AT_MEASUREMENT && mode != SDIM_SNAP_FINAL))
    return fail(ctx, SDIM_EINVAL, "bad argument to sdim_snapshot");
  CK(cudaSetDevice(ctx->device));
  const size_t tb = 4 * (size_t)c->n * c->n + 2 * (size_t)c->n;
  const size_t count = mode == SDIM_SNAP_EVERY_INSTRUCTION ? (size_t)c->nops_user
                       : mode == SDIM_SNAP_AT_MEASUREMENT ? (size_t)c->nmeas
                                                          : (size_t)1;
  const int v = job_variant(c, flags);
  const VariantOps& ops = variant_ops(v);
  const bool grp = ops.group;
  const size_t hot = ops.hot_bytes(c->n), big = ops.big_bytes(c->n);
  // a group snapshot runs the 32 shots [shot - lane, shot - lane + 32) and exports lane's
  const int lane = grp ? (int)(shot % 32) : 0;
  int rc;
  if ((rc = ensure(ctx, ctx->snap, std::max<size_t>(count * tb, 1))) != SDIM_OK) return rc;
  if ((rc = ensure(ctx, ctx->out, std::max<size_t>((size_t)c->nmeas * 32, 1))) != SDIM_OK) return rc;
  if ((rc = ensure(ctx, ctx->status, sizeof(int))) != SDIM_OK) return rc;
  if ((rc = ensure(ctx, ctx->descs, sizeof(CircuitDesc))) != SDIM_OK) return rc;
  if ((rc = set_smem_attr(ctx, v)) != SDIM_OK) return rc;
  CircuitDesc dsc;
  std::memset(&dsc, 0, sizeof(dsc));
  dsc.ops = c->d_ops;
  dsc.out = static_cast<uint8_t*>(ctx->out.p);
  dsc.seed = seed;
  dsc.shot0 = shot - lane;
  dsc.nops = c->nops;
  dsc.n = c->n;
  dsc.d = c->d;
  dsc.nmeas = c->nmeas;
  dsc.nshots = grp ? 32 : 1;
  const bool in_smem = !(flags & SDIM_FLAG_FORCE_GMEM) && hot + big <= smem_usable(ctx);
  if (!in_smem && (rc = ensure(ctx, ctx->gslots, big)) != SDIM_OK) return rc;
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(ctx->descs.p, &dsc, sizeof(dsc), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), s));
  const int block = ops.cta ? cta_block_for(c->n) : 32;
  ops.snapshot(dim3(block), hot + (in_smem ? big : 0), s, static_cast<const CircuitDesc*>(ctx->descs.p), 0,
               static_cast<uint8_t*>(ctx->gslots.p), big, hot, in_smem ? 1 : 0, static_cast<int8_t*>(ctx->snap.p),
               mode, lane, static_cast<int*>(ctx->status.p));
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return cuda_fail(ctx, le, "snapshot launch");
  if (count * tb) CK(cudaMemcpyAsync(out, ctx->snap.p, count * tb, cudaMemcpyDeviceToHost, s));
  if (records_out && c->nmeas)
    CK(cudaMemcpyAsync(records_out, static_cast<uint8_t*>(ctx->out.p) + (size_t)lane * c->nmeas, c->nmeas,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return read_status(ctx);
}

}  // extern "C"
