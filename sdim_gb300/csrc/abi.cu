// C ABI of the GB300 tableau engine: context, program encoder, launch
// planner and the plain / persistent / snapshot launches.  The kernels live
// in k_pershot.cu and k_group.cu behind the launch table of variants.cuh.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sdim_gb300.h"
#include "kernels.cuh"
#include "variants.cuh"

using namespace sdim;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct sdim_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t last_stream = nullptr;  // stream of the last launch (sdim_sync / sdim_query)
  int num_sms = 0;
  int smem_optin = 0;
  int64_t l2_bytes = 0;
  int64_t gmem_bytes = 0;
  size_t gmem_slot_budget = (size_t)8 << 30;
  std::string err;
  DevBuf descs, counters, status, gslots, out, snap, arena;
  void* staging = nullptr;  // pinned host staging of sdim_run_tables
  size_t staging_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timing_pending = false;
  double last_ms = 0.0;
  int smem_attr_set[V_COUNT] = {};
};

struct sdim_circuit {
  int device = 0;
  int n = 0, d = 0, nmeas = 0;
  int64_t nops_user = 0;
  int nops = 0;
  int variant = 0;    // per-shot engine (plain form, per-shot snapshots)
  int gvariant = 0;   // shot-group engine for batched runs
  int gblock = 32;    // threads of one group team
  uint2* h_ops = nullptr;  // pinned host copy
  uint2* d_ops = nullptr;
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

int finish(sdim_ctx* ctx, cudaStream_t s, unsigned flags) {
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->timing_pending = true;
  }
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return cuda_fail(ctx, le, "kernel launch");
  if (flags & SDIM_FLAG_ASYNC) return SDIM_OK;
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->timing_pending = false;
  }
  return read_status(ctx);
}

struct Job {
  const sdim_circuit* c;
  uint64_t seed;
  int64_t shot0, nshots;
  uint8_t* out_dev;
};

// Engine used for a job: the shot-group engine for batched runs (unless
// SDIM_FLAG_PER_SHOT; SDIM_FLAG_TEAM_* override the team kind), the
// per-shot engine for the plain form.
int job_variant(const sdim_circuit* c, unsigned flags) {
  if (flags & (SDIM_FLAG_PLAIN | SDIM_FLAG_PER_SHOT)) return c->variant;
  if (flags & (SDIM_FLAG_TEAM_WARP | SDIM_FLAG_TEAM_CTA)) return group_variant_for(c->d, c->n, flags);
  return c->gvariant;
}

// Launches every job, grouped by engine variant: one persistent launch per
// variant (or one single-warp launch per shot with SDIM_FLAG_PLAIN).  Work
// items are shots for per-shot engines and 32-shot groups for group engines;
// inside a variant the most expensive programs are queued first.
int launch_jobs(sdim_ctx* ctx, std::vector<Job>& jobs, cudaStream_t s, unsigned flags) {
  const bool plain = flags & SDIM_FLAG_PLAIN;
  const bool force_gmem = flags & SDIM_FLAG_FORCE_GMEM;
  ctx->last_stream = s;
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
  if (!hd.empty())
    CK(cudaMemcpyAsync(ddesc, hd.data(), sizeof(CircuitDesc) * hd.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), s));
  CK(cudaMemsetAsync(ctx->counters.p, 0, sizeof(unsigned long long) * V_COUNT, s));
  if (flags & SDIM_FLAG_TIME) CK(cudaEventRecord(ctx->ev0, s));
  int* status = static_cast<int*>(ctx->status.p);
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
      ops.persistent(dim3(p.blocks), dim3(p.team_threads * p.slots_per_block), p.smem_per_block, s,
                     ddesc + g.begin, g.end - g.begin, g.items, counter, static_cast<uint8_t*>(ctx->gslots.p),
                     p.big, p.hot, p.in_smem ? 1 : 0, status);
    }
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(ctx, le, "kernel launch");
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

// Op-table rows (gate id, qudit, target, channel) -> device instruction
// words appended to dev (sdim/program.py:13-32 dispatch table, with CZ /
// CZ_INV / SWAP / M_X expanded as sdim/tableau/tableau_gates.py:229-329 does).
int encode_rows(sdim_ctx* ctx, const int32_t* ops, int64_t nops, const double* noise_prob, int n, int d,
                std::vector<uint2>& dev, int& nmeas) {
  if (n < 1) return fail(ctx, SDIM_EINVAL, "Number of qudits must be greater than 0");
  if (d < 2) return fail(ctx, SDIM_EINVAL, "Dimension must be greater than 1");
  if (!is_prime(d)) return fail(ctx, SDIM_EUNSUPPORTED, "composite dimension: only prime d has a tableau path here");
  if (d > 127) return fail(ctx, SDIM_EUNSUPPORTED, "dimension above 127 is not supported");
  if (n > (1 << 20)) return fail(ctx, SDIM_EINVAL, "too many qudits");
  dev.reserve(dev.size() + (size_t)nops + 8);
  nmeas = 0;
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

}  // namespace

extern "C" {

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
      cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return SDIM_ECUDA;
  }
  ctx->num_sms = prop.multiProcessorCount;
  ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
  ctx->l2_bytes = prop.l2CacheSize;
  ctx->gmem_bytes = (int64_t)prop.totalGlobalMem;
  ctx->gmem_slot_budget = std::min<size_t>((size_t)8 << 30, (size_t)(prop.totalGlobalMem / 8));
  *out = ctx;
  return SDIM_OK;
}

int sdim_ctx_destroy(sdim_ctx* ctx) {
  if (!ctx) return SDIM_EINVAL;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf* bufs[] = {&ctx->descs, &ctx->counters, &ctx->status, &ctx->gslots, &ctx->out, &ctx->snap, &ctx->arena};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  if (ctx->staging) cudaFreeHost(ctx->staging);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
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
  info[2] = (int64_t)(ctx->descs.cap + ctx->counters.cap + ctx->status.cap + ctx->gslots.cap + ctx->out.cap +
                      ctx->snap.cap);
  return SDIM_OK;
}

int sdim_program_bytes(const sdim_circuit* c, int64_t nshots, int64_t out[2]) {
  if (!c || !out || nshots < 0) return SDIM_EINVAL;
  const VariantOps& g = variant_ops(c->gvariant);
  out[0] = (int64_t)nshots * c->nmeas;                   // records
  out[1] = (int64_t)(g.hot_bytes(c->n) + g.big_bytes(c->n));  // one group slot
  return SDIM_OK;
}

int sdim_encode_circuit(sdim_ctx* ctx, const int32_t* ops, int64_t nops, const double* noise_prob, int n, int d,
                        sdim_circuit** out) {
  if (!ctx || !out || (nops > 0 && !ops) || nops < 0) return fail(ctx, SDIM_EINVAL, "null argument");
  *out = nullptr;
  std::vector<uint2> dev;
  int nmeas = 0;
  const int rc = encode_rows(ctx, ops, nops, noise_prob, n, d, dev, nmeas);
  if (rc != SDIM_OK) return rc;
  cudaSetDevice(ctx->device);
  sdim_circuit* c = new sdim_circuit();
  c->device = ctx->device;
  c->n = n;
  c->d = d;
  c->nmeas = nmeas;
  c->nops_user = nops;
  c->nops = (int)dev.size();
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
  *out = c;
  return SDIM_OK;
}

int sdim_circuit_destroy(sdim_circuit* c) {
  if (!c) return SDIM_EINVAL;
  cudaSetDevice(c->device);
  if (c->d_ops) cudaFree(c->d_ops);
  if (c->h_ops) cudaFreeHost(c->h_ops);
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
  int rc = ensure(ctx, ctx->out, std::max<size_t>(bytes, 1));
  if (rc != SDIM_OK) return rc;
  // host -> device: the program's instruction stream; device -> host: records
  CK(cudaMemcpyAsync(c->d_ops, c->h_ops, (size_t)c->nops * sizeof(uint2), cudaMemcpyHostToDevice, ctx->stream));
  std::vector<Job> jobs{Job{c, seed, shot0, nshots, static_cast<uint8_t*>(ctx->out.p)}};
  rc = launch_jobs(ctx, jobs, ctx->stream, flags & ~SDIM_FLAG_ASYNC);
  if (rc != SDIM_OK) return rc;
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->timing_pending = true;
  }
  if (bytes) CK(cudaMemcpyAsync(out, ctx->out.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->timing_pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->timing_pending = false;
  }
  return read_status(ctx);
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
  if (!on_dev && (rc = ensure(ctx, ctx->out, std::max<size_t>(total, 1))) != SDIM_OK) return rc;
  for (int i = 0; i < ncirc; ++i) {
    uint8_t* o = on_dev ? outs[i] : static_cast<uint8_t*>(ctx->out.p) + offs[i];
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
    if (b) CK(cudaMemcpyAsync(outs[i], static_cast<uint8_t*>(ctx->out.p) + offs[i], b, cudaMemcpyDeviceToHost, s));
  }
  if (flags & SDIM_FLAG_ASYNC) {
    // the caller keeps the (pinned) host buffers alive until sdim_query / sdim_sync
    ctx->last_stream = s;
    return SDIM_OK;
  }
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->timing_pending = false;
  }
  return read_status(ctx);
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
  std::vector<sdim_circuit> circs(ncirc);
  int rc;
  for (int i = 0; i < ncirc; ++i) {
    op_off[i] = dev.size();
    int nmeas = 0;
    const int64_t r0 = row_begin[i], r1 = row_begin[i + 1];
    if (r1 < r0) return fail(ctx, SDIM_EINVAL, "row offsets must not decrease");
    rc = encode_rows(ctx, rows + 4 * r0, r1 - r0, noise_prob ? noise_prob + r0 : nullptr, n[i], d[i], dev, nmeas);
    if (rc != SDIM_OK) return rc;
    sdim_circuit& c = circs[i];
    c.device = ctx->device;
    c.n = n[i];
    c.d = d[i];
    c.nmeas = nmeas;
    c.nops_user = r1 - r0;
    c.nops = (int)(dev.size() - op_off[i]);
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
  for (int i = 0; i < ncirc; ++i) circs[i].d_ops = base + op_off[i];
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
  if (!on_dev && (rc = ensure(ctx, ctx->out, std::max<size_t>(total, 1))) != SDIM_OK) return rc;
  std::vector<Job> jobs;
  jobs.reserve(ncirc);
  for (int i = 0; i < ncirc; ++i)
    jobs.push_back(Job{&circs[i], seeds[i], shot0[i], nshots[i],
                       on_dev ? outs[i] : static_cast<uint8_t*>(ctx->out.p) + offs[i]});
  rc = launch_jobs(ctx, jobs, s, flags);
  if (rc != SDIM_OK) return rc;
  if (on_dev) return finish(ctx, s, flags);
  if (flags & SDIM_FLAG_TIME) {
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->timing_pending = true;
  }
  for (int i = 0; i < ncirc; ++i) {
    const size_t b = (size_t)nshots[i] * circs[i].nmeas;
    if (b) CK(cudaMemcpyAsync(outs[i], static_cast<uint8_t*>(ctx->out.p) + offs[i], b, cudaMemcpyDeviceToHost, s));
  }
  if (flags & SDIM_FLAG_ASYNC) return SDIM_OK;
  CK(cudaStreamSynchronize(s));
  if (ctx->timing_pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->timing_pending = false;
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
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->timing_pending = false;
  }
  return ctx->status.p ? read_status(ctx) : SDIM_OK;
}

double sdim_last_kernel_ms(const sdim_ctx* ctx) { return ctx ? ctx->last_ms : -1.0; }

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
