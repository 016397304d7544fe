/*
 * sdim_gb300 C ABI: the GB300 stabilizer-tableau engine behind sdim's
 * prime-dimension tableau path.
 *
 * The reference (events555/sdim) is pure Python; its tableau path is the
 * per-shot loop Program._simulate_tableau (sdim/program.py:269-365) driving
 * ExtendedTableau (sdim/tableau/tableau_prime.py:8-380).  These entry points
 * replace that loop: a Python Program (sdim_gb300/program.py) encodes its
 * Circuit objects (sdim/circuit.py:76-126) into the op table below and runs
 * every shot on the GPU.  ctypes is the binding (sdim_gb300/_lib.py).
 *
 * Conventions: plain pointers and sizes only; every call returns 0 or a
 * negative SDIM_E* status and never aborts; sdim_last_error() gives the
 * message.  The library owns all device memory it allocates; the caller owns
 * the buffers it passes in.  A context is not re-entrant (one host thread at
 * a time), like sdim's Program.
 *
 * Records: one byte per measurement (M, M_X or RESET instruction, in program
 * order) per shot: value | deterministic << 7.  The reference returns the
 * same data as MeasurementResult(qudit_index, deterministic,
 * measurement_value) nested [qudit][round][shot] (sdim/program.py:355-365).
 */
#ifndef SDIM_GB300_H
#define SDIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDIM_OK 0
#define SDIM_EINVAL -1     /* bad argument: gate id, qudit index, dimension, size */
#define SDIM_ECUDA -2      /* CUDA runtime error (no device, launch failure, ...) */
#define SDIM_ENOMEM -3     /* device or host allocation failed */
#define SDIM_EDEVICE -4    /* the kernel reported a bad instruction */
#define SDIM_EUNSUPPORTED -5 /* composite dimension or d >= 128 */

/* run flags */
#define SDIM_FLAG_PLAIN 1u       /* one single-warp launch per shot (the plain form) */
#define SDIM_FLAG_OUT_DEVICE 2u  /* output pointers are device pointers */
#define SDIM_FLAG_ASYNC 4u       /* do not synchronise; call sdim_sync() later */
#define SDIM_FLAG_TIME 8u        /* time the kernels with CUDA events (sdim_last_kernel_ms) */
#define SDIM_FLAG_FORCE_GMEM 16u /* keep tableaux in global memory even when they fit in smem */
#define SDIM_FLAG_PER_SHOT 32u   /* batched runs use one warp per shot instead of the shot-group engine */
#define SDIM_FLAG_TEAM_WARP 64u  /* shot groups on one warp each, whatever n */
#define SDIM_FLAG_TEAM_CTA 128u  /* shot groups on one CTA each, whatever n */
#define SDIM_FLAG_TRACE 256u     /* trace engines (one x / z pass per program, then a per-shot phase
                                    replay) whatever the shot count; by default they run from 128
                                    shots or 160 qudits (n up to 2048) */
#define SDIM_FLAG_NO_TRACE 512u  /* no trace engine: shot-group engines only */
#define SDIM_FLAG_NO_COIN_PASS 1024u /* trace engine: draw N1 coins inside the phase pass, no coin pass */
#define SDIM_FLAG_SPLIT_XZ 2048u /* odd-d trace engine: x / z pass on a CTA pair whenever it fits */
#define SDIM_FLAG_CLUSTER_XZ 4096u /* odd-d trace engine: x / z pass on a cluster of 8 CTAs whatever n,
                                      columns in shared memory where they fit (global memory with
                                      SDIM_FLAG_FORCE_GMEM); by default the cluster takes the programs
                                      that do not fit one CTA in batches of fewer than 76 odd-d trace
                                      programs (larger batches use CTA pairs, then single CTAs streaming
                                      from global memory) */
#define SDIM_FLAG_U8_XZ 16384u /* odd-d trace engine: x / z pass on residue bytes (the forms of d >= 11)
                                 instead of the two-bit-plane tableau (d = 3) or 4-bit lanes (d = 5, 7),
                                 which batches of 76+ odd-d trace programs use by default */
#define SDIM_FLAG_PACKED_XZ 131072u /* odd-d trace engine, d = 3, 5, 7: the packed x / z pass (bit planes,
                                       4-bit lanes) also for runs of fewer than 76 odd-d trace programs */
#define SDIM_FLAG_LANE_SHOTS_1 65536u /* d = 2 trace engine: one shot per phase-pass lane (by default two
                                         from 77,824 shots in one launch) */
#define SDIM_FLAG_REUSE_XZ 262144u /* d = 2 trace engine, one program per call: keep the program's x / z
                                      trace on the device (with the sdim_circuit) and, once a synchronous
                                      call with this flag has written it and ended without an error,
                                      replay it in later calls with this flag without running the x / z
                                      pass (the trace depends on the program alone, not on the seed or
                                      the shots).  Calls that use the kept trace must be ordered on the
                                      device after the call that wrote it (one stream, or synchronous
                                      calls); asynchronous calls and graph capture never make it valid */
#define SDIM_FLAG_COLUMNS 524288u /* d = 2 trace engine, one program: record columns whatever the shot
                                     count -- the records as an affine map over GF(2) of each shot's
                                     outcome draws and N1 fires, a column per input computed once from
                                     the trace, then one lane per shot XORing its columns in.  By
                                     default a single program takes them from max(columns, 19,456)
                                     shots, with rows of up to 32 words (n <= 512) and up to 1,024
                                     measurements */
#define SDIM_FLAG_PHASE_REPLAY 1048576u /* d = 2 trace engine: never the record columns (every shot
                                           replays its phase deltas) */
#define SDIM_FLAG_UNLAYERED 2097152u /* odd-d trace engine: the cluster x / z pass applies the gates one at
                                        a time as written (by default it walks the program's layered
                                        stream: gates between measurements in groups on disjoint qudits) */
#define SDIM_FLAG_DIRECT_HOST 8192u /* host outputs in page-locked memory: the kernels store the records
                                       into the host buffer directly, with no device buffer and no copy
                                       (by default records go to device memory, then one copy down) */

/* snapshot modes for sdim_snapshot */
#define SDIM_SNAP_EVERY_INSTRUCTION 1
#define SDIM_SNAP_AT_MEASUREMENT 2
#define SDIM_SNAP_FINAL 3

typedef struct sdim_ctx sdim_ctx;
typedef struct sdim_circuit sdim_circuit;
typedef struct sdim_graph sdim_graph;

/* Context on one CUDA device: stream, device buffers, error string.
 * Replaces the state Program keeps between calls (sdim/program.py:194-204). */
int sdim_ctx_create(int device, sdim_ctx** out);
int sdim_ctx_destroy(sdim_ctx* ctx);
const char* sdim_last_error(const sdim_ctx* ctx);
/* info[0] = SM count, [1] = opt-in shared memory per block (bytes),
 * [2] = L2 bytes, [3] = total global memory (bytes). */
int sdim_device_info(sdim_ctx* ctx, int64_t info[4]);
/* info[0] = free device bytes, [1] = total device bytes, [2] = bytes this
 * context holds in its buffers.  Used by the serving loop's admission. */
int sdim_memory_info(sdim_ctx* ctx, int64_t info[3]);
/* Device bytes a run of nshots shots of circ needs: out[0] records,
 * out[1] one shot-group slot (shared-memory part plus x / z part) plus,
 * for d = 2, the trace the trace engine writes. */
int sdim_program_bytes(const sdim_circuit* circ, int64_t nshots, int64_t out[2]);

/* Encodes one program.  ops is nops rows of 4 int32:
 *   gate id (sdim/gatedata.py:55-102: I 0, X 1, X_INV 2, Z 3, Z_INV 4, H 5,
 *   H_INV 6, P 7, P_INV 8, CNOT 9, CNOT_INV 10, CZ 11, CZ_INV 12, SWAP 13,
 *   M 14, M_X 15, RESET 16, N1 17), qudit, target (-1 for one-qudit gates),
 *   noise channel for N1 (1 'd', 2 'f', 3 'p'; else 0).
 * noise_prob: nops doubles (only N1 rows are read) or NULL when there is no N1.
 * The instruction list replaces Circuit.operations
 * (sdim/circuit.py:6-41, 76-126) and GATE_FUNCTIONS (sdim/program.py:13-32).
 * Errors: SDIM_EINVAL for unknown gates / qudits out of range (the reference
 * raises ValueError / IndexError), SDIM_EUNSUPPORTED for composite d (the
 * reference switches to WeylTableau, sdim/program.py:196-199). */
int sdim_encode_circuit(sdim_ctx* ctx, const int32_t* ops, int64_t nops, const double* noise_prob,
                        int n, int d, sdim_circuit** out);
int sdim_circuit_destroy(sdim_circuit* circ);
/* info[0] n, [1] d, [2] records per shot, [3] user instructions,
 * [4] device ops, [5] backend (0 residue bytes, 1 bit planes), [6] per-shot
 * tableau slot bytes, [7] shot-group slot bytes (0: no group engine for d). */
int sdim_circuit_info(const sdim_circuit* circ, int64_t info[8]);
/* What a d = 2 program keeps on the device for SDIM_FLAG_REUSE_XZ:
 * out[0] 1 when its x / z trace is valid, out[1] 1 when its record columns
 * are.  Host-only. */
int sdim_circuit_kept(const sdim_circuit* circ, int32_t out[2]);

/* Runs shots [shot0, shot0 + nshots) of one program; out holds
 * nshots x records bytes (host memory unless SDIM_FLAG_OUT_DEVICE).  The
 * records go through a device buffer and one copy down; with
 * SDIM_FLAG_DIRECT_HOST a page-locked host buffer (cudaHostAlloc /
 * cudaMallocHost / sdim_host_alloc, or registered with cudaHostRegister) is
 * written by the kernels directly.
 * Replaces Program.simulate(shots, force_tableau=True) (sdim/program.py:206-267, 269-365). */
int sdim_run(sdim_ctx* ctx, const sdim_circuit* circ, uint64_t seed, int64_t shot0, int64_t nshots,
             uint8_t* out, unsigned flags);
/* Same, with the work on a caller-provided CUDA stream (cudaStream_t as void*,
 * NULL for the context's stream) and out on the device. */
int sdim_run_device(sdim_ctx* ctx, const sdim_circuit* circ, uint64_t seed, int64_t shot0,
                    int64_t nshots, uint8_t* out_dev, void* stream, unsigned flags);
/* The reference's multi-shot route, Program.simulate(shots) without
 * record_tableau / force_tableau (sdim/program.py:244-265): row 0 of out is
 * shot 0 of ref (the same program encoded with every N1 as the identity, as
 * the reference's tableau shot treats it, sdim/program.py:31) run on the
 * tableau engines; rows 1 .. nshots-1 propagate Pauli frames of circ against
 * it (simulate_frame, sdim/program.py:45-165) with the noise of circ.  out
 * holds nshots x records bytes (host memory unless SDIM_FLAG_OUT_DEVICE).
 * SDIM_EINVAL when circ and ref differ in n, d or records; SDIM_EUNSUPPORTED
 * when 64 n bytes of frames do not fit in a block's shared memory. */
int sdim_frame_run(sdim_ctx* ctx, const sdim_circuit* circ, const sdim_circuit* ref, uint64_t seed,
                   int64_t nshots, uint8_t* out, unsigned flags);
/* Parses .chp text (the reference's read_circuit, sdim/circuit_io.py:6-83)
 * straight into op-table rows for sdim_encode_circuit / sdim_run_tables:
 * rows gets 4 int32 per instruction (gate id, qudit, target or -1, N1
 * channel), probs (may be NULL) the N1 probability (0 elsewhere).  Needs no
 * context.  With rows NULL it only counts: *nrows, *n (largest qudit index
 * + 1) and *d are set either way.  SDIM_EINVAL (message in err) for a text
 * the reference's reader rejects (no '#' line, malformed parameter, unknown
 * gate, not one or two indices, bad dimension) or when cap < *nrows. */
int sdim_parse_chp(const char* text, int64_t len, int32_t* rows, double* probs, int64_t cap, int64_t* nrows,
                   int32_t* n, int32_t* d, char* err, size_t errlen);
/* Many programs (uneven n, d, depth, shots) in persistent launches fed by a
 * device work queue.  outs[i] holds nshots[i] x records(circs[i]) bytes.
 * The reference has no batch API; it is Program.simulate called once per program. */
int sdim_run_batch(sdim_ctx* ctx, int ncirc, const sdim_circuit* const* circs, const uint64_t* seeds,
                   const int64_t* shot0, const int64_t* nshots, uint8_t* const* outs, void* stream,
                   unsigned flags);
/* A batch run captured once into a CUDA graph and replayed: the whole shot
 * loop of every program (descriptor upload, work-queue resets, the x / z,
 * coin, phase and shot-group kernels on their streams) is one graph launch.
 * Arguments as sdim_run_batch with device outputs; the circuits and the
 * output buffers must outlive the graph.  Creation runs the batch once
 * uncaptured (which writes its records) to size every buffer, then captures
 * it on a private context, so no later call on ctx can move memory that the
 * graph's nodes use.  SDIM_FLAG_PLAIN is refused; TIME and ASYNC are
 * ignored.  Replaces the reference's Python loop over shots
 * (sdim/program.py:206-267, 269-365), which has no graph form. */
int sdim_graph_create(sdim_ctx* ctx, int ncirc, const sdim_circuit* const* circs, const uint64_t* seeds,
                      const int64_t* shot0, const int64_t* nshots, uint8_t* const* outs_dev, unsigned flags,
                      sdim_graph** out);
/* Queues one replay on `stream` (NULL: the graph's own stream).  seeds and
 * shot0 (each NULL or ncirc entries, batch order) replace the seeds and
 * first shot indices of the programs for this and later replays; records
 * equal an sdim_run_batch with the same values.  Replacing them first waits
 * for the previous replay.  Does not wait for the replay itself. */
int sdim_graph_launch(sdim_graph* g, const uint64_t* seeds, const int64_t* shot0, void* stream);
/* Waits for the last replay and reports a device-side error, if any. */
int sdim_graph_sync(sdim_graph* g);
/* info[0] graph nodes, info[1] kernel nodes, info[2] pinned descriptor bytes. */
int sdim_graph_info(const sdim_graph* g, int64_t info[3]);
const char* sdim_graph_last_error(const sdim_graph* g);
int sdim_graph_destroy(sdim_graph* g);
/* Many programs given as op tables, encoded and run in one call: the serving
 * path.  Program i is rows[row_begin[i] .. row_begin[i+1]) (4 int32 per row as
 * in sdim_encode_circuit), noise_prob (may be NULL) is indexed like rows, and
 * n[i], d[i], seeds[i], shot0[i], nshots[i], outs[i] as in sdim_run_batch.
 * The instruction streams go through a pinned staging buffer and a device
 * arena owned by the context, so no device memory is allocated per program;
 * at most one call may be in flight per context.  With SDIM_FLAG_ASYNC and
 * host outputs, the call returns once the work is queued (see sdim_query).
 * No counterpart in the reference (one Program.simulate per request). */
int sdim_run_tables(sdim_ctx* ctx, int ncirc, const int32_t* rows, const int64_t* row_begin,
                    const double* noise_prob, const int32_t* n, const int32_t* d, const uint64_t* seeds,
                    const int64_t* shot0, const int64_t* nshots, uint8_t* const* outs, void* stream,
                    unsigned flags);
/* The form the odd-d trace engine's x / z pass takes for a program of n
 * qudits and odd prime dimension d in a run with odd_trace_programs odd-d
 * trace programs, on a device with smem_optin bytes of opt-in shared memory
 * per block and num_sms SMs: 0 one CTA, byte tableau in shared memory; 1 a
 * CTA pair; 2 one CTA, byte tableau in global memory; 3 a cluster of 8
 * CTAs, columns in shared memory; 4 the cluster, columns in global memory;
 * 5 (d = 3) one CTA, bit-plane tableau in shared memory; 6 (d = 3) one CTA,
 * bit-plane tableau in global memory; 7 (d = 5, 7) one CTA, 4-bit-lane
 * tableau in shared memory; 8 (d = 5, 7) one CTA, 4-bit-lane tableau in
 * global memory (5-8 for runs of 76+ odd-d trace programs on GB300, or with
 * SDIM_FLAG_PACKED_XZ).  Host-only (no device is touched), so
 * callers such as a roofline model can mirror the library's routing.
 * SDIM_EINVAL for n outside [1, 2048], an even d or non-positive sizes.  No
 * counterpart in the reference. */
int sdim_trace_xz_mode(int32_t n, int32_t d, int64_t odd_trace_programs, unsigned flags, int32_t smem_optin,
                       int32_t num_sms);
/* The device instruction words of a program (rows as in
 * sdim_encode_circuit), or with layered != 0 (odd d) the layered stream the
 * cluster x / z pass walks instead: gates between measurements, RESETs and
 * N1 reordered into layers on disjoint qudits, in groups of up to 8 behind
 * {OP_GROUP = 21, count} headers, each run of gates behind {OP_RUN = 22,
 * words}, no group across a 512-word window.  Word k is out[2k] (opcode |
 * qudit << 8) and out[2k + 1] (target or N1 threshold); *count receives the
 * number of words.  Host-only (no device is touched), for inspection and
 * tests.  The codes of sdim_encode_circuit; SDIM_ENOMEM when cap words are
 * too few (*count still set); SDIM_EINVAL for layered with d = 2.  No
 * counterpart in the reference. */
int sdim_program_words(const int32_t* ops, int64_t nops, const double* noise_prob, int32_t n, int32_t d,
                       int32_t layered, uint32_t* out, int64_t cap, int64_t* count);
/* Measured shared-memory read bandwidth of the device in GB/s (all SMs):
 * the roofline denominator for tableaux resident in shared memory.  No
 * counterpart in the reference (which has no device code). */
int sdim_probe_smem_bandwidth(sdim_ctx* ctx, double* gbs);
/* Measured L2 read + write bandwidth in GB/s: every 16-byte word of a 48 MB
 * buffer read and rewritten, 40 passes after two warm-up passes.  The
 * roofline denominator for tableau columns that stream from global memory
 * but stay in L2 (the odd-d trace engine's streamed CTA clusters).  No
 * counterpart in the reference. */
int sdim_probe_l2_bandwidth(sdim_ctx* ctx, double* gbs);
/* Philox4x32-10 blocks per second the device draws at most (eight
 * independent chains per thread, keys per thread, as the trace engine's coin
 * pass draws them): the compute roofline of sampling N1 coins.  No
 * counterpart in the reference. */
int sdim_probe_philox_rate(sdim_ctx* ctx, double* blocks_per_s);
/* Waits for the context's last launch stream and reports a device-side
 * error, if any.  With SDIM_FLAG_ASYNC, sdim_run_batch with host outputs
 * returns after queueing the kernels and the record copies; the host buffers
 * (pinned, e.g. from sdim_host_alloc) must stay alive until sdim_query
 * returns 1 or sdim_sync returns. */
int sdim_sync(sdim_ctx* ctx);
/* 1 when the context's last launch stream is idle, 0 while it runs, < 0 on error. */
int sdim_query(sdim_ctx* ctx);
/* Pinned host memory for asynchronous record copies. */
int sdim_host_alloc(size_t bytes, void** out);
int sdim_host_free(void* p);
/* Milliseconds of the kernels of the last call made with SDIM_FLAG_TIME. */
double sdim_last_kernel_ms(const sdim_ctx* ctx);
/* The same span split by stage: out[0] the trace engine's x / z passes
 * (with the odd-d cluster's deterministic-header pass after them), out[1]
 * its phase passes, out[2] every other engine's kernels.  In a batch
 * that has both, the shot-group engines run on their own stream beside the
 * trace engines: out[2] is then their own span, which overlaps out[0] and
 * out[1].  No counterpart in the reference (its shot loop is not staged). */
int sdim_last_stage_ms(const sdim_ctx* ctx, double out[3]);
/* Two passes of that span timed by themselves: out[0] from the start of the
 * kernels to the end of the last x / z pass (the coin pass runs alongside on
 * another stream), out[1] the d = 2 coin pass alone (0 when none ran).  No
 * counterpart in the reference. */
int sdim_last_pass_ms(const sdim_ctx* ctx, double out[2]);
/* The passes of that span timed by themselves, first n of: [0] from the
 * start of the kernels to the end of the last x / z pass, [1] the d = 2 coin
 * pass, [2] the d = 2 header and column passes (from the end of the x / z
 * pass; 0 without record columns), [3] the shot-group engines when they ran
 * on their own stream beside the trace engines (0 for a pass that did not
 * run).  No counterpart in the reference. */
int sdim_last_passes_ms(const sdim_ctx* ctx, double* out, int n);

/* Tableau export of one shot in the reference's int8 block order
 * x[n][n], z[n][n], phase[n], destab_x[n][n], destab_z[n][n], destab_phase[n]
 * (sdim/tableau/dataclasses.py:8-47, sdim/tableau/tableau_prime.py:8-95), reduced.
 * mode SDIM_SNAP_EVERY_INSTRUCTION: one tableau after each user instruction
 *   (out: user instructions x (4n^2 + 2n) bytes);
 * mode SDIM_SNAP_AT_MEASUREMENT: one tableau right after each measurement,
 *   before a RESET correction, as record_tableau stores it
 *   (sdim/program.py:322-324) (out: records x (4n^2 + 2n) bytes);
 * mode SDIM_SNAP_FINAL: the state after the last instruction, which a
 *   Program holds as stabilizer_tableau after simulate (out: 4n^2 + 2n bytes).
 * records_out (may be NULL) receives that shot's records.  With the default
 * flags the batched engine of the program runs (for d = 2 the shot-group
 * engine, with the shot simulated inside its group of 32); SDIM_FLAG_PER_SHOT
 * runs the per-shot engine. */
int sdim_snapshot(sdim_ctx* ctx, const sdim_circuit* circ, uint64_t seed, int64_t shot, int mode,
                  int8_t* out, uint8_t* records_out, unsigned flags);

/* Allocation-free run, for callers that cannot call cudaMalloc (code living
 * under another framework's allocator, a process whose device memory is
 * already reserved, or a hot path that must not allocate).  No counterpart
 * in the reference.  Takes the same op table as sdim_encode_circuit, runs
 * shots [shot0, shot0 + nshots) with the per-shot engine on the current
 * device and `stream` (NULL: the legacy default stream), writes
 * nshots x records bytes to the device buffer out_dev, and waits for it.
 * It allocates nothing: its scratch (work-queue counter, status word and the
 * device instruction stream) lives in one fixed file-scope device array of
 * 1 MiB + 256 B per device, kept until the process exits.  Limits: at most
 * 131,072 device instructions (CZ and CZ_INV count 3, SWAP 9, M_X 2) and a
 * tableau that fits in shared memory; larger programs return SDIM_EINVAL.
 * The first call on a device looks up the array's address and sets kernel
 * attributes, so make it before any stream capture.  Calls share the array:
 * each clears its counter and status first, and calls that overlap on the
 * GPU race.  Errors are written to err (err_len bytes) when err is not NULL. */
int sdim_run_noalloc(const int32_t* ops, int64_t nops, const double* noise_prob, int n, int d,
                     uint64_t seed, int64_t shot0, int64_t nshots, uint8_t* out_dev, void* stream,
                     char* err, size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* SDIM_GB300_H */
