#!/usr/bin/env python
"""Benchmark: tableau gate-updates/s of the GB300 tableau engine.

A gate-update is one circuit instruction (N1, M and RESET included) applied
to one shot's tableau; a "step" is one batched run of the whole workload.

Workloads (--workload):
  surface (default)  rotated distance-7 surface-code memory, 97 qubits, 7 rounds
                     (H on X ancillas, 4-step CNOT schedule, H, MEASURE+RESET of
                     the 48 ancillas), depolarizing N1 p=1e-3 after every gate on
                     every qudit it touches, final MEASURE of the 49 data qubits;
                     100,000 shots per step in one persistent launch, d=2.
  pr1                d=3, n=32, 640 gates i.i.d. {H,P,CNOT}, MEASURE all; 1,024 shots.
  oddd5, oddd7       d in {5,7}, n=256, 2,560 gates (H 25%, P 25%, CNOT 50%),
                     MEASURE+RESET on 10% every 256 gates, MEASURE all; 4,096 shots.
  uneven             8,192 programs, n log-uniform in [8,1024], d uniform over
                     {2,3,5,7}, 4n gates {H,P,CNOT} + MEASURE all, shots uniform in
                     [1,64]; one persistent launch per engine variant.

Arms: the default is the GB300 engine (the library's choice: the trace
engines from 128 shots or 160 qudits, shot-group persistent kernels below): `value` from
CUDA events on the launching stream with records in device memory, `e2e`
through the C ABI with pinned host records and the copies inside the timed
region; the other engines, the per-shot engine and the plain form (one
single-warp launch per shot) on the same inputs, and the CPU oracle on a
bounded sample, are reported beside it.  `frame_sampler` times the
reference's other multi-shot route (Pauli frames against a noiseless tableau
shot, `sdim_frame_run`) on the same workload, with its NumPy port on a CPU
sample.  `--impl reference` times the CPU restatement of the reference's
algorithm (the C oracle over every host core) on a bounded sample per step.

Multi-GPU: replicas -- rank r runs the same programs on its own shot range
(shot0 = r * shots), no collective on the data path (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "tableau gate-updates/s"
UNIT = "gate-updates/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="surface",
                    choices=["surface", "pr1", "oddd5", "oddd7", "uneven", "serving"])
    ap.add_argument("--rate", type=float, default=2000.0, help="serving: mean arrivals per second")
    ap.add_argument("--duration", type=float, default=2.0, help="serving: seconds of arrivals")
    ap.add_argument("--n-max", type=int, default=2048, help="serving: largest qudit count")
    ap.add_argument("--shots-max", type=int, default=10_000, help="serving: largest shot count")
    ap.add_argument("--lanes", type=int, default=4, help="serving: batches in flight")
    ap.add_argument("--plain-seconds", type=float, default=1.0,
                    help="serving: arrivals replayed one request at a time for the plain comparison")
    ap.add_argument("--shots", type=int, default=None, help="shots per GPU (single-program workloads)")
    ap.add_argument("--circuits", type=int, default=8192, help="programs of the uneven batch")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU sample budget")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-uneven", action="store_true",
                    help="default workload: leave out the uneven-batch sub-object")
    ap.add_argument("--autotune", action="store_true",
                    help="uneven batch: also time the autotuner's batch-wide routes")
    ap.add_argument("--plain-shots", type=int, default=256)
    ap.add_argument("--per-shot-leg", action="store_true",
                    help="uneven batch: also time the per-shot engine on the whole batch (minutes)")
    ap.add_argument("--quick", action="store_true",
                    help="time the selected engine's step only, no other legs (for profiling runs)")
    ap.add_argument("--engine", default="auto", choices=["auto", "trace", "group", "per_shot"],
                    help="batched engine of the timed run (auto: the library's choice)")
    ap.add_argument("--xz", default="auto", choices=["auto", "packed", "bytes"],
                    help="odd-d trace engine: x/z pass on the packed tableau (bit planes / 4-bit lanes) or on "
                         "residue bytes whatever the batch size (auto: the library's choice)")
    ap.add_argument("--route", default="tableau", choices=["tableau", "frame"],
                    help="with --quick: time the tableau route or the frame route (sdim_frame_run)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def single_workload(args):
    from sdim_gb300 import workloads as W
    if args.workload == "surface":
        spec, shots = W.surface_memory(7, 7, prob=1e-3), 100_000
        desc = ("surface-code memory, rotated distance 7, 7 rounds, depolarizing p=0.001 after every gate, "
                "d=2, 97 qubits")
    elif args.workload == "pr1":
        spec, shots = W.pr1(0), 1024
        desc = "PR1: d=3, n=32, 640 i.i.d. {H,P,CNOT} gates, MEASURE all 32"
    else:
        d = 5 if args.workload == "oddd5" else 7
        spec, shots = W.odd_d(d, seed=0), 4096
        desc = (f"odd d={d}, n=256, 2,560 gates (H 25%, P 25%, CNOT 50%), MEASURE+RESET on 10% every 256 gates, "
                "MEASURE all")
    return spec, (args.shots or shots), desc


def single_config(spec, shots, desc, ws):
    """The config dict of a single-program workload, the same on both arms."""
    return {"workload": desc, "qudits": spec.num_qudits, "dimension": spec.dimension,
            "instructions": len(spec.ops), "shots_per_gpu": shots, "records_per_shot": spec.num_measurements(),
            "seed": 0, "l2": "flushed (256 MB write) between timed steps, outside the events",
            "parallelism": f"replicas x{ws}: per-GPU shot ranges, no collective"}


def uneven_config(items, ws):
    """The config dict of the uneven batch, the same on both arms."""
    ns = np.array([it.spec.num_qudits for it in items])
    return {"workload": f"uneven batch: {len(items)} programs, n log-uniform [8,1024] (median "
                        f"{int(np.median(ns))}), d in {{2,3,5,7}}, 4n gates + MEASURE all, shots 1-64",
            "programs": len(items), "shots_per_gpu": int(sum(it.shots for it in items)),
            "gate_updates_per_step": int(sum(it.shots * len(it.spec.ops) for it in items)),
            "l2": "flushed between timed steps", "parallelism": f"replicas x{ws}"}


def uneven_items(args):
    from sdim_gb300 import workloads as W
    return W.uneven_batch(args.circuits, seed=0)


# ---------------------------------------------------------------------------
# algorithmic bytes (rows R and phase vector P over the 2n generators)
# ---------------------------------------------------------------------------
def row_bytes(n, d):
    g = 2 * n
    if d == 2:
        return -(-g // 8), 2 * -(-g // 8)
    if d == 3:
        return 2 * -(-g // 8), 2 * -(-g // 8)
    return g, g


def algorithmic_bytes_per_shot(enc, det_row, n, d):
    """Bytes one shot's tableau update touches, per instruction type."""
    R, P = row_bytes(n, d)
    h, p, cx, pauli = 4 * R + 2 * P, 3 * R + 2 * P, 6 * R, R + 2 * P
    m_det, m_rand = n * R + P / 2 + R, 2 * (2 * n * R + P)
    total = 0.0
    j = 0
    for gid in enc.ops[:, 0].tolist():
        if gid in (5, 6):
            total += h
        elif gid in (7, 8):
            total += p
        elif gid in (9, 10):
            total += cx
        elif gid in (1, 2, 3, 4, 17):
            total += pauli
        elif gid in (11, 12):
            total += 2 * h + cx
        elif gid == 13:
            total += 3 * cx + 6 * h
        elif gid in (14, 15, 16):
            m = m_det if det_row[j] else m_rand
            if gid == 15:
                m += h
            if gid == 16:
                m += pauli
            total += m
            j += 1
    return total


def group_delta_bytes_per_shot(enc, det_row, resets_fired, n, d):
    """Per-shot phase-delta bytes of the shot-group engine: a random
    measurement reads and writes the delta row (2P), a deterministic one reads
    the stabilizer half (P/2), a RESET whose outcome needs a correction reads
    and writes it (2P).  N1 coins live in registers; fired N1 (rate p) are not
    counted."""
    _, P = row_bytes(n, d)
    total = 0.0
    j = 0
    for gid in enc.ops[:, 0].tolist():
        if gid in (14, 15, 16):
            total += P / 2 if det_row[j] else 2 * P
            j += 1
    return total + 2 * P * resets_fired


def group_bytes(enc, det_row, resets_fired_per_shot, n, d, shots):
    groups = -(-shots // 32)
    return (groups * algorithmic_bytes_per_shot(enc, det_row, n, d)
            + shots * group_delta_bytes_per_shot(enc, det_row, resets_fired_per_shot, n, d))


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax = float(parts[2].split()[0])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# CPU: the C oracle over every host core
# ---------------------------------------------------------------------------
def cpu_rate_single(spec, seconds_budget, seed=0, shot0=0):
    """(gate-updates/s, shots, seconds, threads) on a bounded shot sample."""
    import oracle
    threads = os.cpu_count() or 1
    prog = oracle.OracleProgram([spec], spec.num_qudits, spec.dimension)
    cal = max(threads, 16)
    t0 = time.perf_counter()
    oracle.simulate(prog, seed, shot0, cal, threads=threads)
    per_shot = (time.perf_counter() - t0) / cal
    shots = int(max(threads, min(200_000, seconds_budget / max(per_shot, 1e-9))))
    t0 = time.perf_counter()
    oracle.simulate(prog, seed, shot0 + cal, shots, threads=threads)
    dt = time.perf_counter() - t0
    return len(spec.ops) * shots / dt, shots, dt, threads


def cpu_rate_uneven(items, seconds_budget):
    """C oracle on a systematic sample of the batch, min(shots, 4) shots per program."""
    import oracle
    threads = os.cpu_count() or 1
    units, t_all, used = 0, 0.0, 0
    order = list(range(0, len(items), 97)) + [i for i in range(len(items)) if i % 97]
    for i in order:
        it = items[i]
        prog = oracle.OracleProgram([it.spec], it.spec.num_qudits, it.spec.dimension)
        k = min(it.shots, 4)
        t0 = time.perf_counter()
        oracle.simulate(prog, it.seed, 0, k, threads=threads)
        t_all += time.perf_counter() - t0
        units += len(it.spec.ops) * k
        used += 1
        if t_all > seconds_budget:
            break
    return units / t_all, used, t_all, threads


def run_reference_arm(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    if args.workload == "uneven":
        items = uneven_items(args)
        fn = lambda budget, k: cpu_rate_uneven(items, budget)  # noqa: E731
        cfg = uneven_config(items, ws)
        unit_desc = "programs (systematic sample, min(shots,4) shots each)"
    else:
        spec, shots, desc = single_workload(args)
        fn = lambda budget, k: cpu_rate_single(spec, budget, shot0=k * 1_000_000)  # noqa: E731
        cfg = single_config(spec, shots, desc, ws)
        unit_desc = "shots of the workload"
    for k in range(args.warmup):
        fn(min(1.0, per_step), k)
    rates, samples, t_all, threads = [], [], 0.0, 1
    for k in range(args.steps):
        r, used, dt, threads = fn(per_step, k)
        rates.append(r)
        samples.append(used)
        t_all += dt
    value = statistics.median(rates)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_all / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64 (CPU oracle)",
            "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{statistics.median(samples):.0f} {unit_desc} per step (C restatement "
                                       f"of sdim's ExtendedTableau + shot loop, OpenMP over shots)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
# the library's default switch to the trace engines: from this many shots or
# this many qudits, and for odd d up to this many qudits
TRACE_MIN_SHOTS = 128
TRACE_MIN_QUDITS = 160
TRACE_U8_MAX_QUDITS = 2048


def trace_words(n):
    """Words per trace row of the d = 2 trace engine (0: n too large)."""
    w2 = 2 * ((n + 31) // 32)
    tw = 2
    while tw < w2:
        tw *= 2
    return tw if tw <= 128 else 0


def philox_peak(ctx):
    import ctypes
    from sdim_gb300 import _lib
    v = ctypes.c_double()
    _lib.check(ctx.lib.sdim_probe_philox_rate(ctx.ptr, ctypes.byref(v)), ctx.ptr, "philox probe")
    return v.value


def trace_routed(n, d, shots):
    """Whether the library runs a program on a trace engine (batched form)."""
    if d == 2:
        return trace_words(n) > 0 and (shots >= TRACE_MIN_SHOTS or n >= TRACE_MIN_QUDITS)
    return n <= TRACE_U8_MAX_QUDITS and (shots >= TRACE_MIN_SHOTS or n >= TRACE_MIN_QUDITS)


def u8_single_cta(n, smem_optin):
    """Whether the odd-d x / z pass of n qudits runs on one CTA with its
    tableau in shared memory (else on a CTA pair or from global memory):
    rows of 2n residue bytes padded to an odd word count, 36 rows of shot and
    scratch state, and a 4 KB instruction window."""
    stride = (2 * n + 3) & ~3
    if not (stride >> 2) & 1:
        stride += 4
    npad = (n + 15) & ~15
    hot = ((38 * stride + 2 * npad + 15) & ~15) + 512
    return hot + 2 * n * stride + 4096 + 4096 <= smem_optin


def _split_stride(c):
    s = (c + 3) & ~3
    return s if (s >> 2) & 1 else s + 4


def packed_threads(n, few):
    """Threads of a packed x / z pass CTA (the library's packed_threads)."""
    return 1024 if few and n >= 128 else max(64, min(512, (n + 31) & ~31))


def p3_single_cta(n, smem_optin, threads=512):
    """Whether the d = 3 bit-plane x / z pass of n qudits keeps its tableau in
    one CTA's shared memory: rows of W = 2 ceil(n / 32) plane pairs (8 bytes)
    at an odd stride, a hot part of 3 W + 2 W / 2 + 512 pairs and two n-byte
    columns, and a 4 KB instruction window."""
    wh = (n + 31) // 32
    w = 2 * wh
    r16 = lambda x: (x + 15) & ~15  # noqa: E731
    hot = r16((3 * w + 2 * wh + threads) * 8 + 2 * ((n + 15) & ~15))
    xz = r16(2 * n * (w | 1) * 8)
    return hot + xz + 4096 + 4096 <= smem_optin


def n4_single_cta(n, d, smem_optin, threads=512):
    """Whether the d = 5 / 7 4-bit-lane x / z pass of n qudits keeps its
    tableau in one CTA's shared memory: rows of W = 2 ceil(n / 8) words at an
    odd stride, a hot part of 3 W + W / 2 * 2 + (d - 1) (W + 512) words and two
    n-byte columns, and a 4 KB instruction window."""
    wh = (n + 7) // 8
    w = 2 * wh
    r16 = lambda x: (x + 15) & ~15  # noqa: E731
    hot = r16((3 * w + 2 * wh + (d - 1) * w + (d - 1) * threads) * 4 + 2 * ((n + 15) & ~15))
    xz = r16(2 * n * (w | 1) * 4)
    return hot + xz + 4096 + 4096 <= smem_optin


def u8_xz_layout(n, odd_trace_programs, smem_optin, num_sms=152, d=11):
    """Where the library runs the odd-d x / z pass of n qudits, as (CTAs per
    program, where its columns live: "smem", "l2" or "hbm").  In a batch of
    at least num_sms / 2 odd-d trace programs, and in smaller ones for
    128 <= n while the byte tableau would fit one CTA, d = 3, 5, 7 run on one
    CTA with the packed tableau (bit planes, 4-bit lanes), in shared memory
    when it fits, else streamed from HBM.  Otherwise (other d, smaller batches) one
    CTA when the byte tableau fits in shared memory; else, in a batch of at
    least num_sms / 2, a CTA pair when that fits and one CTA streaming from
    HBM above; in a smaller batch a cluster of 8 CTAs, columns in shared
    memory up to n = 642 and streamed from global memory, held in L2, above."""
    few = 2 * odd_trace_programs < num_sms
    if d in (3, 5, 7) and (not few or (n >= 128 and u8_single_cta(n, smem_optin))):
        th = packed_threads(n, few)
        fits = p3_single_cta(n, smem_optin, th) if d == 3 else n4_single_cta(n, d, smem_optin, th)
        return 1, ("smem" if fits else "hbm")
    if u8_single_cta(n, smem_optin):
        return 1, "smem"
    r16 = lambda x: (x + 15) & ~15  # noqa: E731
    npad, win = (n + 15) & ~15, 4096
    if 2 * odd_trace_programs >= num_sms:
        sl = _split_stride(n)
        pair = r16(2 * n * sl + 2 * sl + 2 * npad) + 4 * sl + 2 * r16(16 + 3 * npad)
        return (2, "smem") if pair + win + 4096 <= smem_optin else (1, "hbm")
    cols = (n + 3) // 4
    sl = _split_stride(cols)
    xchg = 4 * (16 + 2 * npad) + 5 * ((cols + 15) & ~15)
    hot = r16(2 * sl) + 4 * sl + 16 + 2 * r16(xchg)
    return 8, ("smem" if hot + r16(2 * n * sl) + win + 4096 <= smem_optin else "l2")


def xz_kernel_name(mode):
    """The odd-d x / z pass kernel of a sdim_trace_xz_mode form."""
    return {0: "k_trace_pass_u8", 1: "k_trace_pass_split", 2: "k_trace_pass_u8", 3: "k_trace_pass_cluster",
            4: "k_trace_pass_cluster", 5: "k_trace_pass_p3", 6: "k_trace_pass_p3", 7: "k_trace_pass_n4",
            8: "k_trace_pass_n4"}.get(mode, "unknown")


def tableau_place(n, d, on_trace, smem_optin, odd_trace_programs=1, num_sms=152):
    """Where a program's x / z tableau lives ("smem", "l2" or "hbm"): bit
    planes for d = 2 and the odd-d shot-group engine on one CTA, the odd-d
    trace pass as u8_xz_layout places it."""
    if on_trace and d != 2:
        return u8_xz_layout(n, odd_trace_programs, smem_optin, num_sms, d)[1]
    tab = 2 * n * (-(-2 * n // 8) if d == 2 else 2 * n)
    return "smem" if tab <= smem_optin - 16384 else "hbm"


def smem_peak(ctx):
    import ctypes
    from sdim_gb300 import _lib
    v = ctypes.c_double()
    _lib.check(ctx.lib.sdim_probe_smem_bandwidth(ctx.ptr, ctypes.byref(v)), ctx.ptr, "smem probe")
    return v.value


def l2_peak(ctx):
    import ctypes
    from sdim_gb300 import _lib
    v = ctypes.c_double()
    _lib.check(ctx.lib.sdim_probe_l2_bandwidth(ctx.ptr, ctypes.byref(v)), ctx.ptr, "L2 probe")
    return v.value


def read_traffic(name):
    """DRAM bytes per launch of the timed kernel from the committed ncu
    summary (a line 'traffic_bytes_per_launch: <int>'), else None."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


def read_profile_value(name, key):
    """A 'key: <number>' line of a committed ncu summary under profiles/, else None."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def philox_model_peak(num_sms, sm_mhz):
    """Philox4x32-10 blocks/s the integer-multiply pipe allows: 20 wide
    (32 x 32 -> 64-bit) multiplies per block, each taking two of the 64
    32-bit multiply results an SM retires per clock, at the SM clock sampled
    during the timed steps."""
    return num_sms * 64 / (2 * 20) * sm_mhz * 1e6


def hbm_peak():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs", 6800.0)
    except (OSError, ValueError):
        return 6800.0


def hbm_view(traffic, kernel_ms):
    """The step's measured DRAM traffic (ncu, one step) over its CUDA-event
    kernel time, against the measured HBM copy bandwidth: how far the step is
    from being memory-bound.  None without a traffic figure."""
    if not traffic or not kernel_ms or kernel_ms <= 0:
        return None
    peak = hbm_peak()
    gbs = traffic / (kernel_ms / 1e3) / 1e9
    return {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_source": "hbm_gbs of MEASURED_PEAKS.json (fallback 6,800 GB/s)",
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one step under ncu"}


class Timer:
    """Per-step CUDA events on a dedicated stream; L2 flushed between steps."""

    def __init__(self, torch, stream, ctx, ws, dist):
        self.torch, self.stream, self.ctx, self.ws, self.dist = torch, stream, ctx, ws, dist
        self.flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def run(self, steps, step_fn, clocks=None):
        torch = self.torch
        step_ms, kern_ms = [], []
        self.stage_ms, self.pass_ms = [], []
        if self.ws > 1:
            self.dist.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        for _ in range(steps):
            self.flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            step_fn()
            e1.record(self.stream)
            self.ctx.sync()
            step_ms.append(e0.elapsed_time(e1))
            kern_ms.append(self.ctx.last_kernel_ms())
            self.stage_ms.append(self.ctx.last_stage_ms())
            self.pass_ms.append(self.ctx.last_passes_ms())
        torch.cuda.synchronize()
        return step_ms, kern_ms, (clocks.stop() if clocks else None)

    def max_over_ranks(self, value):
        if self.ws == 1:
            return value
        t = self.torch.tensor([value], device="cuda", dtype=self.torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


def graph_replay(args, torch, ctx, timer, stream, entries, units_per_step, expect):
    """The same step captured once as a CUDA graph (sdim_graph_create) and
    replayed over fresh shot ranges: every replay moves each program's
    first shot on by its shot count, as a sampling loop does.  CUDA events
    on the launching stream around each replay, L2 flushed in between; the
    step's records are checked against the ordinary run (``expect``: the
    device output of a replay at the original shot ranges)."""
    from sdim_gb300.graph import CapturedRun
    sizes = [e.shots * e.program.num_records for e in entries]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    gout = torch.empty(int(offs[-1]) + 1, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    run = CapturedRun(ctx, entries, [gout.data_ptr() + int(o) for o in offs[:-1]])
    try:
        info = run.info()

        def moved(k):
            return [e.shot0 + k * e.shots for e in entries]

        for k in range(args.warmup):
            run.launch(shot0=moved(k + 1), stream=stream.cuda_stream)
        run.sync()
        ms = []
        for k in range(args.steps):
            timer.flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run.launch(shot0=moved(args.warmup + 1 + k), stream=stream.cuda_stream)
            e1.record(stream)
            run.sync()
            ms.append(e0.elapsed_time(e1))
        run.launch(shot0=moved(0), stream=stream.cuda_stream)
        run.sync()
        if not np.array_equal(gout[:-1].cpu().numpy(), expect()):
            raise AssertionError("graph replay records differ from the ordinary run")
    finally:
        run.close()
    return {"value": units_per_step * args.steps / (sum(ms) / 1e3), "unit": UNIT,
            "ms_per_step": statistics.mean(ms),
            "form": "the step as one CUDA graph (descriptor upload, queue resets, every kernel on its stream), "
                    "new shot offsets written into its pinned descriptors before each replay",
            "graph_nodes": info["nodes"], "kernel_nodes": info["kernel_nodes"]}


def frame_route(args, torch, ctx, prog, dp, spec, shots, timer):
    """The reference's multi-shot route (Program.simulate(shots) without
    force_tableau): noiseless tableau shot 0, Pauli frames for the rest, on
    the same workload.  Device time by the library's CUDA events, e2e with
    host records, and the NumPy port of the route timed on a CPU sample."""
    from sdim_gb300 import _lib
    ref = prog.compile(False)
    nrec = dp.num_records
    fout = torch.empty((shots, max(nrec, 1)), dtype=torch.uint8, device="cuda")

    def fstep():
        rc = ctx.lib.sdim_frame_run(ctx.ptr, dp.ptr, ref.ptr, 0, shots, fout.data_ptr(),
                                    _lib.FLAG_OUT_DEVICE | _lib.FLAG_TIME)
        _lib.check(rc, ctx.ptr, "frame run")

    for _ in range(args.warmup):
        fstep()
    _, fk, _ = timer.run(args.steps, fstep)
    kms = statistics.mean(fk)
    dev = fout[:, :nrec].cpu().numpy()
    host = torch.empty((shots, max(nrec, 1)), dtype=torch.uint8, pin_memory=True)
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rc = ctx.lib.sdim_frame_run(ctx.ptr, dp.ptr, ref.ptr, 0, shots, host.data_ptr(), 0)
        _lib.check(rc, ctx.ptr, "frame run")
        if k >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if not np.array_equal(host[:, :nrec].numpy(), dev):
        raise AssertionError("frame route: end-to-end records differ from the device-timed run")
    units = len(spec.ops) * shots
    out = {"value": units / (kms / 1e3), "unit": UNIT, "kernel_ms": kms,
           "form": "noiseless tableau shot 0, then one lane per shot carrying x / z frames (k_frame_pass)",
           "e2e": {"value": units * args.steps / (sum(e2e_ms) / 1e3), "unit": UNIT,
                   "ms_per_step": statistics.mean(e2e_ms), "d2h_bytes_per_step": int(shots * nrec)},
           "gpu_launches_per_step": 2}
    if not args.no_cpu:
        import oracle
        from oracle import frame
        oprog = oracle.OracleProgram([spec], spec.num_qudits, spec.dimension)
        sample = 257
        while True:
            t0 = time.perf_counter()
            cpu = frame.simulate(oprog, 0, min(sample, shots), threads=1)
            dt = time.perf_counter() - t0
            if dt > args.cpu_seconds / 4 or sample >= shots:
                break
            sample = min(shots, sample * 4)
        if not np.array_equal(cpu, dev[:cpu.shape[0]]):
            raise AssertionError("frame route: GPU records differ from the NumPy port")
        out["cpu_baseline"] = {"value": len(spec.ops) * cpu.shape[0] / dt, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{cpu.shape[0]} shots in {dt:.1f} s (NumPy port of the reference's "
                                         "frame route, vectorised over shots, one thread)"}
    return out


def run_single(args, torch, dist, ws, rank, local):
    from sdim_gb300 import Program, _lib

    spec, shots, desc = single_workload(args)
    prog = Program(spec.build(), device=local)
    ctx = prog.context
    dp = prog.compile()
    enc = dp.enc
    n, d = spec.num_qudits, spec.dimension
    shot0 = rank * shots
    nrec = dp.num_records
    out = torch.empty((shots, max(nrec, 1)), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()  # the library runs on the handle it is given
    torch.cuda.set_stream(stream)
    timer = Timer(torch, stream, ctx, ws, dist)

    engine_flags = _lib.engine_flags(None if args.engine == "auto" else args.engine)
    engine_flags |= {"auto": 0, "packed": _lib.FLAG_PACKED_XZ, "bytes": _lib.FLAG_U8_XZ}[args.xz]
    trace_used = (d == 2 and trace_words(n) > 0 and
                  (args.engine == "trace" or (args.engine == "auto" and trace_routed(n, d, shots))))
    odd_trace_used = (d != 2 and n <= TRACE_U8_MAX_QUDITS and
                      (args.engine == "trace" or (args.engine == "auto" and trace_routed(n, d, shots))))

    def step(extra=None):
        rc = ctx.lib.sdim_run_device(ctx.ptr, dp.ptr, 0, shot0, shots, out.data_ptr(), stream.cuda_stream,
                                     _lib.FLAG_ASYNC | _lib.FLAG_TIME | (engine_flags if extra is None else extra))
        _lib.check(rc, ctx.ptr, "run")

    if args.quick and args.route == "frame":
        # the frame route alone (profiling runs): shot 0 on the tableau, frames for the rest
        ref = prog.compile(False)

        def fstep():
            rc = ctx.lib.sdim_frame_run(ctx.ptr, dp.ptr, ref.ptr, 0, shots, out.data_ptr(),
                                        _lib.FLAG_OUT_DEVICE | _lib.FLAG_TIME)
            _lib.check(rc, ctx.ptr, "frame run")

        for _ in range(args.warmup):
            fstep()
        _, fk, clk = timer.run(args.steps, fstep, Clocks(local))
        kms = timer.max_over_ranks(statistics.mean(fk))
        return None if rank else {
            "metric": METRIC, "value": len(spec.ops) * shots * ws / (kms / 1e3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": kms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8 residues",
            "data": "synthetic (seeded circuit generator, Philox frame and noise stream)",
            "config": {"workload": desc, "shots_per_gpu": shots, "mode": "quick: frame route only"},
            "route": "frame", "kernel_ms": kms, "gpu_launches": 2 * args.steps, "clocks": clk}
    for _ in range(args.warmup):
        step()
    ctx.sync()
    step_ms, kern_ms, clk = timer.run(args.steps, step, Clocks(local))
    stages = [statistics.mean(v) for v in zip(*timer.stage_ms)]
    passes = [statistics.mean(v) for v in zip(*timer.pass_ms)]
    total_ms = timer.max_over_ranks(sum(step_ms))
    units_per_step = len(spec.ops) * shots
    value = units_per_step * ws * args.steps / (total_ms / 1e3)
    rec = out[:64, :nrec].cpu().numpy()
    if args.quick:
        # the timed engine only (profiling runs): no comparison engines, no CPU leg
        return None if rank else {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 bit planes (d=2) / u8 residues (odd d)",
            "data": "synthetic (seeded circuit generator, Philox outcome and noise stream)",
            "config": {"workload": desc, "shots_per_gpu": shots, "mode": "quick: timed engine only"},
            "engine": args.engine, "kernel_ms": statistics.mean(kern_ms),
            "stages_ms": {"xz_pass": stages[0], "phase_pass": stages[1], "other_engines": stages[2]},
            "passes_ms": {"xz_pass": passes[0], "coin_pass": passes[1], "column_pass": passes[2]},
            "gpu_launches": args.steps, "clocks": clk}

    # per-shot engine (one warp, one full tableau per shot) on the same inputs
    step(_lib.FLAG_PER_SHOT)
    ctx.sync()
    ps_steps = 2
    ps_step_ms, ps_kern_ms, _ = timer.run(ps_steps, lambda: step(_lib.FLAG_PER_SHOT))
    ps_records = out[:64, :nrec].cpu().numpy()
    if not np.array_equal(rec, ps_records):
        raise AssertionError("batched and per-shot engines disagree")
    step()
    ctx.sync()
    full = out[:, :nrec].cpu().numpy()
    engines = {}
    if d == 2:
        # the shot-group engine on the same inputs, for comparison
        for name, fl in (("group", _lib.FLAG_NO_TRACE), ("trace", _lib.FLAG_TRACE),
                         ("trace, phase replay instead of record columns", _lib.FLAG_TRACE | _lib.FLAG_PHASE_REPLAY),
                         ("trace, phase replay, one shot per lane",
                          _lib.FLAG_TRACE | _lib.FLAG_PHASE_REPLAY | _lib.FLAG_LANE_SHOTS_1)):
            step(fl)
            ctx.sync()
            g_ms, g_kern, _ = timer.run(2, lambda: step(fl))
            if not np.array_equal(out[:, :nrec].cpu().numpy(), full):
                raise AssertionError(f"{name} engine disagrees with the timed run")
            engines[name] = {"value": units_per_step * 2 / (sum(g_ms) / 1e3), "unit": UNIT,
                             "kernel_ms": statistics.mean(g_kern),
                             "stages_ms": [statistics.mean(v) for v in zip(*timer.stage_ms)]}
        step()
        ctx.sync()
    warm = None
    if trace_used:
        # a sampling loop over one program: its x / z trace kept on the device
        # (SDIM_FLAG_REUSE_XZ), so each step replays it without the x / z pass.
        # Reported beside the headline step, which runs the x / z pass every time
        keep = engine_flags | _lib.FLAG_REUSE_XZ
        rc = ctx.lib.sdim_run_device(ctx.ptr, dp.ptr, 0, shot0, shots, out.data_ptr(), stream.cuda_stream, keep)
        _lib.check(rc, ctx.ptr, "run")  # synchronous: the kept trace is valid from here on
        warm = {"form": "SDIM_FLAG_REUSE_XZ: the x/z trace written by one synchronous call, then replayed by "
                        "every timed step (same records as the cold step)"}
        for name, fl in (("coin_pass", keep), ("coins_in_phase_pass", keep | _lib.FLAG_NO_COIN_PASS)):
            for _ in range(args.warmup):
                step(fl)
            w_ms, w_kern, _ = timer.run(args.steps, lambda: step(fl))
            if not np.array_equal(out[:, :nrec].cpu().numpy(), full):
                raise AssertionError(f"warm x/z trace ({name}) disagrees with the cold run")
            w_total = timer.max_over_ranks(sum(w_ms))
            warm[name] = {"value": units_per_step * ws * args.steps / (w_total / 1e3), "unit": UNIT,
                          "ms_per_step": w_total / args.steps, "kernel_ms": statistics.mean(w_kern),
                          "gpu_launches_per_step": 1 if fl & _lib.FLAG_NO_COIN_PASS else 2}
        step()
        ctx.sync()
    frames = frame_route(args, torch, ctx, prog, dp, spec, shots, timer) if rank == 0 else None
    graph = None
    if rank == 0:
        from sdim_gb300.batch import BatchEntry
        graph = graph_replay(args, torch, ctx, timer, stream, [BatchEntry(dp, shots, 0, shot0)],
                             len(spec.ops) * shots, lambda: full.reshape(-1))
    det_row = (rec[0] >> 7).astype(bool) if nrec else np.zeros(0, bool)
    assert np.all((rec >> 7) == (rec[0] >> 7)), "deterministic flags differ across shots"
    meas_ids = [g for g in enc.ops[:, 0].tolist() if g in (14, 15, 16)]
    reset_cols = [j for j, g in enumerate(meas_ids) if g == 16]
    if reset_cols:
        fired = float((out[:, reset_cols] & 0x7F).ne(0).sum().item()) / shots
    else:
        fired = 0.0
    gbytes = group_bytes(enc, det_row, fired, n, d, shots)
    per_shot_bytes = algorithmic_bytes_per_shot(enc, det_row, n, d)
    mean_kern = statistics.mean(kern_ms)
    achieved = gbytes / (mean_kern / 1e3) / 1e9
    ps_kern = statistics.mean(ps_kern_ms)
    ps_achieved = per_shot_bytes * shots / (ps_kern / 1e3) / 1e9
    peak = smem_peak(ctx)

    # end to end through the C ABI: pinned host records, instruction stream
    # uploaded and records downloaded inside the timed region
    host = torch.empty((shots, max(nrec, 1)), dtype=torch.uint8, pin_memory=True)
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 0, shot0, shots, host.data_ptr(), 0)
        _lib.check(rc, ctx.ptr, "run")
        if k >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if not np.array_equal(host[:64, :nrec].numpy(), rec):
        raise AssertionError("end-to-end records differ from the device-timed run")
    e2e_total = timer.max_over_ranks(sum(e2e_ms))
    e2e_value = units_per_step * ws * args.steps / (e2e_total / 1e3)
    # the same call with the kernels storing the records into the page-locked
    # host buffer directly
    staged_ms = []
    for k in range(args.warmup + min(args.steps, 5)):
        t0 = time.perf_counter()
        rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 0, shot0, shots, host.data_ptr(), _lib.FLAG_DIRECT_HOST)
        _lib.check(rc, ctx.ptr, "run")
        if k >= args.warmup:
            staged_ms.append((time.perf_counter() - t0) * 1e3)
    if not np.array_equal(host[:, :nrec].numpy(), full):
        raise AssertionError("direct-store end-to-end records differ from the device-timed run")

    if rank != 0:
        return None
    pshots = min(args.plain_shots, shots)
    pout = np.empty((pshots, max(nrec, 1)), dtype=np.uint8)
    t0 = time.perf_counter()
    rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 0, shot0, pshots, pout.ctypes.data, _lib.FLAG_PLAIN)
    _lib.check(rc, ctx.ptr, "plain")
    plain_s = time.perf_counter() - t0
    if not np.array_equal(pout[:64, :nrec], rec[:min(64, pshots)]):
        raise AssertionError("plain form differs from the batched form")
    plain_rate = len(spec.ops) * pshots / plain_s
    cpu = None
    if not args.no_cpu:
        r, cshots, cdt, threads = cpu_rate_single(spec, args.cpu_seconds)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{cshots} shots of the same workload in {cdt:.1f} s (C restatement of sdim's "
                         f"ExtendedTableau + shot loop, OpenMP over shots)"}
    kernel = {2: "k_group_warp<TGroupBits<WarpTeam>>"}.get(d, f"k_group_{'cta' if n >= 160 else 'warp'}"
                                                              f"<TGroupU8<{d}>>")
    if d == 2 and n >= 160:
        kernel = "k_group_cta<TGroupBits<CtaTeam>>"
    group_model = {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                   "kernel": kernel,
                   "peak_source": "shared-memory read bandwidth measured live by sdim_probe_smem_bandwidth",
                   "algorithmic_bytes_per_launch": gbytes,
                   "bytes_model": "x/z rows + common phase once per 32-shot group (per-shot tableau figures), "
                                  "plus each shot's phase-delta rows at measurements and RESET corrections",
                   "per_shot_equivalent_GBps": per_shot_bytes * shots / (mean_kern / 1e3) / 1e9,
                   "hbm_peak_gbs": hbm_peak(), "kernel_ms": mean_kern}
    if trace_used:
        # the step cannot outrun drawing its random numbers: one Philox4x32-10
        # block per 4 N1 ordinals before the last measurement and one per
        # random measurement, per shot
        gids = enc.ops[:, 0]
        meas_at = np.nonzero(np.isin(gids, (14, 15, 16)))[0]
        nn1_used = int((gids[:meas_at[-1]] == 17).sum()) if len(meas_at) else 0
        n_random = int((~det_row).sum())
        blocks = shots * (-(-nn1_used // 4) + n_random)
        coin_blocks = shots * (-(-nn1_used // 32) * 8)
        prate = philox_peak(ctx)
        ach = blocks / (mean_kern / 1e3)
        sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
        model = philox_model_peak(ctx.num_sms, sm_mhz)
        issue_rate = ctx.num_sms * 4 * sm_mhz * 1e6  # warp instructions per second (4 schedulers per SM)
        columns = len(passes) > 2 and passes[2] > 0.0  # record columns ran instead of the phase replay
        last_name = "record_pass" if columns else "phase_pass"
        phase_instr = read_profile_value("trace_engine_surface_L7.md", f"{last_name}_warp_instructions") \
            if args.workload == "surface" else None
        n_meas = int(np.isin(gids, (14, 15, 16)).sum())
        ncols = 1 + n_meas + 2 * nn1_used
        nw = 2
        while 32 * nw < n_meas:
            nw *= 2
        roofline = {"bound": "int-multiply (Philox4x32-10 blocks)", "achieved": ach / 1e9, "peak": prate / 1e9,
                    "unit": "Gblock/s", "frac": ach / prate,
                    "traffic": read_traffic("trace_engine_surface_L7.md") if args.workload == "surface" else None,
                    "kernel": "trace engine step: k_trace_pass (x/z, 1 CTA) alongside k_coin_pass, then " +
                              (f"k_column_pass<{trace_words(n)}> and k_record_pass<{nw}>" if columns else
                               f"k_phase_pass<{trace_words(n)}>"),
                    "peak_source": "Philox throughput measured live by sdim_probe_philox_rate",
                    "algorithmic_blocks_per_launch": blocks,
                    "blocks_model": f"per shot ceil({nn1_used} N1 ordinals / 4) coin blocks + {n_random} "
                                    "random-outcome blocks",
                    "kernel_ms": mean_kern,
                    "stages_ms": {"xz_and_column_passes_beside_coin_pass" if columns else "xz_pass_and_coin_pass":
                                  stages[0], last_name: stages[1]},
                    "peak_cross_check": {
                        "value": model / 1e9, "unit": "Gblock/s", "probe_over_model": prate / model,
                        "model": f"{ctx.num_sms} SMs x 64 32-bit multiplies per clock / (2 per wide multiply x "
                                 "20 wide multiplies per Philox4x32-10 block) x the SM clock sampled in the timed "
                                 "steps",
                        "sm_mhz": sm_mhz},
                    "kernels": {
                        "coin_pass": {
                            "ms": passes[1], "blocks": coin_blocks,
                            "achieved": coin_blocks / (passes[1] / 1e3) / 1e9 if passes[1] else None,
                            "peak": prate / 1e9, "unit": "Gblock/s",
                            "frac": coin_blocks / (passes[1] / 1e3) / prate if passes[1] else None,
                            "timed": "CUDA events around k_coin_pass on its own stream"},
                        "xz_pass": {
                            "ms": passes[0], "measurements": n_meas,
                            "us_per_measurement": 1e3 * passes[0] / max(n_meas, 1),
                            "bound": "latency: one CTA walks the layered schedule; barriers and dependent "
                                     "shared-memory chains per measurement block",
                            "timed": "CUDA events from the step's first kernel to the end of k_trace_pass"},
                        "column_pass": {
                            "ms": passes[2] if columns else None, "columns": ncols, "column_words": nw,
                            "us_per_measurement": 1e3 * passes[2] / max(n_meas, 1) if columns else None,
                            "bound": "latency: each warp walks the measurements from its columns' inputs on, the "
                                     "trace staged in shared memory",
                            "timed": "CUDA events around k_column_pass on the launching stream"} if columns else None,
                        last_name: {
                            "ms": stages[1], "warp_instructions": phase_instr,
                            "issue_bound_ms": (1e3 * phase_instr / issue_rate) if phase_instr else None,
                            "frac": (1e3 * phase_instr / issue_rate / stages[1]) if phase_instr else None,
                            "issue_rate_warp_instr_per_s": issue_rate,
                            "source": "warp instructions of one launch from ncu (smsp__inst_executed.sum, "
                                      "profiles/trace_engine_surface_L7.md); issue rate = SMs x 4 schedulers x "
                                      "the sampled SM clock"}},
                    "group_engine_model": group_model}
        roofline["hbm_view"] = hbm_view(roofline["traffic"], mean_kern)
        roofline["traffic_source"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one step under ncu, read "
                                      "from profiles/trace_engine_surface_L7.md (not measured in this run)")
    else:
        roofline = dict(group_model)
        roofline["traffic"] = None
        if odd_trace_used:
            # the x / z pass updates one tableau per program on one CTA, a CTA
            # pair or a cluster of 8: its algorithmic shared-memory bytes
            # against the share of the measured shared-memory bandwidth of the
            # SMs it runs on
            xz_ms = stages[0]
            sms, _ = u8_xz_layout(n, 1, ctx.smem_optin, ctx.num_sms, d)
            share = peak * sms / ctx.num_sms
            xz_ach = per_shot_bytes / (xz_ms / 1e3) / 1e9
            xz_kernel = xz_kernel_name(ctx.lib.sdim_trace_xz_mode(n, d, 1, 0, ctx.smem_optin, ctx.num_sms))
            roofline = {"bound": f"smem (x/z pass, latency-bound on {sms} CTA{'s' if sms > 1 else ''})",
                        "achieved": xz_ach, "peak": share, "unit": "GB/s", "frac": xz_ach / share,
                        "traffic": read_traffic(f"trace_engine_{args.workload}.md"),
                        "traffic_source": "DRAM bytes of one step under ncu, read from profiles/ (not measured "
                                          "in this run)",
                        "kernel": f"{xz_kernel}<{d}> (x/z pass{', with k_cluster_det_headers after it' if sms == 8 else ''}), "
                                  f"then k_phase_pass_u8<{d}>",
                        "xz_latency": {"ms": xz_ms, "measurements": spec.num_measurements(),
                                       "us_per_measurement": 1e3 * xz_ms / max(spec.num_measurements(), 1),
                                       "bound": "latency: the measurements run one after another, each with its "
                                                "pivot search, barriers and rank-1 update or slice sums; the "
                                                "gates between them are walked in order"},
                        "peak_source": f"sdim_probe_smem_bandwidth x {sms}/{ctx.num_sms} SMs",
                        "algorithmic_bytes_per_launch": per_shot_bytes,
                        "bytes_model": "per-instruction bytes of one tableau update (x/z pass: one tableau per program)",
                        "kernel_ms": xz_ms,
                        "stages_ms": {"xz_pass": stages[0], "phase_pass": stages[1]},
                        "group_engine_model": group_model}
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 bit planes (d=2) / u8 residues (odd d): exact integer mod d",
        "data": "synthetic (seeded circuit generator, Philox outcome and noise stream)",
        "config": single_config(spec, shots, desc, ws),
        "shots_per_s": shots * ws * args.steps / (total_ms / 1e3),
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(dp.num_device_ops * 8),
                "d2h_bytes_per_step": int(shots * nrec), "ms_per_step": e2e_total / args.steps,
                "form": "sdim_run into a page-locked host record buffer: instruction stream copied up, records "
                        "into device memory and copied down (in four chunks behind the record pass when the run "
                        "takes record columns); wall clock per call",
                "direct_host": {"value": units_per_step * len(staged_ms) / (sum(staged_ms) / 1e3), "unit": UNIT,
                                "ms_per_step": statistics.mean(staged_ms),
                                "form": "the same call with SDIM_FLAG_DIRECT_HOST: the kernels store the records "
                                        "into the host buffer directly, no copy"}},
        "plain_gpu": {"value": plain_rate, "unit": UNIT, "shots": pshots, "form": "one single-warp launch per shot"},
        "batched_vs_plain": value / plain_rate,
        "per_shot_engine": {
            "value": units_per_step * ps_steps / (sum(ps_step_ms) / 1e3), "unit": UNIT,
            "form": "persistent kernel, one warp and one full tableau per shot", "kernel_ms": ps_kern,
            "roofline": {"bound": "smem", "achieved": ps_achieved, "peak": peak, "unit": "GB/s",
                         "frac": ps_achieved / peak, "algorithmic_bytes_per_shot": per_shot_bytes}},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "gpu_launches": args.steps * (3 if trace_used else 1),
        "clocks": clk,
        "engine": args.engine,
        "stages_ms": {"xz_pass": stages[0], "phase_pass": stages[1], "other_engines": stages[2]},
        "engines": engines,
        "warm_xz_trace": warm,
        "frame_sampler": frames,
        "graph_replay": graph,
    }


def _leg(name, t0):
    """Wall time of one bench leg, on stderr (the JSON line stays on stdout)."""
    print(f"[bench] {name}: {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)


def plain_uneven(br, entries, budget_s):
    """Plain form (one single-warp launch per shot) on a systematic sample
    of the batch: every 128th program, one shot each, timed by itself.  A
    plain run is one launch sequence per shot, so a program's plain time is
    its one-shot time times its shot count; the rate is the sample's
    gate-updates over that time.  Programs are visited from the smallest
    up and the leg stops once budget_s is spent, so the largest programs of
    the sample may be left out (the count is reported)."""
    from sdim_gb300.batch import BatchEntry, BatchRunner
    sample = sorted(entries[::128], key=lambda e: e.program.num_instructions * e.program.n ** 2)
    units, est_s, spent, used = 0, 0.0, 0.0, 0
    for e in sample:
        one = BatchRunner._view(br.ctx, [BatchEntry(e.program, 1, e.seed, e.shot0)])
        t0 = time.perf_counter()
        one.run(plain=True)
        dt = time.perf_counter() - t0
        spent += dt
        units += e.shots * e.program.num_instructions
        est_s += dt * e.shots
        used += 1
        if spent > budget_s:
            break
    return units / est_s, used, len(sample), spent


def uneven_measure(args, torch, dist, ws, rank, local, sub=False):
    """The uneven batch (8,192 programs by default): device-timed steps, the
    end-to-end run with host records, the plain form on a bounded sample, the
    roofline bound of the batch, and (full run only) the per-shot engine, the
    CPU oracle, the graph replay and the autotuner.  ``sub``: the bounded
    form attached to the default bench line (steps capped, no per-shot
    engine)."""
    from sdim_gb300 import _lib
    from sdim_gb300.batch import BatchRunner

    t_leg = time.perf_counter()
    items = uneven_items(args)
    br = BatchRunner(_lib.Context.default(local))
    ctx = br.ctx
    for it in items:
        br.add_spec(it.spec, it.shots, it.seed, shot0=rank * 64)
    entries = br.entries
    _leg("uneven: generate and encode", t_leg)
    steps = min(args.steps, 10) if sub else args.steps
    warmup = max(3, min(args.warmup, 3)) if sub else args.warmup
    sizes = [e.shots * e.program.num_records for e in entries]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    out = torch.empty(int(offs[-1]) + 1, dtype=torch.uint8, device="cuda")
    ptrs = [out.data_ptr() + int(o) for o in offs[:-1]]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    timer = Timer(torch, stream, ctx, ws, dist)

    def step(extra=0):
        br.run_device(ptrs, stream=stream.cuda_stream, time_kernels=True, asynchronous=True,
                      per_shot=bool(extra & _lib.FLAG_PER_SHOT))

    t_leg = time.perf_counter()
    for _ in range(warmup):
        step()
    ctx.sync()
    step_ms, kern_ms, clk = timer.run(steps, step, Clocks(local))
    total_ms = timer.max_over_ranks(sum(step_ms))
    stages = [statistics.mean(v) for v in zip(*timer.stage_ms)]
    units_per_step = br.total_gate_updates()
    value = units_per_step * ws * steps / (total_ms / 1e3)
    ref_out = out.cpu().numpy()
    _leg(f"uneven: {warmup} warm-up + {steps} timed steps", t_leg)
    if args.quick:
        # the timed step only (profiling runs): no other legs
        if rank != 0:
            return None
        return {"value": value, "unit": UNIT, "steps": steps, "warmup": warmup, "ms_per_step": total_ms / steps,
                "config": dict(uneven_config(items, ws), mode="quick: timed step only"),
                "kernel_ms": statistics.mean(kern_ms),
                "stages_ms": {"xz_pass_and_coin_pass": stages[0], "phase_pass": stages[1],
                              "shot_group_engines_alongside": stages[2]},
                "gpu_launches": steps * len({(e.program.enc.d, e.program.enc.n >= 160) for e in entries}),
                "clocks": clk}

    ps = None
    if not sub and args.per_shot_leg:
        # the per-shot engine on the same batch (minutes: one warp walks each
        # shot's whole tableau, up to 4 MB at n = 1024)
        t_leg = time.perf_counter()
        step(_lib.FLAG_PER_SHOT)
        ctx.sync()
        ps_step_ms, ps_kern_ms, _ = timer.run(1, lambda: step(_lib.FLAG_PER_SHOT))
        if not np.array_equal(out.cpu().numpy(), ref_out):
            raise AssertionError("shot-group and per-shot engines disagree on the uneven batch")
        ps = {"value": units_per_step / (sum(ps_step_ms) / 1e3), "unit": UNIT,
              "kernel_ms": statistics.mean(ps_kern_ms)}
        _leg("uneven: per-shot engine", t_leg)
    graph = None
    if rank == 0 and not sub:
        t_leg = time.perf_counter()
        graph = graph_replay(args, torch, ctx, timer, stream, entries, units_per_step, lambda: ref_out[:-1])
        _leg("uneven: graph replay", t_leg)
    tuned = None
    if rank == 0 and (args.autotune or sub):
        # the autotuner over the batch-wide routes (records checked equal to
        # the default route's; kernel time by the library's CUDA events)
        t_leg = time.perf_counter()
        from sdim_gb300.autotune import Autotuner
        res = Autotuner(ctx, reps=2).tune_batch(br)
        tuned = {"best": res.best.name, "flags": res.best.flags, "kernel_ms": res.times_ms,
                 "aborted_after_one_run": res.aborted,
                 "value": units_per_step / (res.times_ms[res.best.name] / 1e3), "unit": UNIT,
                 "form": "Autotuner.tune_batch: every batch-wide route (trace engines at any shot count, shot groups "
                         "only, CTA-pair / cluster / byte / packed odd-d x/z passes, d = 2 coins in the phase pass, "
                         "one shot per phase-pass lane) timed by the library's CUDA events, median of 2 runs after "
                         "a warm-up, records checked equal to the default route's"}
        _leg("uneven: autotuner", t_leg)

    # algorithmic bytes: det flags per program from its first shot.  The x / z
    # tableau is updated once per program on the trace engines and once per
    # 32-shot group on the shot-group engine; each shot adds its phase-delta
    # bytes.  Tableaux that fit in shared memory are bound by its bandwidth,
    # larger ones stream through HBM: the step cannot beat the sum of both.
    # odd-d trace programs whose columns stream from global memory on CTA
    # clusters (small batches) stay in L2: bound by the measured L2 bandwidth
    peak = smem_peak(ctx)
    hbm = hbm_peak()
    l2 = l2_peak(ctx)
    odd_trace = sum(1 for e in entries if e.program.enc.d != 2 and e.program.enc.n <= TRACE_U8_MAX_QUDITS
                    and trace_routed(e.program.enc.n, e.program.enc.d, e.shots))
    # t_packed: the same bound with the x / z bytes of d = 5, 7 trace programs
    # at the 4-bit lanes their batched x / z pass stores (half of the byte
    # figure the survey's model charges; its d = 3 figure is already two bit
    # planes)
    packed_run = 2 * odd_trace >= ctx.num_sms
    gb, gb_packed, t_min, t_packed, streamed, in_l2 = 0.0, 0.0, 0.0, 0.0, 0.0, 0.0
    for e, o in zip(entries, offs[:-1]):
        enc = e.program.enc
        nr = e.program.num_records
        det_row = (ref_out[int(o):int(o) + nr] >> 7).astype(bool)
        on_trace = trace_routed(enc.n, enc.d, e.shots)
        xz = algorithmic_bytes_per_shot(enc, det_row, enc.n, enc.d) * (1 if on_trace else -(-e.shots // 32))
        delta = e.shots * group_delta_bytes_per_shot(enc, det_row, 0.0, enc.n, enc.d)
        place = tableau_place(enc.n, enc.d, on_trace, ctx.smem_optin, odd_trace, ctx.num_sms)
        bw = {"smem": peak, "l2": l2, "hbm": hbm}[place]
        gb += xz + delta
        t_min += (xz / bw + delta / peak) / 1e9
        xz_p = xz / 2 if (on_trace and packed_run and enc.d in (5, 7)) else xz
        t_packed += (xz_p / bw + delta / peak) / 1e9
        gb_packed += xz_p + delta
        streamed += xz if place == "hbm" else 0.0
        in_l2 += xz if place == "l2" else 0.0
    mean_kern = statistics.mean(kern_ms)

    # end to end: host records (pinned), descriptors up and records down inside
    t_leg = time.perf_counter()
    host = torch.empty(int(offs[-1]) + 1, dtype=torch.uint8, pin_memory=True)
    host_np = host.numpy()
    houts = [host_np[int(a):int(b)].reshape(e.shots, e.program.num_records)
             for a, b, e in zip(offs[:-1], offs[1:], entries)]
    e2e_steps = min(steps, 3) if sub else steps
    e2e_ms = []
    for k in range(warmup + e2e_steps):
        t0 = time.perf_counter()
        br.run(outs=houts)
        if k >= warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if not np.array_equal(host_np[:-1], ref_out[:-1]):
        raise AssertionError("end-to-end records differ")
    e2e_total = timer.max_over_ranks(sum(e2e_ms))
    e2e_value = units_per_step * ws * e2e_steps / (e2e_total / 1e3)
    _leg("uneven: end to end", t_leg)
    if rank != 0:
        return None
    t_leg = time.perf_counter()
    plain_rate, plain_used, plain_sample, plain_s = plain_uneven(br, entries, 15.0 if sub else 60.0)
    _leg("uneven: plain form", t_leg)
    cpu = None
    if not args.no_cpu and not sub:
        t_leg = time.perf_counter()
        r, used, cdt, threads = cpu_rate_uneven(items, args.cpu_seconds)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{used} programs, min(shots,4) shots each, in {cdt:.1f} s (C oracle, OpenMP)"}
        _leg("uneven: CPU oracle", t_leg)
    return {
        "value": value, "unit": UNIT, "steps": steps, "warmup": warmup, "ms_per_step": total_ms / steps,
        "config": uneven_config(items, ws),
        "shots_per_s": br.total_shots() * ws * steps / (total_ms / 1e3),
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "kernel_ms": mean_kern,
        "stages_ms": {"xz_pass_and_coin_pass": stages[0], "phase_pass": stages[1],
                      "shot_group_engines_alongside": stages[2],
                      "note": "the shot-group engines run on their own stream beside the trace engines: their span "
                              "overlaps the other two"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 80 * len(items),
                "d2h_bytes_per_step": int(offs[-1]), "ms_per_step": e2e_total / e2e_steps, "steps": e2e_steps},
        "plain_gpu": {"value": plain_rate, "unit": UNIT, "programs_timed": plain_used,
                      "programs_in_sample": plain_sample, "seconds": plain_s,
                      "form": "one single-warp launch per shot; every 128th program, one shot each timed, "
                              "times its shot count, smallest programs first within a time budget"},
        "batched_vs_plain": value / plain_rate,
        "per_shot_engine": ps,
        "roofline": {"bound": "smem for resident tableaux, L2 for columns streamed by CTA clusters, HBM for "
                              "other streamed tableaux",
                     "achieved": gb_packed / (mean_kern / 1e3) / 1e9, "peak": gb_packed / t_packed / 1e9,
                     "unit": "GB/s", "frac": t_packed * 1e3 / mean_kern, "traffic": None,
                     "kernel": "trace engines (k_trace_pass*, k_phase_pass*) for n >= 160 or 128+ shots, "
                               "k_group_warp / k_group_cta for the rest",
                     "algorithmic_bytes_per_launch": gb_packed, "streamed_bytes": streamed, "l2_bytes": in_l2,
                     "kernel_ms": mean_kern, "bound_ms": t_packed * 1e3, "smem_peak_gbs": peak, "l2_peak_gbs": l2,
                     "hbm_peak_gbs": hbm,
                     "peak_source": "shared-memory read and L2 read+write bandwidth measured live by "
                                    "sdim_probe_smem_bandwidth / sdim_probe_l2_bandwidth; HBM from "
                                    "MEASURED_PEAKS.json",
                     "bytes_model": "x/z tableau updates once per program (trace engines) or per 32-shot group, "
                                    "at the residue width the library stores (bit planes for d = 2, 3; 4-bit lanes "
                                    "for d = 5, 7 in the batched packed x/z pass; bytes otherwise), plus per-shot "
                                    "phase-delta bytes; frac = bound_ms / kernel_ms",
                     "byte_residues": {"bound_ms": t_min * 1e3, "frac": t_min * 1e3 / mean_kern,
                                       "algorithmic_bytes": gb,
                                       "model": "the same bound with d = 5, 7 x/z rows at one byte per residue "
                                                "(the per-gate byte table's figure for d >= 5)"}},
        "cpu_baseline": cpu,
        # one persistent launch per (dimension, team kind) present in the batch
        "gpu_launches": steps * len({(e.program.enc.d, e.program.enc.n >= 160) for e in entries}),
        "clocks": clk,
        "graph_replay": graph,
        "autotune": tuned,
    }


def run_uneven(args, torch, dist, ws, rank, local):
    m = uneven_measure(args, torch, dist, ws, rank, local)
    if m is None:
        return None
    line = {"metric": METRIC, "value": m.pop("value"), "unit": UNIT, "n_gpus": ws, "steps": m.pop("steps"),
            "warmup": m.pop("warmup"), "ms_per_step": m.pop("ms_per_step"), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "u32 bit planes (d=2) / u8 residues (odd d): exact integer mod d",
            "data": "synthetic (seeded generator, Philox outcome stream)"}
    line.update(m)
    return line


def serving_trace(args, seed=0):
    """Poisson arrivals: n log-uniform [16, n_max], d uniform {2,3,5}, 8n
    random {H,P,CNOT} gates + MEASURE all, shots log-uniform [1, shots_max]."""
    from sdim_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(seed))
    trace, t = [], 0.0
    while True:
        t += float(rng.exponential(1.0 / args.rate))
        if t >= args.duration:
            break
        n = int(round(np.exp(rng.uniform(np.log(16), np.log(args.n_max)))))
        d = int((2, 3, 5)[rng.integers(3)])
        shots = max(1, int(round(np.exp(rng.uniform(0.0, np.log(args.shots_max))))))
        table = W.random_hpc_table(n, 8 * n, seed=rng)
        trace.append((t, table, n, d, shots, len(trace)))
    return trace


def run_serving(args, rank, local):
    from sdim_gb300.serving import Server, replay

    trace = serving_trace(args)
    units = sum(s * tb.shape[0] for _, tb, _, _, s, _ in trace)
    # warm-up: compile paths and grow buffers on a few requests
    warm = Server(device=local, lanes=args.lanes)
    replay(warm, [(0.0, *r[1:]) for r in trace[:8]])
    warm.close()
    clocks = Clocks(local)
    clocks.start()
    server = Server(device=local, lanes=args.lanes)
    t0 = time.perf_counter()
    done = replay(server, trace)
    wall = time.perf_counter() - t0
    st = server.stats(done)
    batches = server.batches
    server.close()
    clk = clocks.stop()
    # plain: one request at a time, one lane, the arrivals of the first
    # plain_seconds of the trace (the whole trace one at a time takes minutes)
    ptrace = [r for r in trace if r[0] < args.plain_seconds] or trace[:1]
    punits = sum(s * tb.shape[0] for _, tb, _, _, s, _ in ptrace)
    plain = Server(device=local, lanes=1, max_batch_requests=1)
    tp = time.perf_counter()
    pdone = replay(plain, ptrace)
    pwall = time.perf_counter() - tp
    pst = plain.stats(pdone)
    plain.close()
    if rank != 0:
        return None
    return {
        "metric": METRIC, "value": units / wall, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 bit planes (d=2) / u8 residues (odd d)", "data": "synthetic Poisson trace (seeded)",
        "config": {"workload": f"serving: Poisson {args.rate:g} req/s for {args.duration:g} s, n log-uniform "
                               f"[16,{args.n_max}], d in {{2,3,5}}, 8n gates + MEASURE all, shots log-uniform "
                               f"[1,{args.shots_max}]", "requests": len(trace), "lanes": args.lanes},
        "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"], "mean": st["mean_ms"]},
        "shots_per_s": st["shots_per_s"], "batches": batches,
        "plain_gpu": {"value": punits / pwall, "unit": UNIT, "requests": len(ptrace),
                      "form": f"one request at a time, one lane, the arrivals of the first {args.plain_seconds:g} s",
                      "latency_ms": {"p50": pst["p50_ms"], "p99": pst["p99_ms"]}},
        "batched_vs_plain": (units / wall) / (punits / pwall),
        "e2e": {"value": units / wall, "unit": UNIT, "note": "requests submitted as host op tables, records "
                                                            "returned to host memory"},
        "clocks": clk,
    }


def run_gb300(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_setup()
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    if args.workload == "uneven":
        line = run_uneven(args, torch, dist, ws, rank, local)
    elif args.workload == "serving":
        line = run_serving(args, rank, local)
    else:
        line = run_single(args, torch, dist, ws, rank, local)
        if args.workload == "surface" and not args.quick and not args.no_uneven:
            # the batching target: the uneven batch, bounded, beside the headline
            sub = uneven_measure(args, torch, dist, ws, rank, local, sub=True)
            if line is not None:
                line["uneven"] = sub
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
