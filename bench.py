#!/usr/bin/env python
"""Benchmark: tableau gate-updates/s on the d=2 surface-code memory workload.

Workload (one "step"): rotated distance-7 surface-code memory circuit,
49 data + 48 ancilla qubits, 7 rounds (H on X ancillas, 4-step CNOT schedule,
H, MEASURE+RESET of all ancillas), depolarizing N1 (p = 1e-3) after every gate
on every qudit it touches, final MEASURE of the data; 100,000 shots in one
persistent launch per GPU (bit-plane tableaux in shared memory).  A
gate-update is one circuit instruction (N1, M and RESET included) applied to
one shot's tableau.

Arms:
  default            the GB300 engine (persistent batched kernel); value from
                     CUDA events on the launching stream, e2e through the
                     C ABI with pinned host buffers and copies inside the
                     timed region; plain per-shot form and the CPU oracle on
                     a bounded sample reported beside it.
  --impl reference   the CPU restatement of the reference's algorithm
                     (C oracle, every host core) on a bounded sample per step.

Multi-GPU: replicas -- rank r simulates its own shot range
[r * shots, (r + 1) * shots); no data-path collective (weak scaling).
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
    ap.add_argument("--shots", type=int, default=100_000)
    ap.add_argument("--distance", type=int, default=7)
    ap.add_argument("--rounds", type=int, default=7)
    ap.add_argument("--prob", type=float, default=1e-3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU sample budget")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-shots", type=int, default=256)
    return ap.parse_args()


def workload(args):
    from sdim_gb300 import workloads
    return workloads.surface_memory(args.distance, args.rounds, prob=args.prob)


def config(args, spec, scaling_note):
    return {"workload": f"surface-code memory, rotated distance {args.distance}, {args.rounds} rounds, "
                        f"depolarizing p={args.prob:g} after every gate, d=2",
            "qudits": spec.num_qudits, "dimension": spec.dimension, "instructions": len(spec.ops),
            "shots_per_gpu": args.shots, "records_per_shot": spec.num_measurements(),
            "seed": 0, "l2": "flushed (256 MB write) between timed steps; the flush is outside the events",
            "parallelism": scaling_note}


# ---------------------------------------------------------------------------
# algorithmic bytes per gate-update (residue rows R, phase vector P over 2n)
# ---------------------------------------------------------------------------
def row_bytes(n, d):
    g = 2 * n
    if d == 2:
        return -(-g // 8), 2 * -(-g // 8)
    if d == 3:
        return 2 * -(-g // 8), 2 * -(-g // 8)
    return g, g


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


def algorithmic_bytes_per_shot(enc, det_row, n, d):
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


def cpu_oracle_rate(spec, seconds_budget, seed=0, shot0=0):
    """C oracle on a bounded sample, every host core: (gate-updates/s, shots, s, threads)."""
    import oracle
    threads = os.cpu_count() or 1
    prog = oracle.OracleProgram([spec], spec.num_qudits, spec.dimension)
    t0 = time.perf_counter()
    cal = max(threads, 16)
    oracle.simulate(prog, seed, shot0, cal, threads=threads)
    per_shot = (time.perf_counter() - t0) / cal
    shots = int(max(threads, min(200_000, seconds_budget / max(per_shot, 1e-9))))
    t0 = time.perf_counter()
    oracle.simulate(prog, seed, shot0 + cal, shots, threads=threads)
    dt = time.perf_counter() - t0
    return len(spec.ops) * shots / dt, shots, dt, threads


def run_reference_arm(args):
    ws, rank, _ = dist_setup()
    spec = workload(args)
    if rank != 0:
        return
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_oracle_rate(spec, min(1.0, per_step))
    rates, samples = [], []
    t_all = 0.0
    for k in range(args.steps):
        r, shots, dt, threads = cpu_oracle_rate(spec, per_step, shot0=k * 1_000_000)
        rates.append(r)
        samples.append(shots)
        t_all += dt
    value = statistics.median(rates)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * t_all / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 bit-planes / int64 oracle", "data": "synthetic (seeded)",
            "config": config(args, spec, "host cores, one process"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{statistics.median(samples):.0f} shots per step of the workload "
                                       f"(C restatement of sdim's ExtendedTableau, OpenMP over shots)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_setup()
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from sdim_gb300 import Program, _lib
    from sdim_gb300.encode import DeviceProgram

    spec = workload(args)
    prog = Program(spec.build(), device=local)
    ctx = prog.context
    dp = prog.compile()
    enc = dp.enc
    shots = args.shots
    shot0 = rank * shots
    nrec = dp.num_records
    out = torch.empty((shots, nrec), dtype=torch.uint8, device="cuda")
    # a dedicated stream: the library runs on the stream handle it is given
    # (the legacy default stream has handle 0, which means "context stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def device_step(extra_flags=0):
        rc = ctx.lib.sdim_run_device(ctx.ptr, dp.ptr, 0, shot0, shots, out.data_ptr(), stream.cuda_stream,
                                     _lib.FLAG_ASYNC | _lib.FLAG_TIME | extra_flags)
        _lib.check(rc, ctx.ptr, "run")

    def timed_steps(steps, extra_flags=0, clocks=None):
        step_ms, kern_ms = [], []
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            device_step(extra_flags)
            e1.record(stream)
            ctx.sync()
            step_ms.append(e0.elapsed_time(e1))
            kern_ms.append(ctx.last_kernel_ms())
        torch.cuda.synchronize()
        return step_ms, kern_ms, (clocks.stop() if clocks else None)

    # the per-shot engine (one warp per shot) on the same workload, beside
    for _ in range(2):
        device_step(_lib.FLAG_PER_SHOT)
    ctx.sync()
    ps_steps = max(2, min(args.steps, 3))
    ps_step_ms, ps_kern_ms, _ = timed_steps(ps_steps, _lib.FLAG_PER_SHOT)
    ps_records = out[:64].cpu()

    for _ in range(args.warmup):
        device_step()
    ctx.sync()
    step_ms, kern_ms, clk = timed_steps(args.steps, 0, Clocks(local))
    if ws > 1:
        dist.barrier()
    total_ms = sum(step_ms)
    if ws > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    units_per_step = len(spec.ops) * shots
    value = units_per_step * ws * args.steps / (total_ms / 1e3)
    shots_per_s = shots * ws * args.steps / (total_ms / 1e3)

    # records are bit-identical across engines and runs; det flags are shot independent
    rec = out[:64].cpu().numpy()
    if not np.array_equal(rec, ps_records.numpy()):
        raise AssertionError("shot-group and per-shot engines disagree")
    det_row = (rec[0] >> 7).astype(bool)
    assert np.all((rec >> 7) == (rec[0] >> 7)), "deterministic flags differ across shots"
    n, d = spec.num_qudits, spec.dimension
    bytes_per_shot = algorithmic_bytes_per_shot(enc, det_row, n, d)
    meas_ids = [g for g in enc.ops[:, 0].tolist() if g in (14, 15, 16)]
    reset_cols = [j for j, g in enumerate(meas_ids) if g == 16]
    # RESET records whose outcome needs a correction, per shot (all shots)
    fired = float((out[:, reset_cols] & 0x7F).ne(0).sum().item()) / shots if reset_cols else 0.0
    groups = -(-shots // 32)
    group_bytes = groups * bytes_per_shot + shots * group_delta_bytes_per_shot(enc, det_row, fired, n, d)
    mean_kern = statistics.mean(kern_ms)
    achieved = group_bytes / (mean_kern / 1e3) / 1e9
    ps_kern = statistics.mean(ps_kern_ms)
    ps_achieved = bytes_per_shot * shots / (ps_kern / 1e3) / 1e9
    smem_gbs = C_double_probe(ctx)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    traffic = read_traffic()

    # end to end through the C ABI: pinned host output, instruction stream
    # uploaded and records downloaded inside the timed region
    host = torch.empty((shots, nrec), dtype=torch.uint8, pin_memory=True)
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 0, shot0, shots, host.data_ptr(), 0)
        _lib.check(rc, ctx.ptr, "run")
        if k >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if not torch.equal(host[:64].cuda(), out[:64]):
        raise AssertionError("end-to-end records differ from the device-timed run")
    e2e_total = sum(e2e_ms)
    if ws > 1:
        t = torch.tensor([e2e_total], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = units_per_step * ws * args.steps / (e2e_total / 1e3)

    line = None
    if rank == 0:
        # plain per-shot form (one single-warp launch per shot) on a sample
        pshots = min(args.plain_shots, shots)
        pout = np.empty((pshots, nrec), dtype=np.uint8)
        t0 = time.perf_counter()
        rc = ctx.lib.sdim_run(ctx.ptr, dp.ptr, 0, shot0, pshots, pout.ctypes.data, _lib.FLAG_PLAIN | _lib.FLAG_TIME)
        _lib.check(rc, ctx.ptr, "plain")
        plain_s = time.perf_counter() - t0
        if not np.array_equal(pout[:64], rec[:min(64, pshots)]):
            raise AssertionError("plain form differs from the batched form")
        plain_rate = len(spec.ops) * pshots / plain_s
        cpu = None
        if not args.no_cpu:
            r, cshots, cdt, threads = cpu_oracle_rate(spec, args.cpu_seconds)
            cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"{cshots} shots of the same workload in {cdt:.1f} s (C restatement of sdim's "
                             f"ExtendedTableau + shot loop, OpenMP over shots)"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 bit-planes (exact mod-2 / mod-4 integer)",
            "data": "synthetic (seeded circuit generator, Philox outcome/noise stream)",
            "config": config(args, spec, f"replicas x{ws}: per-GPU shot ranges, no collective"),
            "shots_per_s": shots_per_s,
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(dp.num_device_ops * 8),
                    "d2h_bytes_per_step": int(shots * nrec),
                    "ms_per_step": e2e_total / args.steps},
            "plain_gpu": {"value": plain_rate, "unit": UNIT, "shots": pshots,
                          "form": "one single-warp launch per shot"},
            "batched_vs_plain": value / plain_rate,
            "per_shot_engine": {
                "value": units_per_step * ps_steps / (sum(ps_step_ms) / 1e3), "unit": UNIT,
                "form": "persistent kernel, one warp and one full tableau per shot",
                "kernel_ms": ps_kern,
                "roofline": {"bound": "smem", "achieved": ps_achieved, "peak": smem_gbs, "unit": "GB/s",
                             "frac": ps_achieved / smem_gbs,
                             "algorithmic_bytes_per_shot": bytes_per_shot}},
            "roofline": {"bound": "smem", "achieved": achieved, "peak": smem_gbs, "unit": "GB/s",
                         "frac": achieved / smem_gbs, "traffic": traffic,
                         "kernel": "k_group_persistent<GroupBits>",
                         "peak_source": "shared-memory read bandwidth measured live by sdim_probe_smem_bandwidth",
                         "algorithmic_bytes_per_launch": group_bytes,
                         "bytes_model": "x/z rows + common phase per 32-shot group (per-shot tableau figures), "
                                        "plus each shot's phase-delta rows at measurements and RESET corrections",
                         "per_shot_equivalent_GBps": bytes_per_shot * shots / (mean_kern / 1e3) / 1e9,
                         "hbm_peak_gbs": hbm, "kernel_ms": mean_kern},
            "cpu_baseline": cpu,
            "gpu_launches": args.steps,
            "clocks": clk,
        }
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


def C_double_probe(ctx):  # noqa: N802
    import ctypes
    from sdim_gb300 import _lib
    v = ctypes.c_double()
    _lib.check(ctx.lib.sdim_probe_smem_bandwidth(ctx.ptr, ctypes.byref(v)), ctx.ptr, "smem probe")
    return v.value


def read_traffic():
    """DRAM bytes per launch of the persistent kernel from the committed ncu
    summary (a line 'traffic_bytes_per_launch: <int>'), else None."""
    p = ROOT / "profiles" / "k_group_persistent_bits_surface_L7.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
