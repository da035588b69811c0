#!/usr/bin/env python3
"""Benchmark: Glynn steps/s and time-to-exact for per(A), A 32x32 int.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload generic32|generic24|batch4096|float28|schur|schur41|
                                binary40|grid40|rook28|mod3_40|split36] [--no-cpu]

The default workload is generic32 (below); the others print their own
metric line (batched exact permanents, FP64 forward+gradient, Schur
permanents, binary matrices, rook polynomial, permanent mod 3).

One step = one exact evaluation of per(A) for the seeded workload matrix:
the full 2^(n-1) Gray traversal.  `value` is Glynn steps per second toward
the exact result (2^(n-1) sign vectors per evaluation; the exact engine
needs no CRT repetition, so one step is one sign vector evaluated exactly),
measured with CUDA events on the launching stream with the column tables
already resident in HBM and L2 flushed (256 MiB write) between timed steps.
`e2e` is the same metric through the C-ABI call pg_exact_permanent with host
buffers: table upload, launch, copy-back and the host carry, every step.

--impl reference times the reference algorithm on the host cores (the
reference's own OpenMP extension when it was compiled here, else the C
restatement in oracle/) on a bounded sample of Gray states per step, in the
same unit: sample states per second divided by the reference's CRT prime
count for this matrix.

Multi-GPU (torchrun, WORLD_SIZE > 1): every rank evaluates its own seeded
matrix (replicas of the workload; the units are independent matrices), a
barrier brackets the timed region, the max time over ranks is taken and
`value` is the total over ranks ("scaling": "weak").  --workload split36
instead splits ONE permanent across the ranks by Gray range and gathers
the partial words ("scaling": "strong").
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "rivin-perm_gb300"))

WORKLOADS = {
    "generic32": ("one 32x32 int64 matrix, entries U[-8,8], numpy default_rng(32)", 32, 32),
    "generic24": ("one 24x24 int64 matrix, entries U[-8,8], numpy default_rng(0)", 24, 0),
}
METRIC = "Glynn steps/s (exact per(A), n=32 int)"
# DRAM bytes per launch of the exact kernel measured by ncu on these
# workloads (read + write; the tables are KiB-sized, so the kernel is
# compute-bound and the figure only shows that nothing is re-read)
DRAM_BYTES_PER_LAUNCH = {"generic32": 82_688}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_info() -> dict:
    """The CPU model and the C compiler that built the CPU baseline."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                model = line.split(":", 1)[1].strip()
                if line.startswith("Model name"):
                    break
    except (OSError, subprocess.TimeoutExpired):
        pass
    try:
        cc = subprocess.run(["gcc", "--version"], capture_output=True, text=True,
                            timeout=10).stdout.splitlines()[0]
    except (OSError, subprocess.TimeoutExpired, IndexError):
        cc = None
    import platform
    return {"cpu_model": model, "machine": platform.machine(), "compiler": cc,
            "flags": "-O3 -fopenmp"}


def cpu_sample(matrix, seconds_target: float = 12.0):
    """Time the reference's Glynn residue loop on the host cores over a
    bounded prefix of the Gray walk.  Returns (states/s for one prime, cores,
    kind, sample description)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    n = len(matrix)
    p = 1_073_741_827                      # first reference CRT prime >= 2^30
    threads = os.cpu_count() or 1
    kind = "port"      # the timed loop is the oracle's C restatement
    # calibrate on 2^20 states, then size the sample
    lo, hi = 0, 1 << 20
    t = time.perf_counter()
    oracle.glynn_range_mod_p(matrix, p, lo, hi, threads)
    dt = max(time.perf_counter() - t, 1e-6)
    rate = (hi - lo) / dt
    states = int(min(1 << (n - 1), max(1 << 20, rate * seconds_target)))
    t = time.perf_counter()
    oracle.glynn_range_mod_p(matrix, p, 0, states, threads)
    dt = time.perf_counter() - t
    desc = (f"Gray states [0, {states}) of the workload matrix mod p={p}, "
            f"{threads} OpenMP threads (restatement of perm_c_omp.c:556-639)")
    return states / dt, threads, kind, desc


def cpu_batch_sample(mats, seconds_target: float = 15.0):
    """The reference's per-matrix CPU path (oracle port of perm.py:1076-1212:
    bound, primes from 2^30, Glynn residues on all host cores, CRT) over the
    batch's matrices in order until about `seconds_target` have passed.
    Returns (Glynn states/s over the sample, cores, sample description)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    done, states = 0, 0
    t = time.perf_counter()
    for m in mats:
        oracle.exact_permanent(m.tolist(), threads)
        done += 1
        states += 1 << (m.shape[0] - 1)
        if time.perf_counter() - t >= seconds_target:
            break
    dt = time.perf_counter() - t
    return states / dt, threads, (f"the first {done} of the {len(mats)} matrices, exact by CRT "
                                  f"over oracle Glynn residues (all primes from 2^30 up), "
                                  f"{threads} OpenMP threads")


def cpu_f64_sample(mats, seconds_target: float = 15.0):
    """FP64 Glynn with Kahan summation on the host cores (oracle port of
    perm_parallel_cuda.cu:68-209, forward only: the reference has no
    gradient) over the batch's matrices in order until about
    `seconds_target` have passed."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    done, states = 0, 0
    t = time.perf_counter()
    for m in mats:
        oracle.glynn_f64(m, threads)
        done += 1
        states += 1 << (m.shape[0] - 1)
        if time.perf_counter() - t >= seconds_target:
            break
    dt = time.perf_counter() - t
    return states / dt, threads, (f"forward of the first {done} of the {len(mats)} matrices, "
                                  f"{threads} OpenMP threads")


def cpu_binary_sample(matrix, order: int = 32):
    """The reference's 0/1 ratio-table Glynn (oracle port of
    perm_binary_omp.c:236-347) for one prime on the host cores, on the
    leading order x order block of a 40x40 workload matrix (a full 40x40
    residue is 2^39 states, hours on the host)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    sub = np.ascontiguousarray(np.asarray(matrix)[:order, :order], dtype=np.uint8)
    for i in range(order):                         # no empty row or column
        if not sub[i].any():
            sub[i, i] = 1
        if not sub[:, i].any():
            sub[i, i] = 1
    t = time.perf_counter()
    oracle.binary_mod_p(sub, 2_147_483_647, threads)
    dt = time.perf_counter() - t
    return (1 << (order - 1)) / dt, threads, (f"one residue (p = 2^31 - 1) of the leading "
                                              f"{order}x{order} block of matrix 0, {threads} "
                                              f"OpenMP threads")


def run_reference(args, world, rank):
    import numpy as np
    from permgpu import workloads
    if world > 1 and rank != 0:
        return
    if args.workload not in WORKLOADS:
        # the other workloads carry their CPU baseline (the oracle port on the
        # host cores) in the cpu_baseline field of their gb300 line
        print(json.dumps({"impl": "reference", "unavailable":
                          f"the reference arm times the generic workloads "
                          f"({', '.join(sorted(WORKLOADS))}); batch4096, float28, binary40, "
                          f"rook28 and mod3_40 report their CPU baseline in the cpu_baseline "
                          f"field of the gb300 line"}))
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    desc, n, seed = WORKLOADS[args.workload]
    a = workloads.generic_matrix(n, seed)
    k_ref = oracle.reference_prime_count(a.tolist())
    p = 1_073_741_827
    threads = os.cpu_count() or 1
    # per step: a bounded sample of the Gray walk sized to ~3 s
    t = time.perf_counter()
    oracle.glynn_range_mod_p(a, p, 0, 1 << 20, threads)
    rate = (1 << 20) / max(time.perf_counter() - t, 1e-6)
    states = int(min(1 << (n - 1), max(1 << 20, rate * 3.0)))
    for _ in range(args.warmup):
        oracle.glynn_range_mod_p(a, p, 0, 1 << 18, threads)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.glynn_range_mod_p(a, p, 0, states, threads)
        times.append(time.perf_counter() - t)
    per_prime = states / statistics.mean(times)
    value = per_prime / k_ref
    sample = (f"{states} Gray states of the workload matrix mod one reference prime per step, "
              f"x{k_ref} primes for the exact result, {threads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {desc}", "n": n, "crt_primes": k_ref},
        "time_to_exact_s": (1 << (n - 1)) / value,
        # CRT bits per second, K bits(p) 2^(n-1) / t over the K primes of
        # the exact result: bits(p) times one prime's states per second
        "crt_bits_per_s": p.bit_length() * per_prime,
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads,
                         "kind": "port", "sample": sample, "host": host_info()},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args, world, rank, local):
    import numpy as np
    import torch
    from permgpu import _lib, workloads
    from permgpu.crt import matrix_permanent_bound

    if not _lib.cuda_available():
        raise SystemExit("CUDA device not usable: the GPU path has no CPU fallback")
    torch.cuda.set_device(local)
    desc, n, seed = WORKLOADS[args.workload]
    a = workloads.generic_matrix(n, seed + 1000 * rank)
    states = 1 << (n - 1)
    plan = _lib.ExactPlan(a)
    # A dedicated (non-default) stream: the kernel and the CUDA events that
    # time it are recorded on this same stream.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    assert sptr != 0
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    golden = None
    gpath = ROOT / "tests" / "golden" / ("exact_generic32.json" if n == 32 else "exact_generic.json")
    if rank == 0 and gpath.exists():
        g = json.loads(gpath.read_text())
        if n == 32:
            golden = int(g["permanent"])
        else:
            golden = next((int(c["permanent"]) for c in g["cases"] if c.get("workload") == args.workload), None)

    # warm-up (device-resident)
    for _ in range(args.warmup):
        plan.launch(sptr)
    got = plan.result(sptr)
    if golden is not None and got != golden:
        raise SystemExit(f"parity failure: GPU {got} != reference {golden}")

    # IMAD roofline denominators (measured live)
    peak_lo = _lib.probe_int_throughput(0)
    peak_madw = _lib.probe_int_throughput(1)     # mad.wide.u32, 64-bit addend
    peak_mulw = _lib.probe_int_throughput(4)     # mul.wide.u32, no addend

    clocks = ClockSampler(local).start()
    barrier(world)
    torch.cuda.synchronize()
    kernel_ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.launch(sptr)
        e1.record(stream)
        e1.synchronize()
        kernel_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    got = plan.result(sptr)
    if golden is not None and got != golden:
        raise SystemExit(f"parity failure after timing: GPU {got} != reference {golden}")

    # end-to-end through the C ABI with host buffers; the warm-up calls
    # size the one-shot path's reusable device and pinned workspace
    limbs = _lib.exact_limbs(a)
    for _ in range(args.warmup):
        _lib.exact_permanent(a, limbs)
    e2e_s = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        v = _lib.exact_permanent(a, limbs)
        e2e_s.append(time.perf_counter() - t)
        if golden is not None and v != golden:
            raise SystemExit("parity failure in the end-to-end call")
    clk = clocks.stop()

    step_ms = max_over_ranks(world, statistics.mean(kernel_ms))
    e2e_step = max_over_ranks(world, statistics.mean(e2e_s))
    value = world * states / (step_ms * 1e-3)
    e2e_value = world * states / e2e_step
    # roofline: the algorithm's multiplies counted from the kernel source, in
    # mad.lo.u32 equivalents.  With NG product words a term is n - NG 32-bit
    # row-group multiplies (for small-entry matrices two of every three run
    # as exact FP32 multiplies on the FP32 pipe; they are counted all the
    # same), (NG-2)(NG-1)/2 mul.wide.u32 (the running product) and
    # max(NG-1, 1) mad.wide.u32 into the 64-bit columns.  Every 32x32->64
    # product is weighted by the measured mul.wide.u32 : mad.lo.u32 rate
    # ratio (about 2).  The mad.wide probe (64-bit addend) runs slower still
    # in isolation, but inside the kernels splitting it into mul.wide plus an
    # ALU add was slower, so it is counted at the mul.wide weight (the
    # conservative choice: a larger weight would raise the fraction).
    ng = plan.words
    n_mulw = (ng - 2) * (ng - 1) // 2 if ng >= 2 else 0
    n_madw = max(ng - 1, 1)
    w_mulw = peak_lo / peak_mulw
    slots = plan.imul_per_state + (n_mulw + n_madw) * w_mulw
    achieved = states * slots / (statistics.mean(kernel_ms) * 1e-3)
    # the same count restricted to the multiplies that issue on the IMAD
    # pipe: with float rows a group of size sz runs nf - 1 FMULs and sz - nf
    # IMULs (nf = min(FR, sz - 1) float rows), else sz - 1 IMULs
    imul_imad = 0
    for g in range(ng):
        sz = min(plan.group, n - g * plan.group)
        nf = min(plan.float_rows, sz - 1) if plan.float_rows > 0 else 0
        imul_imad += (sz - nf) if nf > 0 else (sz - 1)
    slots_imad = imul_imad + (n_mulw + n_madw) * w_mulw
    achieved_imad = states * slots_imad / (statistics.mean(kernel_ms) * 1e-3)
    # DRAM bytes per launch from one ncu capture of the same launch
    # (dram__bytes_read.sum + dram__bytes_write.sum of exact_glynn_kernel):
    # the column table and the accumulator words only
    traffic = DRAM_BYTES_PER_LAUNCH.get(args.workload)
    NP = (n + 3) & ~3
    h2d = (n - 1) * 2 * NP * 4 + NP * 4
    d2h = (plan.words + (2 if n > 32 else 1)) * 8 + 16

    cpu_rate, cores, kind, sample = (None, None, None, None)
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        k_ref = oracle.reference_prime_count(a.tolist())
        per_prime, cores, kind, sample = cpu_sample(a, args.cpu_seconds)
        cpu_rate = per_prime / k_ref
        sample += f"; exact rate = per-prime rate / {k_ref} reference CRT primes"

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {desc}", "n": n, "states": states,
                       "engine": "exact Glynn (int32 row sums, exact multi-word terms, no CRT)",
                       "group_size": plan.group, "product_words": plan.words,
                       "l2": "flushed between timed steps (256 MiB write); inputs ~4 KiB"},
            "time_to_exact_s": step_ms * 1e-3,
            # the same unit as a CRT walk's K bits(p) 2^(n-1) / t: the bits of
            # the signed range the exact result covers, times states per second
            "result_bits_per_s": (2 * matrix_permanent_bound(a.tolist()) + 1).bit_length() * value,
            "result_checked_against_reference": golden is not None,
            "roofline": {"bound": "imad", "achieved": achieved / 1e12, "peak": peak_lo / 1e12,
                         "unit": "Tops/s", "frac": achieved / peak_lo, "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                           "one captured launch of this workload"
                                           if traffic is not None else None,
                         "frac_imad_pipe_only": achieved_imad / peak_lo,
                         "imad_pipe_slots_per_state": slots_imad,
                         "peak_source": "measured live: pg_probe_int_throughput mad.lo.u32 "
                                        "(no integer peak in MEASURED_PEAKS.json)",
                         "work_per_state": {"imul": plan.imul_per_state,
                                            "mul_wide": n_mulw, "mad_wide": n_madw,
                                            "wide_weight": w_mulw, "slots": slots},
                         "probe_ops_per_s": {"mad.lo.u32": peak_lo, "mul.wide.u32": peak_mulw,
                                             "mad.wide.u32": peak_madw}},
            "cpu_baseline": None if cpu_rate is None else {
                "value": cpu_rate, "unit": "steps/s", "cores": cores, "kind": kind,
                "sample": sample, "host": host_info()},
            "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_step},
            "clocks": clk,
            # per timed step: the walk kernel and the finishing kernel
            "gpu_launches": 2 * args.steps,
        }
        print(json.dumps(line))
    plan.close()


def run_gpu_split(args, world, rank, local):
    """split36: ONE exact permanent (36x36 int64, entries U[-8,8], numpy
    default_rng(36)) split across the ranks by Gray range: each rank walks
    shard.state_range(n, rank, world) on its GPU through pg_exact_partial,
    the partial words are all-gathered (torch.distributed) and every rank
    combines the same exact value.  Total work is fixed as ranks are added
    ("scaling": "strong").  Each step is timed on the host around the whole
    call (table upload, kernel, read-back, exchange, combine), so value and
    e2e coincide."""
    import torch
    from permgpu import _lib, shard, workloads
    torch.cuda.set_device(local)
    n = args.split_order
    a = workloads.generic_matrix(n, n)
    states = 1 << (n - 1)
    lo, hi = shard.state_range(n, rank, world)
    gather = shard.torch_gather if world > 1 else (lambda w: [list(w)])
    for _ in range(args.warmup):
        got = shard.split_exact_permanent(a, rank, world, gather=gather)
    checked = None
    if rank == 0:
        # independent check: per(A) modulo two primes from the residue kernel
        primes = [2_147_483_647, 2_147_483_629]
        if _lib.residues(a, primes) != [got % q for q in primes]:
            raise SystemExit("split36: combined value disagrees with the residue kernel")
        checked = "per(A) mod 2147483647 and 2147483629 from the residue kernel (pg_residues)"
    clocks = ClockSampler(local).start()
    ts = []
    for _ in range(args.steps):
        barrier(world)
        torch.cuda.synchronize()
        t = time.perf_counter()
        v = shard.split_exact_permanent(a, rank, world, gather=gather)
        ts.append(time.perf_counter() - t)
        if v != got:
            raise SystemExit("split36: results changed between steps")
    barrier(world)
    clk = clocks.stop()
    step_s = max_over_ranks(world, statistics.mean(ts))
    if rank == 0:
        print(json.dumps({
            "metric": f"Glynn steps/s (one exact per(A), n={n} int, split by Gray range)",
            "value": states / step_s, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": f"split36: one {n}x{n} int64 matrix, entries U[-8,8], numpy "
                                   f"default_rng({n}); rank r walks Gray states "
                                   f"state_range(n, r, {world})", "states": states,
                       "rank0_range": [lo, hi], "exchange": "torch.distributed all_gather of "
                                                            f"{shard.GATHER_WIDTH} int64 words",
                       "l2": "inputs ~10 KiB; compute-bound"},
            "time_to_exact_s": step_s, "result": str(got),
            "result_checked_against_reference": checked is not None, "result_check": checked,
            "e2e": {"value": states / step_s, "unit": "steps/s",
                    "h2d_bytes_per_step": (n - 1) * 2 * ((n + 3) & ~3) * 4,
                    "d2h_bytes_per_step": 8 * shard.GATHER_WIDTH,
                    "note": "whole call timed on the host (value and e2e coincide)"},
            "clocks": clk, "gpu_launches": 2 * args.steps,     # walk + finishing kernel
        }))


def run_gpu_batch(args, world, rank, local):
    """batch4096: 4096 int64 matrices, n ~ U[12,28], entries U[-3,3], seed 4
    (+rank); value = Glynn states of the whole batch per second through the
    graph-captured persistent launch; compared with per-matrix GPU loops."""
    import torch
    from permgpu import _lib, workloads
    from permgpu.autotune import tuned_parameters
    from permgpu.generic import residue_plan
    from permgpu.crt import matrix_permanent_bound, signed_lift

    torch.cuda.set_device(local)
    mats = workloads.batch4096(seed=4 + 1000 * rank)
    states = sum(1 << (m.shape[0] - 1) for m in mats)
    tune = tuned_parameters(mats)
    plan = _lib.BatchPlan(mats, tune)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        plan.launch(sptr)
    ref = plan.results(sptr)
    clocks = ClockSampler(local).start()
    barrier(world)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.launch(sptr)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    if plan.results(sptr) != ref:
        raise SystemExit("batched results changed between replays")
    # end to end through the C ABI (host buffers in, host results out)
    e2e = []
    for _ in range(max(1, args.steps // 2)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        vals = _lib.batch_exact(mats)
        e2e.append(time.perf_counter() - t)
        if vals != ref:
            raise SystemExit("one-shot batched results differ from the plan")
    clk = clocks.stop()
    # plain per-matrix GPU loops (the same results, one launch per matrix)
    torch.cuda.synchronize()
    t = time.perf_counter()
    loop_exact = [_lib.exact_permanent(m, _lib.exact_limbs(m)) for m in mats]
    t_loop_exact = time.perf_counter() - t
    if loop_exact != ref:
        raise SystemExit("batched results differ from the per-matrix exact path")
    # the reference-style loop: per matrix its CRT primes (one residue launch
    # per matrix, all its primes in it) and the signed lift, every matrix
    t = time.perf_counter()
    sample = mats[: args.residue_loop_sample]
    loop_res = []
    for m in sample:
        bound = matrix_permanent_bound(m.tolist())
        primes = residue_plan(bound)
        loop_res.append(signed_lift(_lib.residues(m, primes), primes, bound))
    t_loop_res = (time.perf_counter() - t) * len(mats) / len(sample)
    if loop_res != ref[:len(sample)]:
        raise SystemExit("batched results differ from the per-matrix residue path")

    step_ms = max_over_ranks(world, statistics.mean(ms))
    value = world * states / (step_ms * 1e-3)
    e2e_s = max_over_ranks(world, statistics.mean(e2e))
    packed, _, _ = _lib.pack_batch(mats)
    cpu = cpu_batch_sample(mats, args.cpu_seconds) if rank == 0 and not args.no_cpu else None
    if rank == 0:
        print(json.dumps({
            "metric": "batched Glynn steps/s (4096 uneven int matrices, exact)", "value": value,
            "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "batch4096: 4096 int64 matrices, n ~ U[12,28], entries U[-3,3], "
                                   "numpy default_rng(4)", "states": states, "tune": list(tune),
                       "tasks": plan.tasks, "blocks": plan.blocks, "graph_captured": True,
                       "l2": "flushed between timed steps (256 MiB write)"},
            "cpu_baseline": None if cpu is None else {
                "value": cpu[0], "unit": "steps/s", "cores": cpu[1], "kind": "port",
                "sample": cpu[2], "est_s_for_batch": states / cpu[0], "host": host_info()},
            "speedup_vs_plain_exact_loop": t_loop_exact / (step_ms * 1e-3),
            "speedup_vs_plain_residue_loop": t_loop_res / (step_ms * 1e-3),
            "plain_exact_loop_s": t_loop_exact, "plain_residue_loop_s": t_loop_res,
            "plain_residue_loop_matrices": len(sample),
            "e2e": {"value": world * states / e2e_s, "unit": "steps/s",
                    "h2d_bytes_per_step": int(packed.nbytes), "d2h_bytes_per_step": len(mats) * plan.limbs * 4,
                    "ms_per_step": 1e3 * e2e_s},
            "clocks": clk, "gpu_launches": args.steps,
        }))
    plan.close()


def exact_dyadic(matrix):
    """(per(A) as a Fraction, row exponents k, exact integer-row matrix):
    every FP64 entry is a dyadic rational, so row i times 2^k_i is an
    integer row and per(A) = per(A_int) / 2^(sum k_i); per(A_int) comes from
    the exact integer path (permgpu.matrix_permanent, residue engine for
    entries beyond the exact engine's widths)."""
    from fractions import Fraction
    import permgpu
    rows, ks = [], []
    for row in matrix:
        fr = [Fraction(float(v)) for v in row]
        k = max(max(f.denominator.bit_length() - 1 for f in fr), 0)
        rows.append([int(f * (1 << k)) for f in fr])
        ks.append(k)
    return Fraction(permgpu.matrix_permanent(rows), 1 << sum(ks)), ks, rows


def run_gpu_float28(args, world, rank, local):
    """float28: 256 float64 matrices 28x28, entries N(0, 1/28), seed 5 (+rank);
    one step = forward + hand-written gradient of the whole batch;
    value = Glynn states per second (256 * 2^27 per step)."""
    import numpy as np
    import torch
    from permgpu import workloads
    from permgpu.f64 import permanent_f64

    torch.cuda.set_device(local)
    A_host = workloads.float28(count=args.batch, seed=5 + 1000 * rank)
    batch, n = A_host.shape[0], A_host.shape[1]
    states = batch * (1 << (n - 1))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    A = torch.from_numpy(A_host).cuda()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        per, grad, s, gs = permanent_f64(A)
    # accuracy against the oracle (forward, 2 matrices; gradient via the
    # row-expansion identity sum_j a_ij g_ij = per for every row)
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    rel = []
    for b in range(2):
        want, _ = oracle.glynn_f64(A_host[b], os.cpu_count() or 1)
        rel.append(abs(per[b].item() - want) / s[b].item())
    g = grad.cpu().numpy()
    # against the EXACT value of the same FP64 inputs (dyadic rationals made
    # integer row by row, exact integer permanents): the forward of sampled
    # matrices and 8 sampled gradient entries of each (the minors, exact),
    # errors relative to the sums of |terms| the kernel returns
    from fractions import Fraction
    import permgpu
    exact_fwd, exact_grad = [], []
    sample = [0, batch - 1] if rank == 0 else []
    pick = np.random.default_rng(28)
    for b in sample:
        want, ks, rows = exact_dyadic(A_host[b])
        exact_fwd.append(abs(Fraction(per[b].item()) - want) / Fraction(s[b].item()))
        for _ in range(8):
            i, j = (int(x) for x in pick.integers(0, n, 2))
            minor = [r[:j] + r[j + 1:] for t, r in enumerate(rows) if t != i]
            gw = Fraction(permgpu.matrix_permanent(minor), 1 << (sum(ks) - ks[i]))
            exact_grad.append(abs(Fraction(float(g[b, i, j])) - gw) /
                              Fraction(gs[b, i].item()))
    # forward-only arm (the same traversal without the gradient columns)
    for _ in range(2):
        permanent_f64(A, want_grad=False)
    torch.cuda.synchronize()
    ms_fwd = []
    for _ in range(max(1, args.steps // 2)):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        permanent_f64(A, want_grad=False)
        e1.record(stream)
        e1.synchronize()
        ms_fwd.append(e0.elapsed_time(e1))
    from permgpu import _lib
    fma32 = _lib.probe_int_throughput(5)        # fma.rn.f32 thread-instructions/s
    fma64 = _lib.probe_int_throughput(6)
    exp_err = max(float(np.max(np.abs((A_host[b] * g[b]).sum(axis=1) - per[b].item())
                               / (np.abs(A_host[b]) * gs[b].cpu().numpy()[:, None]).sum(axis=1)))
                  for b in range(batch))
    clocks = ClockSampler(local).start()
    barrier(world)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        permanent_f64(A)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    e2e = []
    pinned = torch.from_numpy(A_host).pin_memory()
    for _ in range(max(1, args.steps // 2)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        Ad = pinned.cuda(non_blocking=True)
        p, gr, _, _ = permanent_f64(Ad)
        p_host, g_host = p.cpu(), gr.cpu()
        e2e.append(time.perf_counter() - t)
    clk = clocks.stop()
    step_ms = max_over_ranks(world, statistics.mean(ms))
    e2e_s = max_over_ranks(world, statistics.mean(e2e))
    fwd_ms = statistics.mean(ms_fwd)
    cpu = cpu_f64_sample(A_host, args.cpu_seconds) if rank == 0 and not args.no_cpu else None
    # roofline: FP32-pipe instructions of the algorithm per state, counted
    # from the kernel source for the n live rows (lanes): one double-float
    # add per row update (11 FP32 instructions), 5 double-float products in
    # the butterfly for the full product (7 each), one double-float division
    # for the all-but-self product (10 FP32 instructions and a reciprocal),
    # one add for the forward term and 1 + M (M = 4) for the gradient
    # columns; the forward-only walk drops the division and 5 adds
    df_add, df_mul, df_div = 11, 7, 10
    fwd_bwd_ops = n * (df_add * (1 + 1 + 1 + 4) + df_mul * 5 + df_div)
    fwd_ops = n * (df_add * 2 + df_mul * 5)
    achieved = states * fwd_bwd_ops / (step_ms * 1e-3)
    achieved_fwd = states * fwd_ops / (fwd_ms * 1e-3)
    if rank == 0:
        print(json.dumps({
            "metric": "FP64 Glynn forward+gradient steps/s (256 x 28x28)",
            "value": world * states / (step_ms * 1e-3), "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (double-float on FP32 pipes, FP64 re-initialisation and Kahan flushes)",
            "data": "synthetic",
            "config": {"workload": "float28: 256 float64 matrices 28x28, entries N(0,1/28), "
                                   "numpy default_rng(5)", "states": states,
                       "l2": "flushed between timed steps (256 MiB write)"},
            "max_rel_err_forward_vs_oracle": max(rel),
            "max_rel_err_row_expansion": exp_err,
            "max_rel_err_forward_vs_exact": float(max(exact_fwd)),
            "max_rel_err_gradient_vs_exact": float(max(exact_grad)),
            "exact_check": f"matrices {sample} of the batch: forward and 8 gradient entries each "
                           "against exact integer permanents of the row-scaled dyadic inputs; "
                           "errors relative to the kernel's sums of |terms|",
            "tolerance": 1e-10,
            "forward_only_ms": fwd_ms,
            "gradient_cost_ratio": step_ms / fwd_ms,
            "cpu_baseline": None if cpu is None else {
                "value": cpu[0], "unit": "steps/s (forward)", "cores": cpu[1], "kind": "port",
                "sample": cpu[2], "est_s_forward_for_batch": states / cpu[0], "host": host_info()},
            "roofline": {"bound": "fp32 issue", "achieved": achieved / 1e12, "peak": fma32 / 1e12,
                         "unit": "Tops/s", "frac": achieved / fma32, "traffic": None,
                         "peak_source": "measured live: pg_probe_int_throughput fma.rn.f32",
                         "work_per_state": {"fp32_instructions": fwd_bwd_ops,
                                            "forward_only": fwd_ops},
                         "frac_forward_only": achieved_fwd / fma32,
                         "fp64_fma_ops_per_s": fma64},
            "e2e": {"value": world * states / e2e_s, "unit": "steps/s",
                    "h2d_bytes_per_step": int(A_host.nbytes),
                    "d2h_bytes_per_step": int(batch * 8 + A_host.nbytes),
                    "ms_per_step": 1e3 * e2e_s},
            "clocks": clk, "gpu_launches": 2 * args.steps,
        }))


def run_gpu_poly(args, world, rank, local):
    """rook28: exact rook polynomial (matching counts k = 0..28) of a 28x28
    Bernoulli(0.5) 0/1 matrix, numpy default_rng(28 + rank), through
    permgpu.rook_polynomial: the coefficients of per(J + x A) modulo every
    CRT prime (< 2^30) in one launch, CRT, division by (n-k)!.  value =
    prime-states per second of the residue launch (one state = one Gray sign
    vector for one prime: the product of 28 linear factors); e2e = the
    whole rook_polynomial call from host lists to exact integers."""
    import numpy as np
    import torch
    import permgpu
    from permgpu import _lib, poly
    torch.cuda.set_device(local)
    n = 28
    a = (np.random.default_rng(28 + rank).random((n, n)) < 0.5).astype(np.int64)
    ones = np.ones((n, n), dtype=np.int64)
    am = tuple(tuple(int(v) for v in row) for row in a)
    bounds = poly._bounds(tuple((1,) * n for _ in range(n)), am)
    primes = poly._gpu_primes(max(bounds))
    states = len(primes) * (1 << (n - 1))
    # C = J has equal rows, so the uniform kernel runs: per state the
    # elementary-symmetric recurrence (factor r = 1..n-1: r Montgomery
    # products), n - 1 powers of the common row sum and n weighted
    # coefficients, n(n-1)/2 + 2n - 1 Montgomery products of mul.wide,
    # mul.lo and mad.wide each; every 32x32->64 product is weighted by the
    # measured mul.wide : mad.lo ratio
    redc_per_state = n * (n - 1) // 2 + 2 * n - 1
    imad_per_state = 3 * redc_per_state
    for _ in range(args.warmup):
        got = permgpu.rook_polynomial(a.tolist())
        _lib.affine_residues(ones, a, primes)
    if got[1] != int(a.sum()):
        raise SystemExit("rook polynomial failed its r_1 = #ones check")
    peak_lo = _lib.probe_int_throughput(0)
    peak = peak_lo / 1e12                         # mad.lo.u32 ops/s -> Tops/s
    w = peak_lo / _lib.probe_int_throughput(4)    # mul.wide.u32 weight
    slots_per_state = redc_per_state * (2 * w + 1)
    clocks = ClockSampler(local).start()
    barrier(world)
    ts, te = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        _lib.affine_residues(ones, a, primes)
        ts.append(time.perf_counter() - t)
        t = time.perf_counter()
        res = permgpu.rook_polynomial(a.tolist())
        te.append(time.perf_counter() - t)
        if res != got:
            raise SystemExit("results changed between steps")
    barrier(world)
    clk = clocks.stop()
    step_s = max_over_ranks(world, statistics.mean(ts))
    e2e_s = max_over_ranks(world, statistics.mean(te))
    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        oracle.affine_range_mod_p(ones, a, primes[0], 0, 1 << 14, threads)
        rate = (1 << 14) / max(time.perf_counter() - t, 1e-6)
        sample = int(min(1 << (n - 1), max(1 << 14, rate * args.cpu_seconds)))
        t = time.perf_counter()
        oracle.affine_range_mod_p(ones, a, primes[0], 0, sample, threads)
        per_prime = sample / (time.perf_counter() - t)
        cpu = {"value": per_prime, "unit": "prime-states/s", "cores": threads, "kind": "port",
               "sample": f"Gray states [0, {sample}) of per(J + xA) for the workload matrix mod "
                         f"one prime, {threads} OpenMP threads (restatement of "
                         f"perm_polynomial.py:268-329); the exact vector needs "
                         f"{len(primes)} primes x 2^{n - 1} states",
               "time_to_exact_s_est": states / per_prime}
    if rank == 0:
        achieved = states * slots_per_state / step_s / 1e12
        print(json.dumps({
            "metric": "polynomial Glynn prime-states/s (rook28)", "value": world * states / step_s,
            "unit": "prime-states/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 Montgomery",
            "data": "synthetic",
            "config": {"workload": "rook28: rook polynomial of a 28x28 Bernoulli(0.5) 0/1 "
                                   "matrix, numpy default_rng(28)", "crt_primes": len(primes),
                       "states": states},
            "time_to_exact_s": e2e_s, "results_r1_rn": [str(got[1]), str(got[-1])],
            "roofline": {"bound": "imad", "achieved": achieved, "peak": peak, "unit": "Tops/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_source": "measured live: pg_probe_int_throughput mad.lo.u32",
                         "work_per_state": {"imad_class_instructions": imad_per_state,
                                            "wide_weight": w, "slots": slots_per_state}},
            "cpu_baseline": cpu,
            "e2e": {"value": world * states / e2e_s, "unit": "prime-states/s",
                    "h2d_bytes_per_step": 2 * 8 * n * n, "d2h_bytes_per_step": 8 * (n + 1) * len(primes),
                    "ms_per_step": 1e3 * e2e_s},
            "clocks": clk, "gpu_launches": 2 * args.steps,
        }))


def run_gpu_mod3(args, world, rank, local):
    """mod3_40: per(A) mod 3 of a 40x40 matrix with entries U{0,1,2}, numpy
    default_rng(40 + rank), through permgpu.mod3.permanent_mod3_fast (Ryser
    over F_3 with bit-sliced row sums, one launch).  value = subsets per
    second (2^40 per evaluation); the call is timed from the host matrix to
    the returned residue, so value and e2e coincide."""
    import numpy as np
    import torch
    from permgpu import _lib, mod3
    torch.cuda.set_device(local)
    n = args.mod3_order
    a = np.random.default_rng(n + rank).integers(0, 3, (n, n)).astype(np.int64)
    states = 1 << n
    for _ in range(args.warmup):
        got = mod3.permanent_mod3_fast(a)
    clocks = ClockSampler(local).start()
    barrier(world)
    ts = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = mod3.permanent_mod3_fast(a)
        ts.append(time.perf_counter() - t)
        if res != got:
            raise SystemExit("results changed between steps")
    barrier(world)
    clk = clocks.stop()
    step_s = max_over_ranks(world, statistics.mean(ts))
    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        oracle.mod3_range(a, 0, 1 << 24, threads)
        rate = (1 << 24) / max(time.perf_counter() - t, 1e-6)
        sample = int(min(states, max(1 << 24, rate * args.cpu_seconds)))
        t = time.perf_counter()
        oracle.mod3_range(a, 0, sample, threads)
        cpu_rate = sample / (time.perf_counter() - t)
        cpu = {"value": cpu_rate, "unit": "subsets/s", "cores": threads, "kind": "port",
               "sample": f"Gray subsets [0, {sample}) of the workload matrix, {threads} OpenMP "
                         "threads (bit-sliced F_3 Ryser, restatement of perm_mod3_omp.c:54-160)",
               "time_to_result_s_est": states / cpu_rate}
    if rank == 0:
        # per subset: one 64-bit column update (3 three-input bitwise ops on
        # two words), the full-magnitude test and a popcount
        print(json.dumps({
            "metric": f"Ryser subsets/s (perm mod 3, {n}x{n})", "value": world * states / step_s,
            "unit": "subsets/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "F_3 bit-sliced (u64 words)", "data": "synthetic",
            "config": {"workload": f"mod3_40: {n}x{n} matrix, entries U{{0,1,2}}, numpy "
                                   f"default_rng({n})", "subsets": states},
            "time_to_result_s": step_s, "result": got, "cpu_baseline": cpu,
            "e2e": {"value": world * states / step_s, "unit": "subsets/s",
                    "h2d_bytes_per_step": 2 * 8 * n, "d2h_bytes_per_step": 16,
                    "note": "whole-call API timed end to end"},
            "clocks": clk, "gpu_launches": args.steps,
        }))


def necklace_representatives(length: int) -> int:
    """Orbits of {0,1}^length under rotation and complement (Burnside)."""
    phi = lambda d: sum(1 for k in range(1, d + 1) if math.gcd(k, d) == 1)
    divisors = [d for d in range(1, length + 1) if length % d == 0]
    rot = sum(phi(d) * 2 ** (length // d) for d in divisors)
    comp = sum(phi(d) * 2 ** (length // d) for d in divisors if d % 2 == 0)
    return (rot + comp) // (2 * length)


def run_gpu_exact_set(args, world, rank, local):
    """schur: exact perm(S_31) and perm(S_33) (residue engine, primes == 1 mod
    n, below 2^31, Graham-Lehmer congruence at CRT time); binary40: eight
    40x40 Bernoulli(0.5) 0/1 matrices (seeds 300..307) through the binary
    API (matching blocks, exact engine).  One step = the whole set; value =
    Glynn steps per second (minor / block states, times primes for Schur)."""
    import numpy as np
    import torch
    import permgpu
    from permgpu import workloads
    from permgpu.crt import plan_schur
    torch.cuda.set_device(local)
    table = json.loads((ROOT / "tests" / "golden" / "schur.json").read_text())["table"]
    if args.workload == "schur":
        items = [31, 33]
        states = sum(len(plan_schur(n)[0]) * (1 << (n - 2)) for n in items)

        def step():
            return [permgpu.permanent(n) for n in items]
        want = [int(table[str(n)]) for n in items]
        desc = "perm(S_31), perm(S_33): (n-1)x(n-1) minors, primes == 1 (mod n) < 2^31"
    elif args.workload == "schur41":
        # prime order (41 unless --order says otherwise): the (n-1)x(n-1)
        # circulant minor through the necklace quotient; "states" counts the
        # rotation+complement orbits (times primes)
        n = args.order
        items = [n]
        states = len(plan_schur(n)[0]) * necklace_representatives(n - 1)

        def step():
            return [permgpu.permanent(n) for n in items]
        want = [int(table[str(n)])]
        desc = (f"perm(S_{n}): {n - 1}x{n - 1} circulant cofactor minor, rotation+complement "
                f"necklace orbits, primes == 1 (mod {n}) < 2^30")
    elif args.workload == "grid40":
        # the reference's showcase binary matrix: biadjacency of the 4x4x5
        # grid graph, periodic in two axes (tests/golden/binary.json)
        g = json.loads((ROOT / "tests" / "golden" / "binary.json").read_text())
        grid = g["grid_4x4x5_periodic01"]
        items = [grid["matrix"]]
        states = 1 << 39

        def step():
            return [permgpu.binary_permanent(m) for m in items]
        want = [int(grid["permanent"])]
        desc = "40x40 biadjacency of the 4x4x5 grid, periodic in axes 0 and 1"
    else:
        mats = workloads.binary40(8)
        items = [m.tolist() for m in mats]
        states = len(items) * (1 << 39)

        def step():
            return [permgpu.binary_permanent(m) for m in items]
        want = None
        desc = "eight 40x40 Bernoulli(0.5) 0/1 matrices, numpy default_rng(300..307)"
    for _ in range(args.warmup):
        got = step()
    if want is not None and got != want:
        raise SystemExit(f"parity failure: {got} != {want}")
    check_method = "published/golden values" if want is not None else None
    if args.workload == "binary40":
        # no published values: every exact result is checked modulo two
        # primes against pg_binary_residues, an independent full traversal
        # pinned to the reference's binary_permanent_mod_p
        from permgpu import _lib
        check_primes = [2_147_483_647, 2_147_483_629]
        for m, v in zip(mats, got):
            if _lib.binary_residues(m, check_primes) != [v % q for q in check_primes]:
                raise SystemExit("binary40: exact result disagrees with the residue kernel")
        check_method = ("each result mod 2147483647 and 2147483629 equals pg_binary_residues "
                        "(independent 2^39-state residue walk, pinned to the reference's "
                        "binary_permanent_mod_p)")
    clocks = ClockSampler(local).start()
    barrier(world)
    ts = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = step()
        ts.append(time.perf_counter() - t)
        if res != got:
            raise SystemExit("results changed between steps")
    barrier(world)
    clk = clocks.stop()
    step_s = max_over_ranks(world, statistics.mean(ts))
    cpu = None
    if rank == 0 and args.workload == "binary40" and not args.no_cpu:
        rate, cores, sample = cpu_binary_sample(mats[0])
        from permgpu import binary
        from permgpu.crt import binary_primes_above
        k = [len(binary_primes_above(binary.binary_permanent_bound(m.tolist()))) for m in mats]
        cpu = {"value": rate, "unit": "steps/s (one prime)", "cores": cores, "kind": "port",
               "sample": sample,
               "est_s_for_set": sum(kk * (1 << 39) for kk in k) / rate,
               "estimate": f"{sum(k)} residues of 2^39 states at the sampled rate",
               "host": host_info()}
    if rank == 0 and args.workload == "schur41":
        n = args.order
        # published: perm(S_41) by the reference's CUDA necklace kernel in
        # 47.39 s on a GH200 (README.md:596)
        published = 47.39 if n == 41 else None
        print(json.dumps({
            "metric": f"seconds to exact perm(S_{n})", "value": step_s, "unit": "s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * step_s, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": step_s / published if published else None,
            "dtype": "int32", "data": f"none (the matrix is S_{n})",
            "config": {"workload": f"{args.workload}: {desc}", "orbits": states},
            "orbits_per_s": states / step_s, "results": [str(v) for v in got],
            "result_checked_against_reference": True,
            "e2e": {"value": step_s, "unit": "s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None,
                    "note": f"whole-call API permgpu.permanent({n}) timed end to end"},
            "clocks": clk, "gpu_launches": args.steps,
        }))
    elif rank == 0 and args.workload == "grid40":
        # published: the reference's CUDA binary kernel, two residues plus
        # CRT, 22.73 s end to end on a GH200 (BINARY_APPLICATIONS.md:165-171)
        print(json.dumps({
            "metric": "seconds to exact per(grid 4x4x5, 40x40 0/1)", "value": step_s,
            "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * step_s, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": step_s / 22.73, "dtype": "int32",
            "data": "none (the matrix is the grid biadjacency)",
            "config": {"workload": f"{args.workload}: {desc}", "states": states},
            "steps_per_s": states / step_s, "results": [str(v) for v in got],
            "result_checked_against_reference": True,
            "e2e": {"value": step_s, "unit": "s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None,
                    "note": "whole-call API permgpu.binary_permanent timed end to end"},
            "clocks": clk, "gpu_launches": 2 * args.steps,     # 0/1 walk + finishing kernel
        }))
    elif rank == 0:
        print(json.dumps({
            "metric": f"Glynn steps/s ({args.workload})", "value": world * states / step_s,
            "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {desc}", "states": states},
            "time_to_exact_s": step_s, "results": [str(v) for v in got],
            "result_checked_against_reference": check_method is not None,
            "result_check": check_method,
            "cpu_baseline": cpu,
            "e2e": {"value": world * states / step_s, "unit": "steps/s",
                    "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                    "note": "whole-call API timed end to end (host inputs, host results)"},
            "clocks": clk,
            # binary40: per matrix and step a 0/1 walk and a finishing kernel
            "gpu_launches": 2 * len(got) * args.steps if args.workload == "binary40" else None,
        }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="generic32",
                    choices=sorted(WORKLOADS) + ["batch4096", "float28", "schur", "schur41",
                                                 "binary40", "grid40", "rook28", "mod3_40",
                                                 "split36"])
    ap.add_argument("--residue-loop-sample", type=int, default=4096,
                    help="batch4096: matrices in the timed per-matrix residue loop (all by default)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--batch", type=int, default=256,
                    help="float28: matrices per step (256 is the workload; smaller for profiling)")
    ap.add_argument("--order", type=int, default=41,
                    help="schur41: prime Schur order (41 is the workload; 37 for profiling)")
    ap.add_argument("--split-order", type=int, default=36,
                    help="split36: order of the one split permanent (36 is the workload)")
    ap.add_argument("--mod3-order", type=int, default=40,
                    help="mod3_40: matrix order (40 is the workload; smaller for profiling)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "batch4096":
        run_gpu_batch(args, world, rank, local)
    elif args.workload == "split36":
        run_gpu_split(args, world, rank, local)
    elif args.workload == "float28":
        run_gpu_float28(args, world, rank, local)
    elif args.workload in ("schur", "schur41", "binary40", "grid40"):
        run_gpu_exact_set(args, world, rank, local)
    elif args.workload == "mod3_40":
        run_gpu_mod3(args, world, rank, local)
    elif args.workload == "rook28":
        run_gpu_poly(args, world, rank, local)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
