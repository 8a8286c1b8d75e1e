#!/usr/bin/env python
"""Benchmark of the GCOO sparse x dense multiply on GB300.

Workload: A 8192 x 8192 FP32 with a Bernoulli(0.01) nonzero mask (sparsity
0.99) and U(-1,1) values, B 8192 x 8192 FP32 U(-1,1), seeded synthetic data.
One step = one mutiplyBy (dense -> GCOO conversion + FP32 multiply), the
measure the reference publishes. value = 2 * nnz * n / step time (GFLOP/s),
summed over ranks (each rank runs its own replica: the path needs no
exchange between GPUs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (the oracle
port; the reference itself has no CPU implementation of this path) on the
host cores, on a bounded row sample of the same workload.
Prints one JSON line (rank 0).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 8192
METRIC = "SpDM GFLOP/s (2*nnz*n), dense->GCOO conversion + FP32 multiply per step"
UNIT = "GFLOP/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=8192, help="m = k = n of the square workload")
    ap.add_argument("--sparsity", type=float, default=0.99)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the extra precision/batched lines")
    ap.add_argument("--no-gpu-baselines", action="store_true",
                    help="skip timing the reference algorithm, cuSPARSE and cuBLAS on the same GPU")
    ap.add_argument("--sweep", action="store_true", help="print the FP32 n x sparsity sweep instead")
    ap.add_argument("--no-sweep", action="store_true", help="skip the sweep key of the main line")
    ap.add_argument("--case", choices=["tc_bf16", "tc_split", "convert", "fp32", "batched", "fp8", "bf16_fma",
                                       "fp32_block", "convert_irregular", "spdm_irregular", "spdm_irregular_split"],
                    help="run one small case a few times (for profiling) and exit")
    return ap.parse_args()


def run_case(args):
    """A few launches of one kernel on a small case (sized for ncu captures)."""
    import torch
    import gcoospdm_gb300 as g
    from gcoospdm_gb300 import datagen as dg
    dev = torch.device("cuda", 0)
    if args.case in ("tc_bf16", "tc_split", "fp32_block"):
        m, n = 8192, 1024
        A = dg.block_dense_torch(4096 + 750, m, m, 0.25, device=dev)
        B = dg.dense_pm1_torch(4096, 5, m, n, device=dev)
        h = g.GcooHandle(A).build()
        prec = {"tc_bf16": "bf16", "tc_split": "split_bf16", "fp32_block": "fp32"}[args.case]
        for _ in range(3):
            h.spdm(B, prec=prec)
    elif args.case == "batched":
        res = run_batched(g, dg, torch, dev, count=64)
        print(json.dumps(res))
    elif args.case == "convert_irregular":
        # the irregular workload's dense operand (65536^2, 17 GB): a first build, then rebuilds
        m = 65536
        rows, cols, vals = dg.zipf_coo(65536, m, m, 1_200_000, alpha=2.0, cap=4096)
        A = torch.zeros(m, m, device=dev)
        A[torch.from_numpy(rows).to(dev), torch.from_numpy(cols).to(dev)] = torch.from_numpy(vals).to(dev)
        h = g.GcooHandle(A)
        print(json.dumps({"first_build_ms": round(_time(torch, h.build, reps=1, warm=0), 4),
                          "rebuild_ms": round(_time(torch, h.build, reps=3, warm=0), 4), "nnz": h.nnz}))
    elif args.case in ("spdm_irregular", "spdm_irregular_split"):
        # the irregular workload's multiply, from COO input (no 17 GB dense operand);
        # _split: the long rows summed in 32-entry pieces (gcoo_params.fp32_sum = split)
        m, n = 65536, 256
        rows, cols, vals = dg.zipf_coo(65536, m, m, 1_200_000, alpha=2.0, cap=4096)
        r32, c32 = torch.from_numpy(rows.astype("int32")).to(dev), torch.from_numpy(cols.astype("int32")).to(dev)
        mode = "split" if args.case == "spdm_irregular_split" else "chain"
        hc = g.GcooHandle.from_coo(r32, c32, torch.from_numpy(vals).to(dev), m=m, k=m, fp32_sum=mode).build()
        B = torch.from_numpy(dg.normal_dense(65536, 40, m, n)).to(dev)
        Cd = torch.empty(m, n, device=dev)
        print(json.dumps({"spdm_ms": round(_time(torch, lambda: hc.spdm(B, Cd), reps=3, warm=1), 4)}))
    else:
        n = args.size
        A = dg.bernoulli_dense_torch(SEED, n, n, 1.0 - args.sparsity, device=dev)
        B = dg.dense_pm1_torch(SEED, 5, n, n, device=dev)
        h = g.GcooHandle(A).build()
        for _ in range(3):
            if args.case == "convert":
                h.build()
            elif args.case == "fp32":
                h.spdm(B)
            elif args.case == "fp8":
                h.spdm(B, prec="fp8_b")
            else:
                h.spdm(B, prec="bf16")
    torch.cuda.synchronize()
    print(f"case {args.case} done", flush=True)


def dist_setup(gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampling around the timed region (every 20 ms, timestamped);
    the summary keeps the samples taken inside the region that mark() names."""

    SAMPLE_MS = 20

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None
        self.window = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.SAMPLE_MS)],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def mark(self, t0: float, t1: float):
        """The timed region in host wall-clock seconds (time.time())."""
        self.window = (t0, t1)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        import datetime
        rows = []  # (time, sm MHz, max MHz, reason flags, power W)
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    rows.append((ts, float(p[2]), float(p[3]), p[6:10],
                                 float(p[4]) if p[4] not in ("[N/A]", "") else 0.0))
                except ValueError:
                    continue
        os.unlink(self.path)
        if not rows:
            return None
        inside = [r for r in rows if self.window and self.window[0] <= r[0] <= self.window[1]]
        if inside:
            use = inside
        else:  # a region shorter than the sampling period: the samples nearest to it
            mid = (self.window[0] + self.window[1]) / 2 if self.window else rows[-1][0]
            use = sorted(rows, key=lambda r: abs(r[0] - mid))[:2]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in use for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": max(r[2] for r in use),
                "reasons": reasons, "samples": len(use), "samples_in_region": len(inside),
                "sample_ms": self.SAMPLE_MS}


def workload_config(n: int, sparsity: float, nnz: int, world: int) -> dict:
    """The bench line's config, key for key the same in both arms: the square
    FP32 workload (A n x n Bernoulli(1 - sparsity), B n x n), its nonzeros and
    the GPU arm's timing hygiene (no L2 flush: A and B each exceed L2)."""
    p = 1.0 - sparsity
    mb = 4 * n * n / 1e6
    return {"workload": f"fp32 gcoo convert+multiply, A {n}x{n} bernoulli p={p:g} U(-1,1), B {n}x{n} U(-1,1)",
            "m": n, "k": n, "n": n, "sparsity": sparsity, "nnz": int(nnz), "rows_per_group": 4,
            "l2": f"no flush: inputs larger than L2 (A and B {mb:.0f} MB each, L2 129 MB)",
            "parallelism": f"replicas x{world}"}


def cpu_sample_gflops(A_rows, B, cpg=4, target_s=1.0, max_runs=20):
    """Oracle port (convert + multiply) on a row sample, all host threads:
    repeated for about target_s seconds (at least 3, at most max_runs runs)."""
    import numpy as np
    import oracle
    nt = oracle.max_threads() or os.cpu_count() or 1
    rows = A_rows
    nnz = int(np.count_nonzero(rows))
    n = B.shape[1]
    oracle.multiply_by(rows[: min(64, rows.shape[0])], B, cpg, nt)  # warm the pages
    times = []
    t_end = time.perf_counter() + target_s
    while len(times) < 3 or (time.perf_counter() < t_end and len(times) < max_runs):
        t0 = time.perf_counter()
        oracle.multiply_by(rows, B, cpg, nt)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return 2.0 * nnz * n / t / 1e9, nt, len(times), t


def run_reference(args, rank, world):
    """The reference algorithm's CPU implementation (oracle port), host cores."""
    if rank != 0:
        return
    import numpy as np
    from gcoospdm_gb300 import datagen as dg
    import oracle
    oracle.build()
    n = args.size
    p = 1.0 - args.sparsity
    B = dg.dense_pm1(SEED, 5, n, n)
    probe = dg.bernoulli_dense(SEED, 256, n, p)
    g, nt, _, t = cpu_sample_gflops(probe, B, target_s=0.2)
    rows = int(max(256, min(n, 256 * 0.5 / max(t, 1e-6)))) // 4 * 4  # ~0.5 s per step
    A = dg.bernoulli_dense(SEED, rows, n, p)
    nnz = int(np.count_nonzero(A))
    for _ in range(args.warmup):
        oracle.multiply_by(A, B, 4, nt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.multiply_by(A, B, 4, nt)
    dt = (time.perf_counter() - t0) / args.steps
    value = 2.0 * nnz * n / dt / 1e9
    sample = f"rows 0..{rows} of the {n}x{n} s={args.sparsity} matrix (convert + multiply), B {n}x{n}"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded splitmix64)",
        "config": workload_config(n, args.sparsity, dg.bernoulli_nnz(SEED, n, n, p), world),
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": nt, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU implementation of this path; the oracle restates its algorithm "
                "(src/gcoo_spdm_kernels.cu) in C with OpenMP",
    }
    gk = reference_gpu_kernels(args, oracle)
    if gk:
        line["reference_gpu_kernels"] = gk
    print(json.dumps(line), flush=True)


def reference_gpu_kernels(args, oracle):
    """The reference's own GPU kernels (its kernel file compiled into a cubin
    where the reference tree was present), launched with its plugin's shapes and
    synchronisation, on the full workload: mutiplyBy with device-resident inputs
    and end to end with host buffers. None when there is no GPU or no cubin."""
    try:
        import torch
        if not torch.cuda.is_available() or not oracle.refgpu_available():
            return None
        from gcoospdm_gb300 import datagen as dg
        n = args.size
        A = dg.bernoulli_dense_torch(SEED, n, n, 1.0 - args.sparsity, device="cuda")
        B = dg.dense_pm1_torch(SEED, 5, n, n, device="cuda")
        Cd = torch.empty(n, n, device="cuda")
        oracle.refgpu()
        nnz = oracle.refgpu_convert(A, 4)["nnz"]
        flop = 2.0 * nnz * n

        def step():
            r = oracle.refgpu_convert(A, 4)
            oracle.refgpu_spdm(r, B, Cd)

        Ah, Bh = A.cpu().pin_memory(), B.cpu().pin_memory()
        Ch = torch.empty(n, n).pin_memory()

        def e2e_step():
            A.copy_(Ah, non_blocking=True)
            B.copy_(Bh, non_blocking=True)
            step()
            Ch.copy_(Cd, non_blocking=True)
            torch.cuda.synchronize()

        out = {}
        for name, fn in (("multiply_by", step), ("e2e", e2e_step)):
            for _ in range(max(args.warmup, 1)):
                fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            reps = max(args.steps, 5)
            for _ in range(reps):
                fn()
            torch.cuda.synchronize()
            ms = (time.perf_counter() - t0) * 1e3 / reps
            out[name] = {"ms_per_step": round(ms, 4), "value": round(flop / ms / 1e6, 3), "unit": UNIT}
        out["e2e"]["h2d_bytes_per_step"] = int(Ah.numel() * 4 + Bh.numel() * 4)
        out["e2e"]["d2h_bytes_per_step"] = int(Ch.numel() * 4)
        out["note"] = ("src/gcoo_spdm_kernels.cu compiled unmodified for sm_103a; host orchestration of "
                       "src/ShGCOOSpDM.cu:19-180 restated (synchronous, nnz read back per call)")
        out["gpu"] = torch.cuda.get_device_name(0)
        return out
    except Exception as e:  # the CPU line above stands on its own
        return {"error": f"{type(e).__name__}: {e}"}


def load_profile_traffic():
    p = os.path.join(ROOT, "profiles", "spdm_fp32_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except OSError:
        return None


def run_ours(args, rank, world, local, pg):
    import torch
    import gcoospdm_gb300 as g
    from gcoospdm_gb300 import datagen as dg

    if not os.path.exists(g.LIB_PATH):
        g.build()
    torch.cuda.set_device(local)
    L = g.lib()
    n = args.size
    m = k = n
    p = 1.0 - args.sparsity
    dev = torch.device("cuda", local)
    A = dg.bernoulli_dense_torch(SEED, m, k, p, device=dev)
    B = dg.dense_pm1_torch(SEED, 5, k, n, device=dev)
    Cd = torch.empty(m, n, device=dev)
    h = g.GcooHandle(A).build()
    nnz = h.nnz
    flop = 2.0 * nnz * n
    stream = torch.cuda.current_stream()

    # ---- headline: convert + multiply per step, device-resident inputs -------------
    for _ in range(args.warmup):
        h.multiply_by(B, Cd)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(pg)
    torch.cuda.synchronize()
    launches0 = L.gcoo_kernel_launches()
    with Clocks(local) as clk:
        t_region = time.time()
        e0.record(stream)
        for _ in range(args.steps):
            h.multiply_by(B, Cd)
        e1.record(stream)
        torch.cuda.synchronize()
        clk.mark(t_region, time.time())
    launches = L.gcoo_kernel_launches() - launches0
    barrier(pg)
    ms = max_over_ranks(pg, e0.elapsed_time(e1) / args.steps)
    value = flop * world / (ms * 1e-3) / 1e9
    clocks = clk.summary()

    # ---- the dominant kernel alone (multiply only), for the roofline --------------
    reps = max(args.steps, 10)
    for _ in range(3):
        h.spdm(B, Cd)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        h.spdm(B, Cd)
    e1.record(stream)
    torch.cuda.synchronize()
    t_spdm = e0.elapsed_time(e1) / reps * 1e-3
    ng = (m + 3) // 4
    alg_bytes = 12 * nnz + 8 * (ng + 1) + 4 * k * n + 4 * m * n
    peaks, peak_kind = measured_peaks()
    achieved = alg_bytes / t_spdm / 1e9
    # the L2 -> SM read peak, measured live on this GPU (512-byte gathers from an L2-resident region)
    l2_peak = g.measure_l2_read_gbs()
    l2_bytes = 4.0 * nnz * n  # the B rows the multiply gathers: n floats per entry
    prof = load_profile_traffic()
    traffic = None
    if prof and prof.get("n") == n and abs(prof.get("sparsity", 0) - args.sparsity) < 1e-9:
        traffic = prof.get("dram_bytes_per_launch")
    fma_peak = 152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    # The binding path: one 4-byte B value per FMA comes through L2 (ncu: L2
    # reads per launch, and their share of the L2 peak at the ncu duration).
    l2_path = None
    if traffic and prof.get("l2_read_bytes_per_launch"):
        l2b = prof["l2_read_bytes_per_launch"]
        l2_path = {"l2_read_bytes_per_launch": l2b, "achieved_gbs": round(l2b / t_spdm / 1e9, 1),
                   "ncu_l2_throughput_pct_of_peak": prof.get("l2_throughput_pct_of_peak"),
                   "note": "L2 reads from one ncu capture; achieved = those bytes / this run's kernel time"}
    # conversion alone (build: count + scan + scatter, one readback)
    for _ in range(2):
        h.build()
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(5):
        h.build()
    e1.record(stream)
    torch.cuda.synchronize()
    t_conv = e0.elapsed_time(e1) / 5 * 1e-3
    err = h.error_norm(B, Cd)

    # ---- end to end through the C ABI with host buffers ------------------------------
    e2e = None
    if not args.no_e2e:
        # Through the host-buffer entry point (gcoo_session_multiply): pinned A, B
        # in, C out, every step; copy-in, conversion, multiply and copy-out of
        # row panels overlap on the session's streams.
        Ah = A.cpu().pin_memory()
        Bh = B.cpu().pin_memory()
        Ch = torch.empty(m, n, dtype=torch.float32).pin_memory()
        sess = g.GcooSession()

        def e2e_step():
            sess.multiply(Ah, Bh, Ch, stream=stream)

        for _ in range(args.warmup):
            e2e_step()
        torch.cuda.synchronize()
        barrier(pg)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks(pg, e0.elapsed_time(e1) / args.steps)
        assert torch.equal(Ch.to(dev).view(torch.int32), Cd.view(torch.int32))
        st = sess.stats()
        sess.close()
        # the same step done one copy after another (copy A, B; mutiplyBy; copy C)
        Ad, Bd = torch.empty_like(A), torch.empty_like(B)
        h2 = g.GcooHandle(Ad)

        def seq_step():
            Ad.copy_(Ah, non_blocking=True)
            Bd.copy_(Bh, non_blocking=True)
            h2.multiply_by(Bd, Cd)
            Ch.copy_(Cd, non_blocking=True)

        ms_seq = _time(torch, seq_step, reps=5, warm=2)
        del h2, Ad, Bd
        e2e = {"value": round(flop * world / (ms_e2e * 1e-3) / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(Ah.numel() * 4 + Bh.numel() * 4), "d2h_bytes_per_step": int(Ch.numel() * 4),
               "ms_per_step": round(ms_e2e, 4), "api": "gcoo_session_multiply (host buffers, pinned)",
               "panels": st["panels"], "launches_per_step": st["launches"],
               "sequential_copies_ms_per_step": round(ms_seq, 4)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import numpy as np
        # the whole step (all rows of A, convert + multiply) repeated for about 10 s of host work
        Ah_rows = A.cpu().numpy()
        Bh_np = B.cpu().numpy()
        gfl, nt, nrep, t = cpu_sample_gflops(np.ascontiguousarray(Ah_rows), np.ascontiguousarray(Bh_np),
                                             target_s=10.0, max_runs=400)
        cpu = {"value": round(gfl, 3), "unit": UNIT, "cores": nt, "kind": "port",
               "sample": f"the full step (all {Ah_rows.shape[0]} rows of A, convert + multiply, full B), "
                         f"median of {nrep} runs of {t:.3f} s ({nrep * t:.1f} s of host work)"}

    forms = None
    if not args.no_forms:
        forms = run_forms(args, g, dg, torch, dev)

    sweep = None
    if rank == 0 and world == 1 and not args.no_sweep:
        try:
            sweep = {"note": "multiply alone (FP32), square A n x n Bernoulli, B n x n, timed as CUDA-graph "
                             "replays of back-to-back calls; hbm_frac of the measured copy peak, l2_frac of the "
                             "live L2 read peak; B fits L2 for n <= 4096",
                     "l2_peak_gbs": round(l2_peak, 1),
                     "points": sweep_points(g, dg, torch, dev, peaks, l2_peak)}
        except Exception as e:  # the main line still prints
            sweep = {"error": f"{type(e).__name__}: {e}"}
        torch.cuda.empty_cache()

    gpu_baselines = None
    if rank == 0 and world == 1 and not args.no_gpu_baselines:
        gpu_baselines = run_gpu_baselines(g, torch, A, B, flop)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": round(value / 117.1, 3) if (n == 8192 and abs(args.sparsity - 0.99) < 1e-9) else None,
        "dtype": "f32", "data": "synthetic (seeded splitmix64; U(-1,1) values, Bernoulli mask)",
        "config": workload_config(n, args.sparsity, nnz, world),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic,
                     "kernel": "spdm_fp32_kernel", "algorithmic_bytes": alg_bytes,
                     "kernel_ms": round(t_spdm * 1e3, 4), "peak_source": peak_kind,
                     "l2_read_bytes": int(l2_bytes), "l2_achieved_gbs": round(l2_bytes / t_spdm / 1e9, 1),
                     "l2_peak_gbs": round(l2_peak, 1), "l2_peak_source": "measured live (bench.py)",
                     "l2_frac": round(l2_bytes / t_spdm / 1e9 / l2_peak, 4) if l2_peak else None,
                     "binding": "l2" if l2_peak and l2_bytes / l2_peak > alg_bytes / peaks["hbm_gbs"] else "hbm"},
        "l2_path": l2_path,
        "fma_roofline": {"achieved_tflops": round(flop / t_spdm / 1e12, 3), "nominal_peak_tflops": round(fma_peak, 1),
                         "frac": round(flop / t_spdm / 1e12 / fma_peak, 4)},
        "spdm_only_gflops": round(flop / t_spdm / 1e9, 3),
        "convert_ms": round(t_conv * 1e3, 4),
        "rel_fro_vs_fp64": err,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if gpu_baselines:
        line["gpu_baselines"] = gpu_baselines
    if forms:
        line["forms"] = forms
    if sweep:
        line["sweep"] = sweep
    print(json.dumps(line), flush=True)


def _time(torch, fn, reps=5, warm=2):
    stream = torch.cuda.current_stream()
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps  # ms


def _time_graph(torch, fn, per_graph=10, replays=3):
    """Device time per call of fn, from a CUDA graph holding per_graph calls
    (replayed `replays` times after one warm replay): no host launch gaps
    between calls, which dominate kernels of a few tens of microseconds."""
    fn()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for _ in range(per_graph):
            fn()
    graph.replay()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(replays):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    del graph
    return e0.elapsed_time(e1) / (replays * per_graph)  # ms


def _rel_fro_rows(torch, A, B, C, rows):
    """Relative Frobenius error of C on sampled rows against an FP64 product."""
    idx = torch.as_tensor(rows, device=A.device)
    ref = A[idx].double() @ B.double()
    return float(torch.linalg.norm(C[idx].double() - ref) / torch.linalg.norm(ref))


def run_precision_forms(g, dg, torch, dev, sparsities=(0.5, 0.75, 0.9), m=8192, n=1024):
    """Block-clustered A (16x16 blocks), every form, time + error vs FP64."""
    out = {}
    B = dg.dense_pm1_torch(4096, 5, m, n, device=dev)
    sample = list(range(0, m, 97))
    for s in sparsities:
        A = dg.block_dense_torch(4096 + int(s * 1000), m, m, 1.0 - s, device=dev)
        h = g.GcooHandle(A).build()
        nnz = h.nnz
        flop = 2.0 * nnz * n
        Cd = torch.empty(m, n, device=dev)
        row = {"nnz": nnz}
        for prec in ("fp32", "bf16", "split_bf16", "fp8_b"):
            h.prepare(n, prec)
            ms = _time(torch, lambda: h.spdm(B, Cd, prec=prec))
            row[prec] = {"ms": round(ms, 4), "gflops": round(flop / ms / 1e6, 1),
                         "rel_fro_vs_fp64": _rel_fro_rows(torch, A, B, Cd, sample),
                         "engine": "tensor" if (prec != "fp32" and h.query_engine(prec)) else "fma"}
        row["bf16_speedup_vs_fp32"] = round(row["fp32"]["ms"] / row["bf16"]["ms"], 2)
        row["split_speedup_vs_fp32"] = round(row["fp32"]["ms"] / row["split_bf16"]["ms"], 2)
        out[f"s{s}"] = row
        del A, h, Cd
        torch.cuda.empty_cache()
    return {"workload": f"A {m}x{m} 16x16 block mask, B {m}x{n}", **out}


def run_batched(g, dg, torch, dev, count=512):
    """512 independent multiplies: sequential FP32 launches vs one persistent launch."""
    shapes = dg.batched_shapes(5120, count)
    probs = []
    flop = 0.0
    for i, (m, k, n, s) in enumerate(shapes):
        A = dg.bernoulli_dense_torch(6000 + i, m, k, 1.0 - s, device=dev)
        B = dg.dense_pm1_torch(6000 + i, 5, k, n, device=dev)
        h = g.GcooHandle(A).build()
        C = torch.empty(m, n, device=dev)
        probs.append((h, A, B, C))
        flop += 2.0 * h.nnz * n
    seq_ms = _time(torch, lambda: [h.spdm(B, C) for h, A, B, C in probs], reps=3, warm=1)
    res = {"workload": f"{count} problems, m,k U[256,4096], n in {{32,64,128}}, s U[0.9,0.999]",
           "gflop": round(flop / 1e9, 3), "sequential_fp32": {"ms": round(seq_ms, 4), "launches": count,
                                                              "gflops": round(flop / seq_ms / 1e6, 1)}}
    refs = [C.clone() for h, A, B, C in probs]  # the sequential launches' results, all problems
    L = g.lib()
    for prec in ("fp32", "bf16"):
        bt = g.GcooBatch([(h, B, C) for h, A, B, C in probs], prec=prec)
        l0 = L.gcoo_kernel_launches()
        ms = _time(torch, bt.run, reps=10, warm=2)
        launches = (L.gcoo_kernel_launches() - l0) // 12
        errs = [_rel_fro_rows(torch, A, B, C, list(range(0, A.shape[0], 7))) for h, A, B, C in probs]
        same = all(torch.equal(C, r) for (h, A, B, C), r in zip(probs, refs)) if prec == "fp32" else None
        res[f"batched_{prec}"] = {"ms": round(ms, 4), "gflops": round(flop / ms / 1e6, 1), "launches": int(launches),
                                  "speedup_vs_sequential_fp32": round(seq_ms / ms, 2),
                                  "max_rel_fro_vs_fp64": max(errs), "problems_checked": len(errs),
                                  "bit_identical_to_single": same}
        bt.close()
    return res


def run_irregular(g, dg, torch, dev, m=65536, n=256, nnz=1_200_000):
    """Zipf(2) row counts capped at 4096, 65536^2 sparse operand (dense: 17 GB)."""
    rows, cols, vals = dg.zipf_coo(65536, m, m, nnz, alpha=2.0, cap=4096)
    A = torch.zeros(m, m, device=dev)
    A[torch.from_numpy(rows).to(dev), torch.from_numpy(cols).to(dev)] = torch.from_numpy(vals).to(dev)
    B = dg.normal_dense(65536, 40, m, n)
    B = torch.from_numpy(B).to(dev)
    h = g.GcooHandle(A)
    conv_ms = _time(torch, h.build, reps=3, warm=1)
    Cd = torch.empty(m, n, device=dev)
    ms = _time(torch, lambda: h.spdm(B, Cd), reps=10)
    ms_graph = _time_graph(torch, lambda: h.spdm(B, Cd), per_graph=10)
    err = h.error_norm(B, Cd)
    flop = 2.0 * h.nnz * n
    # the long rows summed in 32-entry pieces (gcoo_params.fp32_sum = split)
    hs = g.GcooHandle(A, fp32_sum="split").build()
    Cs = torch.empty(m, n, device=dev)
    hs.spdm(B, Cs)
    split = {"spdm_ms": round(_time(torch, lambda: hs.spdm(B, Cs), reps=10), 4),
             "spdm_graph_ms": round(_time_graph(torch, lambda: hs.spdm(B, Cs), per_graph=10), 4),
             "rel_fro_vs_fp64": hs.error_norm(B, Cs),
             "note": "rows of >= 256 entries as 32-entry pieces added in piece order: deterministic, "
                     "not bit-identical to the chain; shorter rows keep the chain"}
    split["gflops"] = round(flop / split["spdm_graph_ms"] / 1e6, 1)
    del hs, Cs
    counts = torch.bincount(torch.from_numpy(rows), minlength=m)
    # the same matrix ingested from COO triplets, without the 17 GB dense buffer
    r32, c32 = torch.from_numpy(rows.astype("int32")).to(dev), torch.from_numpy(cols.astype("int32")).to(dev)
    v32 = torch.from_numpy(vals).to(dev)
    hc = g.GcooHandle.from_coo(r32, c32, v32, m=m, k=m)
    coo_ms = _time(torch, hc.build, reps=3, warm=1)
    same = bool(torch.equal(hc.spdm(B), Cd))
    # the same multiply through cuSPARSE SpMM and the reference's CSR plugin restated (kernel only)
    base = {}
    Cb = torch.empty(m, n, device=dev)
    for algo in ("cusparse", "csr"):
        try:
            b = g.SpGemmBuilder.getShGemmAlgo(A, m, m, algo)
            b.build()
            ker = _time(torch, lambda: b.runKernelTest(B, m, n, Cb), reps=5, warm=1)
            base[algo] = {"multiply_ms": round(ker, 4), "multiply_gflops": round(flop / ker / 1e6, 1)}
            del b
        except Exception as e:
            base[algo] = {"error": f"{type(e).__name__}: {e}"}
    del Cb
    res = {"workload": f"A {m}x{m} Zipf(2) rows capped 4096, nnz {h.nnz}, B {m}x{n} N(0,1)",
           "max_row_nnz": int(counts.max()), "convert_ms": round(conv_ms, 4),
           "coo_ingest_ms": round(coo_ms, 4), "coo_result_identical": same, "spdm_ms": round(ms, 4),
           "spdm_graph_ms": round(ms_graph, 4),
           "gflops": round(flop / ms / 1e6, 1), "rel_fro_vs_fp64": err, "split_sum": split,
           "spdm_gbps": round((12 * h.nnz + 8 * (m // 4 + 1) + 4 * m * n * 2) / ms / 1e6, 1),
           "gpu_baselines": base}
    del A
    torch.cuda.empty_cache()
    return res


def run_gpu_baselines(g, torch, A, B, flop):
    """Same workload through the baselines built for this GPU: the reference's
    GCOO algorithm restated on the GPU, cuSPARSE SpMM (CSR), cuBLAS SGEMM on
    the dense-with-zeros operand, and the reference's auxiliary CSR plugin
    restated. Each: convert+multiply and multiply only."""
    m, k = A.shape
    n = B.shape[1]
    Cd = torch.empty(m, n, device=A.device)
    out = {}
    try:
        ref = g.RefAlgoBaseline(A)
        e2e = _time(torch, lambda: ref.multiply_by(B, Cd), reps=3, warm=1)
        ref.build()
        ker = _time(torch, lambda: ref.run_kernel(B, Cd), reps=3, warm=1)
        out["reference_algorithm_gcoo"] = {"multiply_by_ms": round(e2e, 4), "multiply_ms": round(ker, 4),
                                           "multiply_gflops": round(flop / ker / 1e6, 1),
                                           "note": "the reference's GCOO algorithm restated for the GPU"}
        ref.close()
    except Exception as e:
        out["reference_algorithm_gcoo"] = {"error": f"{type(e).__name__}: {e}"}
    for algo in ("cusparse", "cublas", "csr"):
        try:
            b = g.SpGemmBuilder.getShGemmAlgo(A, m, k, algo)
            e2e = _time(torch, lambda: b.mutiplyBy(B, k, n, Cd), reps=3, warm=1)
            b.build()
            ker = _time(torch, lambda: b.runKernelTest(B, k, n, Cd), reps=3, warm=1)
            out[algo] = {"multiply_by_ms": round(e2e, 4), "multiply_ms": round(ker, 4),
                         "multiply_gflops": round(flop / ker / 1e6, 1)}
            del b
        except Exception as e:
            out[algo] = {"error": f"{type(e).__name__}: {e}"}
    return out


def run_forms(args, g, dg, torch, dev):
    """Extra measurements: precision forms, batched, irregular."""
    out = {}
    for name, fn in (("precision_forms", lambda: run_precision_forms(g, dg, torch, dev)),
                     ("batched", lambda: run_batched(g, dg, torch, dev)),
                     ("irregular", lambda: run_irregular(g, dg, torch, dev))):
        try:
            out[name] = fn()
        except Exception as e:  # report, never hide: the main line still prints
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        torch.cuda.empty_cache()
    return out


def sweep_points(g, dg, torch, dev, peaks, l2_peak, full=False):
    """The FP32 sweep (n x sparsity grid, square A Bernoulli, B n x n): the
    multiply alone per point, with its HBM fraction (algorithmic bytes
    12 nnz + 8 (nGroup + 1) + 8 n^2) and L2 fraction (the B rows gathered,
    nnz * n * 4 bytes, against the live L2 read peak). full=True adds the
    conversion, mutiplyBy and (n <= 4096) the error against FP64."""
    out = []
    for n in (2048, 4096, 8192, 16384):
        B = dg.dense_pm1_torch(n, 5, n, n, device=dev)
        Cd = torch.empty(n, n, device=dev)
        for s in (0.95, 0.98, 0.99, 0.995, 0.999):
            A = dg.bernoulli_dense_torch(n + int(s * 1e4), n, n, 1.0 - s, device=dev)
            h = g.GcooHandle(A)
            conv = _time(torch, h.build, reps=3, warm=1) if full else None
            if not full:
                h.build()
            ms = _time_graph(torch, lambda: h.spdm(B, Cd), per_graph=10 if n <= 8192 else 3)
            nnz = h.nnz
            alg = 12 * nnz + 8 * (n // 4 + 1) + 8 * n * n
            l2b = 4.0 * nnz * n
            pt = {"n": n, "sparsity": s, "nnz": nnz, "spdm_ms": round(ms, 4),
                  "spdm_gflops": round(2.0 * nnz * n / ms / 1e6, 1),
                  "hbm_frac": round(alg / ms / 1e6 / peaks["hbm_gbs"], 4),
                  "l2_read_gbps": round(l2b / ms / 1e6, 1),
                  "l2_frac": round(l2b / ms / 1e6 / l2_peak, 4) if l2_peak else None}
            pt["binding"] = "l2" if (pt["l2_frac"] or 0) >= pt["hbm_frac"] else "hbm"
            if full:
                e2e = _time(torch, lambda: h.multiply_by(B, Cd), reps=3)
                pt.update({"convert_ms": round(conv, 4), "multiply_by_ms": round(e2e, 4),
                           "multiply_by_gflops": round(2.0 * nnz * n / e2e / 1e6, 1),
                           "rel_fro_vs_fp64": h.error_norm(B, Cd) if n <= 4096 else None})
            out.append(pt)
            del A, h
        del B, Cd
        torch.cuda.empty_cache()
    return out


def run_sweep(args):
    """The FP32 sweep, one JSON line per point."""
    import torch
    import gcoospdm_gb300 as g
    from gcoospdm_gb300 import datagen as dg
    dev = torch.device("cuda", 0)
    peaks, _ = measured_peaks()
    l2_peak = g.measure_l2_read_gbs()
    for pt in sweep_points(g, dg, torch, dev, peaks, l2_peak, full=True):
        print(json.dumps({**pt, "l2_peak_gbs": round(l2_peak, 1)}), flush=True)


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args.gpus)
    if args.case:
        run_case(args)
    elif args.sweep:
        run_sweep(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
