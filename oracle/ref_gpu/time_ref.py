"""Times the reference's own GCOO kernels (the cubin compiled from its kernel
file, launched by ref_gpu_runner.c with the reference plugin's shapes and
synchronisation) next to this library on the same GPU and the same device
buffers, and checks that both give the same bits.

Run from the repository root on a GPU machine, after `__graft_entry__.build()`:
    python oracle/ref_gpu/time_ref.py [--size 8192] [--sparsity 0.99] [--reps 20]
Prints one JSON line. The reference's conversion allocates its nnz-sized arrays
per call; here they come from PyTorch's caching allocator, which is cheaper
than the reference's cudaMalloc, so its conversion time is a lower bound.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--sparsity", type=float, default=0.99)
    ap.add_argument("--reps", type=int, default=20)
    args = ap.parse_args()

    import torch

    import gcoospdm_gb300 as g
    import oracle
    from gcoospdm_gb300 import datagen as dg

    if not oracle.refgpu_available():
        print(json.dumps({"unavailable": "reference cubin not built (needs the reference tree at build time)"}))
        return
    n = args.size
    A = dg.bernoulli_dense_torch(0x6C02, n, n, 1.0 - args.sparsity, device="cuda")
    B = dg.dense_pm1_torch(0x6C02, 5, n, n, device="cuda")
    oracle.refgpu()
    stream = torch.cuda.current_stream()

    def ev_time(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def wall_time(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3 / reps

    # reference: conversion (synchronous, host round trip), multiply, and both (mutiplyBy)
    r = oracle.refgpu_convert(A, 4)
    nnz = r["nnz"]
    flop = 2.0 * nnz * n
    Cr = torch.empty(n, n, device="cuda")
    ref_convert = wall_time(lambda: oracle.refgpu_convert(A, 4), args.reps)
    ref_mul = ev_time(lambda: oracle.refgpu_spdm(r, B, Cr), args.reps)

    def ref_step():
        rr = oracle.refgpu_convert(A, 4)
        oracle.refgpu_spdm(rr, B, Cr)

    ref_e2e = wall_time(ref_step, args.reps)

    # this library: build, multiply, multiply_by (device-resident)
    h = g.GcooHandle(A).build()
    Co = torch.empty(n, n, device="cuda")
    ours_convert = ev_time(lambda: h.build(), args.reps)
    ours_mul = ev_time(lambda: h.spdm(B, Co), args.reps)
    ours_e2e = ev_time(lambda: h.multiply_by(B, Co), args.reps)
    oracle.refgpu_spdm(r, B, Cr)
    h.spdm(B, Co)
    torch.cuda.synchronize()
    same = bool(torch.equal(Co.view(torch.int32), Cr.view(torch.int32)))
    a = h.export()
    same_arrays = all(bool(torch.equal(a[f].cuda().view(torch.int32), r[f].view(torch.int32)))
                      for f in ("groupIndex", "nnzPerGroup", "vals", "rows", "cols"))
    out = {
        "workload": f"A {n}x{n} bernoulli p={1 - args.sparsity:g} U(-1,1), B {n}x{n} U(-1,1), FP32",
        "nnz": nnz,
        "reference_kernels": {"convert_ms": round(ref_convert, 4), "multiply_ms": round(ref_mul, 4),
                              "multiply_by_ms": round(ref_e2e, 4),
                              "multiply_gflops": round(flop / ref_mul / 1e6, 1),
                              "multiply_by_gflops": round(flop / ref_e2e / 1e6, 1)},
        "library": {"convert_ms": round(ours_convert, 4), "multiply_ms": round(ours_mul, 4),
                    "multiply_by_ms": round(ours_e2e, 4), "multiply_gflops": round(flop / ours_mul / 1e6, 1),
                    "multiply_by_gflops": round(flop / ours_e2e / 1e6, 1)},
        "speedup": {"convert": round(ref_convert / ours_convert, 2), "multiply": round(ref_mul / ours_mul, 2),
                    "multiply_by": round(ref_e2e / ours_e2e, 2)},
        "bit_identical_product": same, "bit_identical_arrays": same_arrays,
        "gpu": torch.cuda.get_device_name(0),
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
