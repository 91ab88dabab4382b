"""Tunes the named benchmark workloads on this GPU and writes the tuner store.

    python -m gemmbitserial_gb300.tune_workloads [--out PATH] [--reps R]

For each workload of gemmbitserial_gb300.datagen.WORKLOADS (the reference's
plain GEMM shapes, seeded synthetic operands) gbs_tune times every pipe and
variant that applies -- CUDA-core tile classes, b1 mma.sync, the tcgen05
digit kernels with each SM-pair tile width and K split, the persistent and
stream-K pair kernels, the shared-memory decode kernels -- on the context's own
data, and records the fastest for the workload's shape class.  The store is
written to gemmbitserial_gb300/tuned/gb300_sm103a.txt (the file bench.py and
the tests load) unless --out says otherwise.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
STORE = os.path.join(HERE, "tuned", "gb300_sm103a.txt")
PIPES = {1: "popc", 2: "bmma", 3: "tc", 4: "tc_pairs", 5: "tc_smem"}


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--out", default=STORE)
    p.add_argument("--reps", type=int, default=10)
    args = p.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    import torch

    from gemmbitserial_gb300 import _capi, datagen
    from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext
    lib = _capi.load()
    _capi.check(lib.gbs_tuner_clear())
    s = torch.cuda.Stream()
    for name in datagen.WORKLOADS:
        M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
        ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
        try:
            with torch.cuda.stream(s):
                ctx.lhs.importRegular(torch.from_numpy(A).cuda(), stream=s)
                ctx.rhs.importRegular(torch.from_numpy(B).cuda(), stream=s)
            s.synchronize()
            best = C.c_int()
            _capi.check(lib.gbs_tune(ctx._h, args.reps, C.byref(best), C.c_void_p(s.cuda_stream)))
            pipe, variant, us = C.c_int(), C.c_int(), C.c_double()
            _capi.check(lib.gbs_tuner_lookup(ctx._h, C.byref(pipe), C.byref(variant), C.byref(us)))
            print(f"{name}: {PIPES.get(pipe.value, pipe.value)} variant {variant.value} {us.value:.2f} us")
        finally:
            deallocGEMMContext(ctx)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    _capi.check(lib.gbs_tuner_save(args.out.encode()))
    print("store:", args.out, lib.gbs_tuner_entries(), "entries")


if __name__ == "__main__":
    main()
