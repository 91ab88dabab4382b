"""Benchmark of the bit-serial GEMM hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]
                    [--pipe auto|popc|bmma|tc|tc_pairs|tc_smem] [--variant V] [--no-configs ...]

A step is one gemmBitSerial over one pair of packed operands: by default the
2048 x 4096 x 2048 GEMM of a 3-bit unsigned lhs with a 2-bit signed rhs.  The
metric is the reference's GOPS = 2*M*K*N / time (benchmark/benchmark.cpp:107).

* value: inputs already packed in HBM; each step's forward kernel is timed
  with CUDA events on the launching stream; L2 is flushed (256 MiB write,
  outside the events) before every step.
* e2e: the same metric through the C ABI from pinned HOST buffers: both
  imports (the pack kernels read the host buffers over the host link) and
  gbs_gemm_to, whose kernels write the result into the host buffer -- the
  calls the C++ drop-in's importRegular / gemmBitSerial make.
* roofline: the forward kernel's rate against the measured peak of the pipe it
  ran on (tcgen05 e4m3 for the default workload, measured in this process).
* cpu_baseline: the reference's algorithm on this host's cores (the compiled
  reference when present, else the oracle's C restatement), same workload.

--impl reference times that CPU implementation alone, as the reference arm.
With N > 1 GPUs (torchrun) every rank runs an independent replica.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bit-exact GOPS @2048x4096x2048 w3/w2; grouped & adjoint speedup vs plain GPU"
PIPE_CHOICES = {"auto": 0, "popc": 1, "bmma": 2, "tc": 3, "tc_pairs": 4, "tc_smem": 5}  # GBS_PIPE_*
DEFAULT_WORKLOAD = "gemm_2048x4096x2048_u3s2"


E2E_LANES = 4  # host threads (steps in flight) of the end-to-end measurement
# device-side hold before the timed loop: ~6 us at 2 GHz per step (the host enqueues a gbs_gemm call in
# ~4 us) plus ~10 us for the first
HOLD_CYCLES_PER_STEP, HOLD_CYCLES_FIXED = 12000, 20000


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default=DEFAULT_WORKLOAD)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample (seconds)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-grouped", action="store_true", help="skip the grouped 512-problem measurement")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    p.add_argument("--no-configs", action="store_true", help="skip the per-config forward measurements")
    p.add_argument("--pipe", default="auto", choices=sorted(PIPE_CHOICES),
                   help="force the forward pipe of the headline workload (default: the library's choice)")
    p.add_argument("--variant", type=int, default=-1,
                   help="force the pipe variant (gbs_set_variant) of the headline workload")
    p.add_argument("--no-tuner", action="store_true",
                   help="ignore the committed tuner store (the library's built-in rule picks every kernel)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


TUNER_STORE = os.path.join(ROOT, "gemmbitserial_gb300", "tuned", "gb300_sm103a.txt")


def load_tuner(lib, args):
    """Loads the committed GB300 tuner store (written by gemmbitserial_gb300.tune_workloads) unless
    --no-tuner or GBS_TUNER_STORE names another; returns the path in use or None."""
    from gemmbitserial_gb300 import _capi
    if args.no_tuner:
        _capi.check(lib.gbs_tuner_clear())
        return None
    if os.environ.get("GBS_TUNER_STORE"):
        return os.environ["GBS_TUNER_STORE"]
    if not os.path.exists(TUNER_STORE):
        return None
    _capi.check(lib.gbs_tuner_load(TUNER_STORE.encode(), 1))
    return os.path.relpath(TUNER_STORE, ROOT)


def tuner_entry(lib, ctx):
    """The tuner store's entry a context's AUTO choice follows, or None."""
    pipe, variant, us = C.c_int(), C.c_int(), C.c_double()
    if lib.gbs_tuner_lookup(ctx._h, C.byref(pipe), C.byref(variant), C.byref(us)) != 0:
        return None
    return {"pipe": {1: "popc", 2: "bmma", 3: "tc", 4: "tc_pairs", 5: "tc_smem"}.get(pipe.value, pipe.value),
            "variant": variant.value, "tuned_us": round(us.value, 2)}


def pair_kernel_name(last_pair):
    """The SM-pair kernel a context's last launch ran (gbs_debug_last_pair), or None if none did."""
    bn, _, kind = (x.value for x in last_pair)
    if not bn:
        return None
    return {0: "gemm_tc_pair_kernel", 1: "gemm_tc_pair_persistent_kernel", 2: "gemm_tc_pair_streamk_kernel"}[kind]


def workload_desc(name):
    from gemmbitserial_gb300 import datagen
    M, K, N, (wA, eA), (wB, eB) = datagen.WORKLOADS[name]
    return {"workload": name, "M": M, "K": K, "N": N, "lhs": f"{eA}{wA}", "rhs": f"{eB}{wB}",
            "rhs_layout": "transposed (N x K)", "result_layout": "transposed (N x M) int32"}


L2_BYTES = 129 << 20  # GB300 L2 (2 x 64.5 MiB)


def resident_contexts(M, K, N, wA, wB) -> int:
    """Contexts the resident measurement rotates over: their operands (packed planes and e4m3 digit
    matrices) and results together hold more than twice the L2, so back-to-back steps read and
    write HBM instead of lines the previous step left in L2."""
    kpad = (K + 255) // 256 * 256
    per = (M + N) * kpad * (1 + max(wA, wB) / 8.0) + 4.0 * M * N
    return int(min(16, max(2, -(-2 * L2_BYTES // max(1, int(per))))))


L2_NOTE = ("GPU: back-to-back steps rotating over {P} contexts whose operands and results "
           "({MB:.0f} MB) exceed twice the 129 MB L2; host: the reference benchmark's loop")


def bench_config(desc, M, K, N, wA, wB) -> dict:
    """The `config` of both arms' lines: the workload and how L2 is kept out of the timing."""
    P = resident_contexts(M, K, N, wA, wB)
    kpad = (K + 255) // 256 * 256
    mb = P * ((M + N) * kpad * (1 + max(wA, wB) / 8.0) + 4.0 * M * N) / 1e6
    return dict(desc, l2=L2_NOTE.format(P=P, MB=mb))


def gops(M, K, N, seconds):
    return 2.0 * M * K * N / seconds / 1e9


def reduce_max(x: float, world: int, device=None) -> float:
    """The largest of a per-rank scalar over all ranks: the slowest replica sets the step time.
    Works with the nccl (CUDA tensor) and gloo (CPU tensor) process groups."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_gops(M, K, N, seconds_max: float, world: int) -> float:
    """Whole-job rate of `world` replicas, each running one M x K x N GEMM per step: the GEMMs
    of all ranks over the slowest rank's step time."""
    return gops(M, K, N, seconds_max) * world


# ---------------------------------------------------------------- CPU side

def cpu_time(name, seconds_budget, threads, max_reps=1000):
    """Times the reference's gemmBitSerial on the host (imports untimed). Returns (sec/call, kind, sample)."""
    from gemmbitserial_gb300 import datagen
    from oracle import oracle as O
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    if O.ref_available():
        R = O.ref()
        t1 = R.ref_time_gemm(M, K, N, wA, wB, int(sA), int(sB), O._ptr(A), O.DT_I8, O._ptr(B), O.DT_I8, 1, threads, None)
        reps = int(max(1, min(max_reps, seconds_budget / max(t1, 1e-6))))
        t = R.ref_time_gemm(M, K, N, wA, wB, int(sA), int(sB), O._ptr(A), O.DT_I8, O._ptr(B), O.DT_I8, reps, threads, None)
        return t, "reference", f"full {M}x{K}x{N} GEMM, {reps} timed calls after 1 warm-up, {threads} threads (rhs rows split)"
    ctx = O.OracleContext(M, K, N, wA, wB, sA, sB)
    ctx.import_(0, A)
    ctx.import_(1, B)
    ctx.gemm(threads)  # warm-up
    t0 = time.perf_counter()
    ctx.gemm(threads)
    t1 = time.perf_counter() - t0
    reps = int(max(1, min(max_reps, seconds_budget / max(t1, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.gemm(threads)
    t = (time.perf_counter() - t0) / reps
    ctx.close()
    return t, "port", f"full {M}x{K}x{N} GEMM, {reps} timed calls after 1 warm-up, {threads} threads (rhs rows split)"


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    desc = workload_desc(args.workload)
    M, K, N = desc["M"], desc["K"], desc["N"]
    threads = os.cpu_count() or 1
    from gemmbitserial_gb300 import datagen
    from oracle import oracle as O
    _, _, _, wA, sA, wB, sB, A, B = datagen.workload(args.workload)
    if O.ref_available():
        R = O.ref()
        R.ref_time_gemm(M, K, N, wA, wB, int(sA), int(sB), O._ptr(A), O.DT_I8, O._ptr(B), O.DT_I8, args.warmup, threads, None)
        sec = R.ref_time_gemm(M, K, N, wA, wB, int(sA), int(sB), O._ptr(A), O.DT_I8, O._ptr(B), O.DT_I8, args.steps, threads, None)
        kind = "reference"
    else:
        ctx = O.OracleContext(M, K, N, wA, wB, sA, sB)
        ctx.import_(0, A)
        ctx.import_(1, B)
        for _ in range(max(1, args.warmup)):
            ctx.gemm(threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.gemm(threads)
        sec = (time.perf_counter() - t0) / max(1, args.steps)
        ctx.close()
        kind = "port"
    v = gops(M, K, N, sec)
    sec1, _, sample1 = cpu_time(args.workload, args.cpu_seconds / 3, 1)
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "GOPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded splitmix64)", "config": bench_config(desc, M, K, N, wA, wB),
            "parallelism": f"host threads x{threads}",
            "cpu_baseline": {"value": round(v, 3), "unit": "GOPS", "cores": threads, "kind": kind,
                             "sample": f"full {M}x{K}x{N} gemmBitSerial per step, imports untimed, rhs rows split over {threads} threads",
                             "one_core": {"value": round(gops(M, K, N, sec1), 3), "unit": "GOPS", "cores": 1,
                                          "sample": sample1}},
            "e2e": {"value": round(v, 3), "unit": "GOPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side

class ClockSampler:
    """nvidia-smi clocks / throttle reasons of this process's GPU, sampled every 100 ms while running."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = str(index)
        try:
            import torch
            u = getattr(torch.cuda.get_device_properties(index), "uuid", None)
            if u is not None:
                self.index = "GPU-" + str(u)
        except Exception:
            pass
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)  # let the sampler start before the measured work
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "window": "warm-up and timed loops of both the resident and the end-to-end measurement"}


def read_traffic(kernel, workload):
    """dram bytes per launch recorded from an ncu capture (profiles/ncu_<kernel>_<workload>.txt)."""
    path = os.path.join(ROOT, "profiles", f"ncu_{kernel}_{workload}.txt")
    if not os.path.exists(path):
        return None
    m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def measure_grouped(lib, dev, stream, reps=5, warmup=2, mix=None, desc=None):
    """512-problem mix (or another mix): plain per-problem path vs one persistent grouped launch
    (and its CUDA graph)."""
    import torch
    from gemmbitserial_gb300 import _capi, datagen
    from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext
    from gemmbitserial_gb300.grouped import Group
    mix = datagen.grouped_mix() if mix is None else mix
    gen = torch.Generator(device=dev)
    gen.manual_seed(4321)
    ops = [(datagen.torch_operand(gen, M, K, wA, eA, dev), datagen.torch_operand(gen, N, K, wB, eB, dev))
           for (M, K, N, wA, eA, wB, eB) in mix]
    ctxs = [allocGEMMContext(M, K, N, wA, wB, eA != "u", eB != "u") for (M, K, N, wA, eA, wB, eB) in mix]
    sh = C.c_void_p(stream.cuda_stream)
    L = (C.c_void_p * len(ops))(*[a.data_ptr() for a, _ in ops])
    R = (C.c_void_p * len(ops))(*[b.data_ptr() for _, b in ops])

    def plain_gemm():
        for c in ctxs:
            _capi.check(lib.gbs_gemm(c._h, sh))

    def plain_full():
        for c, (a, b) in zip(ctxs, ops):
            _capi.check(lib.gbs_import(c._h, 0, C.c_void_p(a.data_ptr()), _capi.GBS_I8, 0, sh))
            _capi.check(lib.gbs_import(c._h, 1, C.c_void_p(b.data_ptr()), _capi.GBS_I8, 0, sh))
            _capi.check(lib.gbs_gemm(c._h, sh))

    def timed(fn):
        for _ in range(warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    with torch.cuda.stream(stream):
        t_plain_full = timed(plain_full)
        t_plain = timed(plain_gemm)
        ref = [c.res.copy() for c in ctxs[:: 37]]
        g = Group(ctxs)
        t_group = timed(lambda: _capi.check(lib.gbs_group_gemm(g._h, sh)))
        _capi.check(lib.gbs_group_capture(g._h, L, R, None, sh))
        t_graph = timed(lambda: _capi.check(lib.gbs_group_replay(g._h, sh)))
    ok = lib.gbs_group_status(g._h, sh) == 0 and all(
        np.array_equal(r, c.res) for r, c in zip(ref, ctxs[:: 37]))
    stats = g.stats()
    g.free()
    for c in ctxs:
        deallocGEMMContext(c)
    gops_total = sum(2.0 * M * K * N for (M, K, N, *_r) in mix)
    binops = sum(2.0 * M * N * ((K + 63) // 64 * 64) * wA * wB for (M, K, N, wA, _a, wB, _b) in mix)
    # algorithmic HBM bytes of the GEMMs: both operands' packed planes read once, the int32 results written
    alg_bytes = sum((M * wA + N * wB) * ((K + 63) // 64) * 8 + 4.0 * M * N for (M, K, N, wA, _a, wB, _b) in mix)
    hbm = measured_peaks().get("hbm_gbs")
    achieved_gbs = alg_bytes / (t_group * 1e-3) / 1e9
    return {"problems": len(mix), "plain_gemm_ms": round(t_plain, 4), "grouped_gemm_ms": round(t_group, 4),
            "speedup_gemm": round(t_plain / t_group, 3),
            "plain_pack_gemm_ms": round(t_plain_full, 4), "graph_pack_gemm_ms": round(t_graph, 4),
            "speedup_pack_gemm": round(t_plain_full / t_graph, 3),
            "grouped_gops": round(gops_total / (t_group * 1e-3) / 1e9, 1),
            "plain_gops": round(gops_total / (t_plain * 1e-3) / 1e9, 1),
            "grouped_tbinops": round(binops / (t_group * 1e-3) / 1e12, 2),
            "tiles": stats["tiles"], "grid": stats["grid"], "smem_bytes": stats["smem_bytes"],
            "popc_problems": stats["popc_problems"], "tc_problems": stats["tc_problems"],
            "tc_tiles": stats["tc_tiles"], "tc_kernel": stats["tc_kernel"],
            "hbm_roofline": {"algorithmic_bytes": alg_bytes, "achieved": round(achieved_gbs, 1), "unit": "GB/s",
                             "peak": hbm, "frac": round(achieved_gbs / hbm, 4) if hbm else None,
                             "bytes": "packed planes of both operands + int32 results, per grouped GEMM launch",
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)" if hbm else None},
            "parity": "grouped == plain (sampled 14 problems)" if ok else "MISMATCH",
            "mix": desc or "M log-uniform [1,256], K = 64*U{4..128}, N = U{64..4096}, wA {1,2,4}, wB {1,2,3,4}, u/s/b"}


def launch_floor(lib, ctx, stream, reps, per_graph=20):
    """The same GEMM launched back to back on one stream (operands stay in L2; for tiny GEMMs this
    is the host's call rate), and replayed from a CUDA graph holding per_graph gbs_gemm calls (the
    GPU-side cost of one GEMM, without the host's per-call work): (ms, ms) per GEMM."""
    import torch
    from gemmbitserial_gb300 import _capi
    sh = C.c_void_p(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(3):
            _capi.check(lib.gbs_gemm(ctx._h, sh))
        e0.record(stream)
        for _ in range(reps):
            _capi.check(lib.gbs_gemm(ctx._h, sh))
        e1.record(stream)
    stream.synchronize()
    b2b = e0.elapsed_time(e1) / reps
    g = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    cap.wait_stream(stream)
    with torch.cuda.graph(g, stream=cap):
        for _ in range(per_graph):
            _capi.check(lib.gbs_gemm(ctx._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    with torch.cuda.stream(stream):
        for _ in range(3):
            g.replay()
        e0.record(stream)
        for _ in range(reps):
            g.replay()
        e1.record(stream)
    stream.synchronize()
    return b2b, e0.elapsed_time(e1) / (reps * per_graph)


def measure_configs(lib, dev, stream, reps=50, warmup=5):
    """Every named workload (C1, C2, C3a, C3b, the adjoint layer's forward): forward time with packed
    operands resident and L2 flushed before each launch, the pipe the built-in rule chose, its rate,
    bytes moved, and bit-exactness against the reference's own result (sha256)."""
    import torch
    from gemmbitserial_gb300 import _capi, datagen
    from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_configs.json")))
    names = {_capi.GBS_PIPE_POPC: "popc", _capi.GBS_PIPE_BMMA: "b1-mma", _capi.GBS_PIPE_TC: "tcgen05-digits",
             _capi.GBS_PIPE_TC_PAIRS: "tcgen05-plane-pairs", _capi.GBS_PIPE_TC_SMEM: "tcgen05-smem-digits"}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sh = C.c_void_p(stream.cuda_stream)
    out = {}
    for name in datagen.WORKLOADS:
        M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
        ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
        with torch.cuda.stream(stream):
            ctx.lhs.importRegular(torch.from_numpy(A).to(dev), stream=stream)
            ctx.rhs.importRegular(torch.from_numpy(B).to(dev), stream=stream)
            for _ in range(warmup):
                flush.zero_()
                _capi.check(lib.gbs_gemm(ctx._h, sh))
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                _capi.check(lib.gbs_gemm(ctx._h, sh))
                e1.record(stream)
        stream.synchronize()
        ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
        b2b_ms, graph_ms = launch_floor(lib, ctx, stream, reps)
        res = ctx.res.reshape(N, M)
        ok = hashlib.sha256(np.ascontiguousarray(res).tobytes()).hexdigest() == gold.get(name, {}).get("sha256")
        pipe = ctx.pipe
        tuned = tuner_entry(lib, ctx)
        lp = [C.c_int(0), C.c_int(0), C.c_int(0)]
        _capi.check(lib.gbs_debug_last_pair(ctx._h, *(C.byref(x) for x in lp)))
        deallocGEMMContext(ctx)
        cuda_core_ms = None
        if max(wA, wB) > 4 and pipe == _capi.GBS_PIPE_TC:  # wide operands: the CUDA-core pipe beside it
            c2 = allocGEMMContext(M, K, N, wA, wB, sA, sB)
            c2.set_pipe(_capi.GBS_PIPE_POPC)
            with torch.cuda.stream(stream):
                c2.lhs.importRegular(torch.from_numpy(A).to(dev), stream=stream)
                c2.rhs.importRegular(torch.from_numpy(B).to(dev), stream=stream)
                flush.zero_()
                _capi.check(lib.gbs_gemm(c2._h, sh))
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                flush.zero_()
                e0.record(stream)
                _capi.check(lib.gbs_gemm(c2._h, sh))
                e1.record(stream)
            stream.synchronize()
            cuda_core_ms = e0.elapsed_time(e1)
            deallocGEMMContext(c2)
        kpad = (K + 63) // 64 * 64
        packed = wA * M * kpad // 8 + wB * N * kpad // 8 + 4 * M * N
        out[name] = {"ms": round(ms, 4), "gops": round(gops(M, K, N, ms * 1e-3), 1), "pipe": names.get(pipe, pipe),
                     "tbinops": round(2.0 * M * N * kpad * wA * wB / (ms * 1e-3) / 1e12, 2),
                     "gbs_packed_bytes": round(packed / (ms * 1e-3) / 1e9, 1),
                     "b2b_ms": round(b2b_ms, 4), "graph_replay_ms": round(graph_ms, 4),
                     "tuned": tuned, "pair_kernel": pair_kernel_name(lp),
                     **({"cuda_core_ms": round(cuda_core_ms, 4), "speedup_vs_cuda_cores": round(cuda_core_ms / ms, 1),
                         "how": "operands split into plane parts of <= 4 bits, one digit GEMM per part pair"}
                        if cuda_core_ms else {}),
                     "parity": "bit-exact vs reference (sha256)" if ok else "MISMATCH"}
    return out


def measure_adjoint(lib, dev, stream, reps=10, warmup=3):
    """QAT layer adjoint: A 4096x2048 u2, B 2048x2048 bipolar, dC ~ N(0,1).  Ours (FP32 from the packed
    planes) vs the plain GPU path (export values, two FP32 cuBLAS matmuls with TF32 off)."""
    import torch
    from gemmbitserial_gb300 import _capi, datagen
    from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext
    M, K, N = 4096, 2048, 2048
    A = datagen.operand(datagen.SEED_BASE + 50, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 51, N, K, 1, "b")
    dC = datagen.normal_f32(datagen.SEED_BASE + 52, (N, M))
    ctx = allocGEMMContext(M, K, N, 2, 1, False, True)
    sh = C.c_void_p(stream.cuda_stream)
    with torch.cuda.stream(stream):
        ctx.lhs.importRegular(torch.from_numpy(A).to(dev), stream=stream)
        ctx.rhs.importRegular(torch.from_numpy(B).to(dev), stream=stream)
        d = torch.from_numpy(dC).to(dev)
        dA = torch.empty(M, K, device=dev)
        dB = torch.empty(N, K, device=dev)
        Ai = torch.empty(M, K, dtype=torch.int32, device=dev)
        Bi = torch.empty(N, K, dtype=torch.int32, device=dev)
    stream.synchronize()

    def ours():
        _capi.check(lib.gbs_adjoint(ctx._h, C.c_void_p(d.data_ptr()), C.c_void_p(dA.data_ptr()),
                                    C.c_void_p(dB.data_ptr()), sh))

    prev_tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False

    def plain():
        _capi.check(lib.gbs_export(ctx._h, 0, C.c_void_p(Ai.data_ptr()), sh))
        _capi.check(lib.gbs_export(ctx._h, 1, C.c_void_p(Bi.data_ptr()), sh))
        pa = d.T @ Bi.float()
        pb = d @ Ai.float()
        return pa, pb

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                fn()
            stream.synchronize()
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / reps

    # float64 adjoint for the error figures: A's values are its low 2 bits (unsigned),
    # B's are +1 where the input is positive and -1 elsewhere (bipolar)
    d64 = dC.astype(np.float64)
    dA64 = d64.T @ np.where(B > 0, 1.0, -1.0)
    dB64 = d64 @ (A.astype(np.int64) & 3).astype(np.float64)

    def errs():
        return {"dA": float(np.max(np.abs(dA.cpu().numpy() - dA64)) / np.max(np.abs(dA64))),
                "dB": float(np.max(np.abs(dB.cpu().numpy() - dB64)) / np.max(np.abs(dB64)))}

    t_ours = timed(ours)  # tensor-core adjoint (the default)
    err_ours = errs()
    os.environ["GBS_ADJOINT_PIPE"] = "simt"
    try:
        t_simt = timed(ours)  # CUDA-core FP32 adjoint
        err_simt = errs()
    finally:
        del os.environ["GBS_ADJOINT_PIPE"]
    t_plain = timed(plain)
    torch.backends.cuda.matmul.allow_tf32 = prev_tf32
    fma, f8, bf16 = C.c_double(), C.c_double(), C.c_double()
    _capi.check(lib.gbs_fma_peak(C.byref(fma)))
    _capi.check(lib.gbs_tc_peaks(C.byref(f8), C.byref(bf16)))
    deallocGEMMContext(ctx)
    flops = 2.0 * 2.0 * M * K * N  # the FP32 math of dA and dB
    achieved = flops / (t_ours * 1e-3) / 1e12
    tc_work = 3.0 * flops  # bf16 MMA work: three split terms of dC
    tc_achieved = tc_work / (t_ours * 1e-3) / 1e12
    simt_achieved = flops / (t_simt * 1e-3) / 1e12
    return {"shape": f"A {M}x{K} u2, B {N}x{K} bipolar, dC {N}x{M} fp32", "ms": round(t_ours, 4),
            "pipe": "tcgen05 bf16, dC split exactly into 3 bf16 terms, fp32 TMEM accumulation",
            "tflops_fp32_equivalent": round(achieved, 2), "plain_ms": round(t_plain, 4),
            "plain": "export values + 2 FP32 cuBLAS matmuls (TF32 off)",
            "speedup_vs_plain": round(t_plain / t_ours, 3),
            "roofline": adjoint_roofline(tc_achieved, bf16.value / 1e12, achieved),
            "max_rel_err_normwise": err_ours,
            "simt": {"ms": round(t_simt, 4), "tflops": round(simt_achieved, 2),
                     "frac_of_fp32_fma_peak": round(simt_achieved / (fma.value / 1e12), 4),
                     "fma_peak": round(fma.value / 1e12, 2), "max_rel_err_normwise": err_simt}}


def measured_peaks() -> dict:
    """Measured peaks of this GPU type (HBM copy GB/s, cuBLAS bf16 TF/s burst and sustained), if present."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def adjoint_roofline(achieved: float, mma_rate: float, algorithmic: float | None = None) -> dict:
    """The bf16 adjoint kernel against the measured bf16 peak of this GPU type (cuBLAS burst: the kernel is
    timed alone), with this process's raw MMA-loop rate beside it.  `achieved` counts the MMA work executed
    (three bf16 split terms per FP32 product); `algorithmic` the FP32 math itself (2 x 2*M*N*K), reported
    against the same denominators."""
    mp = measured_peaks()
    peak, src = mp.get("bf16_tflops"), "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 GEMM, burst)"
    if not peak:
        peak, src = 1900.0, "fallback 1.9 PFLOP/s bf16 (no MEASURED_PEAKS.json)"
    return {"bound": "tensor", "kernel": "adjoint_tc_kernel", "achieved": round(achieved, 2),
            "peak": round(peak, 2), "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
            "work": "3 x 2 x 2*M*N*K bf16 FLOPs (split terms x (dA, dB))", "peak_source": src,
            "mma_loop_rate": round(mma_rate, 1),
            "frac_of_mma_loop_rate": round(achieved / mma_rate, 4) if mma_rate > 0 else None,
            **({"algorithmic_fp32": {"achieved": round(algorithmic, 2), "unit": "TFLOP/s",
                                     "work": "2 x 2*M*N*K FP32 FLOPs (dA and dB)",
                                     "frac": round(algorithmic / peak, 4),
                                     "frac_of_mma_loop_rate": round(algorithmic / mma_rate, 4) if mma_rate > 0 else None}}
               if algorithmic is not None else {})}


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from gemmbitserial_gb300 import _capi, datagen
    from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext
    lib = _capi.load()
    tuner_store = load_tuner(lib, args)
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(args.workload)
    desc = workload_desc(args.workload)
    stream = torch.cuda.Stream(device=dev)
    sh = C.c_void_p(stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def force(c):  # --pipe / --variant: the same choice for the resident and the end-to-end context
        if args.pipe != "auto":
            c.set_pipe(PIPE_CHOICES[args.pipe])
        if args.variant != -1:
            _capi.check(lib.gbs_set_variant(c._h, args.variant))

    # ---- resident path: packed operands in HBM.  P contexts over the same inputs, each with its
    # own planes, digit matrices and result, together more than twice the L2: the timed steps
    # rotate over them back to back, so no step finds its operands or result in L2.
    P = resident_contexts(M, K, N, wA, wB)
    ctxs = [allocGEMMContext(M, K, N, wA, wB, sA, sB) for _ in range(P)]
    dA = torch.from_numpy(A).to(dev)
    dB = torch.from_numpy(B).to(dev)
    with torch.cuda.stream(stream):
        for ctx in ctxs:
            force(ctx)
            ctx.lhs.importRegular(dA, stream=stream)
            ctx.rhs.importRegular(dB, stream=stream)
    stream.synchronize()
    del dA, dB
    clk = ClockSampler(local).__enter__()
    with torch.cuda.stream(stream):
        for i in range(max(args.warmup, P)):
            _capi.check(lib.gbs_gemm(ctxs[i % P]._h, sh))
    barrier()
    launches0 = lib.gbs_debug_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        # a device-side sleep holds the stream (before the first event, untimed) while the host
        # enqueues the K launches, so the events time the GPU's back-to-back rate rather than the
        # host's enqueue of the first launch into an idle GPU (~0.7 us per step at K = 20)
        torch.cuda._sleep(HOLD_CYCLES_FIXED + HOLD_CYCLES_PER_STEP * args.steps)
        e0.record(stream)
        for i in range(args.steps):
            _capi.check(lib.gbs_gemm(ctxs[i % P]._h, sh))
        e1.record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall
    launches = lib.gbs_debug_launch_count() - launches0
    ms = reduce_max(e0.elapsed_time(e1) / max(1, args.steps), world, dev)
    # the same GEMM launched alone after a 256 MiB L2 flush (launch latency included), for reference
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            _capi.check(lib.gbs_gemm(ctxs[i % P]._h, sh))
            ev[i][1].record(stream)
    barrier()
    del flush
    isolated_ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
    want = json.load(open(os.path.join(ROOT, "tests", "golden", "ref_configs.json"))).get(args.workload, {}).get("sha256")
    got = {hashlib.sha256(np.ascontiguousarray(c.res.reshape(N, M)).tobytes()).hexdigest() for c in ctxs}
    parity = ("bit-exact vs reference (sha256, every context)" if got == {want} else
              ("MISMATCH" if want else "unchecked"))
    pipe = ctxs[0].pipe
    tuned = tuner_entry(lib, ctxs[0])
    last_pair = [C.c_int(0), C.c_int(0), C.c_int(0)]  # tile width, K split / pairs, kernel kind of the last pair launch
    _capi.check(lib.gbs_debug_last_pair(ctxs[0]._h, *(C.byref(x) for x in last_pair)))
    for ctx in ctxs:
        deallocGEMMContext(ctx)

    # ---- end to end through the C ABI from pinned host buffers.  Every step imports both operands
    # from host memory and stores its result into a pinned host buffer (gbs_gemm_to); both calls
    # return once the host memory has been read or written, as the reference's importRegular and
    # gemmBitSerial do.  Serial: one host thread, one context, one stream.  In flight: E2E_LANES host
    # threads, each with its own context, stream and result buffer, each running its share of the
    # steps, so that some threads' result stores overlap others' operand reads (the link carries
    # both directions at once); every step still moves all of its own bytes.  Measured on GB300
    # (ms per step; copy-engine imports): 1 thread 0.222, 2 threads 0.147, 3 0.129, 4 0.127.
    hA = torch.from_numpy(A).pin_memory()
    hB = torch.from_numpy(B).pin_memory()
    hR = [torch.empty(M * N, dtype=torch.int32).pin_memory() for _ in range(E2E_LANES)]
    e2e_ctx = [allocGEMMContext(M, K, N, wA, wB, sA, sB) for _ in range(1 + E2E_LANES)]
    e2e_streams = [stream] + [torch.cuda.Stream(device=dev) for _ in range(E2E_LANES - 1)]
    for c in e2e_ctx:
        force(c)
    # the threads' contexts import through the copy engines (GBS_HOST_IMPORT_STAGED): another
    # thread's GEMM holds most SMs while it stores its result, which starves pack kernels that read
    # host memory themselves (two threads: 0.147 against 0.187 ms per step); the serial context reads
    # its sources in place (0.221 against 0.234 ms)
    for c in e2e_ctx[1:]:
        c.set_host_import(_capi.GBS_HOST_IMPORT_STAGED)

    def e2e_step(i, lanes):
        c = e2e_ctx[0] if lanes == 1 else e2e_ctx[1 + i % lanes]
        st, r = C.c_void_p(e2e_streams[i % lanes].cuda_stream), hR[i % lanes]
        _capi.check(lib.gbs_import(c._h, 0, C.c_void_p(hA.data_ptr()), _capi.GBS_I8, 0, st))
        _capi.check(lib.gbs_import(c._h, 1, C.c_void_p(hB.data_ptr()), _capi.GBS_I8, 0, st))
        # gemmBitSerial + the read of ctx.res, as the C++ drop-in issues them
        _capi.check(lib.gbs_gemm_to(c._h, C.c_void_p(r.data_ptr()), st))

    def e2e_time(lanes):
        import threading
        for r in hR:
            r.zero_()
        start = threading.Barrier(lanes + 1)
        errors = []

        def lane(k):  # steps k, k + lanes, k + 2 * lanes, ... on this thread's context and stream
            try:
                torch.cuda.set_device(dev)
                for i in range(k, args.warmup * lanes, lanes):
                    e2e_step(i, lanes)
                start.wait()
                for i in range(k, args.steps, lanes):
                    e2e_step(i, lanes)
            except BaseException as ex:  # noqa: BLE001 -- reported after the join
                errors.append(ex)
                start.abort()

        threads = [threading.Thread(target=lane, args=(k,)) for k in range(lanes)]
        for t in threads:
            t.start()
        try:
            start.wait()
        except threading.BrokenBarrierError:  # a lane failed: its error is raised after the join
            pass
        t0 = time.perf_counter()
        for t in threads:
            t.join()
        barrier()
        sec = (time.perf_counter() - t0) / args.steps
        if errors:
            raise errors[0]
        ok = all(hashlib.sha256(hR[k].numpy().tobytes()).hexdigest() == want for k in range(lanes))
        return reduce_max(sec, world, dev), ok

    e2e_serial_s, e2e_serial_ok = e2e_time(1)
    e2e_s, e2e_ok = e2e_time(E2E_LANES)
    clk.__exit__()
    for c in e2e_ctx:
        deallocGEMMContext(c)

    if rank != 0:
        return
    # ---- roofline of the forward kernel against the measured peak of the pipe it ran on
    kpad = (K + 63) // 64 * 64
    if pipe in (_capi.GBS_PIPE_TC, _capi.GBS_PIPE_TC_PAIRS, _capi.GBS_PIPE_TC_SMEM):
        f8, bf16 = C.c_double(), C.c_double()
        _capi.check(lib.gbs_tc_peaks(C.byref(f8), C.byref(bf16)))
        if pipe == _capi.GBS_PIPE_TC and (args.variant in (128, 256) or
                                          (args.variant == -1 and tuned and tuned["variant"] in (128, 256))):
            kernel = "gemm_tc_tma_kernel"
        elif pipe == _capi.GBS_PIPE_TC:  # the kernel the library's rule, the tuner or a forced variant launched
            kernel = pair_kernel_name(last_pair) or "gemm_tcg_kernel"
        else:
            kernel = "gemm_tc_kernel"
        digits = pipe != _capi.GBS_PIPE_TC_PAIRS
        # fp8 multiply-adds the tensor pipe must do: one per (m, n, k) in digit mode, one per plane pair otherwise
        work = 2.0 * M * N * K * (1 if digits else wA * wB)
        achieved = work / (ms * 1e-3) / 1e12
        peak = f8.value / 1e12
        roof = {"bound": "tensor", "kernel": kernel, "achieved": round(achieved, 2), "peak": round(peak, 2),
                "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
                "peak_source": "measured in-process at full SM clock (gbs_tc_peaks: back-to-back "
                               "tcgen05.mma kind::f8f6f4 M=128 N=256 on every SM; no e4m3 figure in MEASURED_PEAKS.json)",
                "work": "2*M*N*K fp8 FLOPs (digit mode: all plane pairs in one MMA)" if digits
                        else "2*M*N*K*wA*wB fp8 plane-pair FLOPs",
                "bf16_peak_measured": round(bf16.value / 1e12, 1)}
        if kernel in ("gemm_tc_pair_kernel", "gemm_tc_pair_persistent_kernel"):  # the tile and K split that ran
            roof["pair_tile"] = f"256x{last_pair[0].value}"
            roof["k_split"] = last_pair[1].value
        elif kernel == "gemm_tc_pair_streamk_kernel":
            roof["pair_tile"] = "256x256"
            roof["sm_pairs"] = last_pair[1].value
    else:
        popc, bmma = C.c_double(), C.c_double()
        _capi.check(lib.gbs_pipe_peaks(C.byref(popc), C.byref(bmma)))
        kernel = "gemm_bmma_kernel" if pipe == _capi.GBS_PIPE_BMMA else "gemm_popc_tiled"
        binops = 2.0 * M * N * kpad * wA * wB  # AND + add per bit of each plane pair
        achieved = binops / (ms * 1e-3) / 1e12
        peak = 2.0 * popc.value / 1e12
        roof = {"bound": "popc", "kernel": kernel, "achieved": round(achieved, 3), "peak": round(peak, 3),
                "unit": "Tbinop/s", "frac": round(achieved / peak, 4),
                "peak_source": "measured in-process (gbs_pipe_peaks: CUDA-core AND+POPC loop)",
                "bmma_peak": round(2.0 * bmma.value / 1e12, 3)}
    roof["traffic"] = read_traffic(kernel, args.workload)
    roof["tuner"] = {"store": tuner_store, "entry": tuned}
    roof["algorithmic_bytes"] = int(wA * M * kpad // 8 + wB * N * kpad // 8 + 4 * M * N)
    clocks = clk.summary()

    configs = None if args.no_configs else measure_configs(lib, dev, stream)
    grouped = None if args.no_grouped else measure_grouped(lib, dev, stream)
    caffenet = None
    if not args.no_grouped:  # the reference's CaffeNet chain (benchmark.cpp:174-237) as a second group
        caffenet = measure_grouped(lib, dev, stream, reps=20, warmup=3, mix=datagen.caffenet_mix(),
                                   desc="CaffeNet chain, 8 GEMMs, 2-bit unsigned x 2-bit unsigned")
    adjoint = None if args.no_adjoint else measure_adjoint(lib, dev, stream)

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        threads = os.cpu_count() or 1
        sec, kind, sample = cpu_time(args.workload, args.cpu_seconds, threads)
        sec1, _, sample1 = cpu_time(args.workload, args.cpu_seconds / 3, 1)
        cpu = {"value": round(gops(M, K, N, sec), 3), "unit": "GOPS", "cores": threads, "kind": kind, "sample": sample,
               "one_core": {"value": round(gops(M, K, N, sec1), 3), "unit": "GOPS", "cores": 1, "sample": sample1}}

    v = replica_gops(M, K, N, ms * 1e-3, world)
    line = {"metric": METRIC, "value": round(v, 3), "unit": "GOPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded splitmix64)",
            "config": bench_config(desc, M, K, N, wA, wB),
            "parallelism": f"replicas x{world}",
            "pipe": {1: "popc", 2: "bmma", 3: "tcgen05 (HBM digits, TMA)", 4: "tcgen05 (smem plane pairs)",
                     5: "tcgen05 (smem digits)"}.get(pipe, str(pipe)),
            **({"forced": {"pipe": args.pipe, "variant": args.variant}}
               if args.pipe != "auto" or args.variant != -1 else {}),
            "timing": "CUDA events around the K back-to-back launches, queued behind an untimed device-side "
                      "hold so that the host's enqueue is not in the timed region; wall_s_timed_region includes "
                      "the hold",
            "isolated_launch": {"ms": round(isolated_ms, 5), "gops": round(gops(M, K, N, isolated_ms * 1e-3), 1),
                                "how": "each launch alone after a 256 MiB L2 flush, CUDA events around it "
                                       "(launch latency included); median of the steps"},
            "parity": parity,
            "e2e": {"value": round(replica_gops(M, K, N, e2e_s, world), 3), "unit": "GOPS",
                    "h2d_bytes_per_step": int(A.nbytes + B.nbytes), "d2h_bytes_per_step": int(M * N * 4),
                    "ms_per_step": round(e2e_s * 1e3, 4), "parity": "bit-exact" if e2e_ok else "MISMATCH",
                    "how": "gbs_import x2 from pinned host buffers + gbs_gemm_to a pinned host buffer per step "
                           f"(each call returns once its host memory is read or written); {E2E_LANES} steps in flight: "
                           f"{E2E_LANES} host threads, each with its own context (imports through the copy "
                           "engines, GBS_HOST_IMPORT_STAGED), stream and result buffer; wall clock over all steps",
                    "serial": {"value": round(replica_gops(M, K, N, e2e_serial_s, world), 3),
                               "ms_per_step": round(e2e_serial_s * 1e3, 4),
                               "parity": "bit-exact" if e2e_serial_ok else "MISMATCH",
                               "how": "the same calls from one host thread, one context (sources read in place by the "
                                      "pack kernels), one stream"}},
            "roofline": roof,
            "configs": configs, "grouped": grouped, "caffenet": caffenet, "adjoint": adjoint,
            "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clocks,
            "wall_s_timed_region": round(t_wall, 4)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
    world, _, _ = dist_env()
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
