"""One library operation per case, repeated, for per-kernel profiling.

    python -m gemmbitserial_gb300.kernel_cases CASE [--reps N]

Each case sets up seeded synthetic operands of a named workload, runs the
operation once to warm up, then --reps times (default 3), synchronises and
prints "ok <case>".  The kernels each case launches:

  gemm            2048x4096x2048 u3 x s2 forward, the library's choice (gemm_tc_pair_kernel)
  gemm_streamk    the same on the stream-K SM-pair kernel (gemm_tc_pair_streamk_kernel)
  gemm_popc       the same on the CUDA cores (gemm_popc_tiled)
  gemm_bmma       the same on b1 mma.sync (gemm_bmma_kernel)
  gemm_tc_smem    the same, planes decoded in shared memory (gemm_tc_kernel)
  gemm_skinny     8x8192x8 u1 x u1 (gemm_popc_skinny)
  gemm_rows       9 x 8192 x 32768, 1-bit unsigned x 2-bit signed on the CUDA cores (gemm_popc_rows: at most
                  16 lhs rows, 64 rhs rows x every lhs row per CTA)
  import_device   importRegular of the 2048x4096 int8 lhs from device memory, planes + digits (pack_rowmajor)
  import_host     the same from pinned host memory, read over the host link (pack_rowmajor)
  import_colmajor the same operand read column-major (pack_colmajor)
  import_quantize importRegularAndQuantize of a 2048x4096 float lhs, 7 thresholds per row (pack_quantize_kernel)
  expand          column-major imports, then a forward that first expands the planes (expand_one_kernel)
  group           the 512-problem mix as one group: import, row sums, GEMMs (pack_grouped, rowsum_grouped,
                  gemm_tcg_kernel, gemm_popc_grouped)
  group_small     the same on a 96-problem mix of the same distribution (a few hundred MB on the device)
  adjoint         A 4096x2048 u2, B 2048x2048 bipolar, dC ~ N(0,1) (split_kernel, values_t_kernel, adjoint_tc_kernel)
  adjoint_simt    the same on the CUDA cores (adjoint_kernel)
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys

CASES = ["gemm", "gemm_streamk", "gemm_popc", "gemm_bmma", "gemm_tc_smem", "gemm_skinny", "gemm_rows", "import_device",
         "import_host", "import_colmajor", "import_quantize", "expand", "group", "group_small", "adjoint",
         "adjoint_simt"]


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("case", choices=CASES)
    p.add_argument("--reps", type=int, default=3)
    args = p.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    if args.case == "adjoint_simt":
        os.environ["GBS_ADJOINT_PIPE"] = "simt"
    import torch

    from gemmbitserial_gb300 import _capi, datagen
    from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext
    lib = _capi.load()
    s = torch.cuda.Stream()
    sh = C.c_void_p(s.cuda_stream)
    dev = torch.device("cuda")
    case = args.case

    def ctx_of(name, pipe=None, variant=None):
        M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
        c = allocGEMMContext(M, K, N, wA, wB, sA, sB)
        if pipe is not None:
            c.set_pipe(pipe)
        if variant is not None:
            _capi.check(lib.gbs_set_variant(c._h, variant))
        return c, torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)

    if case.startswith("gemm"):
        pipe, variant, name = None, None, "gemm_2048x4096x2048_u3s2"
        if case == "gemm_streamk":
            pipe, variant = _capi.GBS_PIPE_TC, 515
        elif case == "gemm_popc":
            pipe = _capi.GBS_PIPE_POPC
        elif case == "gemm_bmma":
            pipe = _capi.GBS_PIPE_BMMA
        elif case == "gemm_tc_smem":
            pipe, variant = _capi.GBS_PIPE_TC_SMEM, 256
        elif case == "gemm_skinny":
            name = "gemm_8x8192x8_u1u1"
        if case == "gemm_rows":
            c = allocGEMMContext(9, 8192, 32768, 1, 2, False, True)
            c.set_pipe(_capi.GBS_PIPE_POPC)
            dA = torch.from_numpy(datagen.operand(datagen.SEED_BASE + 61, 9, 8192, 1, "u")).to(dev)
            dB = torch.from_numpy(datagen.operand(datagen.SEED_BASE + 62, 32768, 8192, 2, "s")).to(dev)
        else:
            c, dA, dB = ctx_of(name, pipe, variant)
        with torch.cuda.stream(s):
            c.lhs.importRegular(dA, stream=s)
            c.rhs.importRegular(dB, stream=s)
        run = lambda: _capi.check(lib.gbs_gemm(c._h, sh))  # noqa: E731
    elif case.startswith("import"):
        c, dA, dB = ctx_of("gemm_2048x4096x2048_u3s2")
        if case == "import_device":
            run = lambda: _capi.check(lib.gbs_import(c._h, 0, C.c_void_p(dA.data_ptr()), _capi.GBS_I8, 0, sh))  # noqa
        elif case == "import_host":
            hA = dA.cpu().pin_memory()
            run = lambda: _capi.check(lib.gbs_import(c._h, 0, C.c_void_p(hA.data_ptr()), _capi.GBS_I8, 0, sh))  # noqa
        elif case == "import_colmajor":
            dT = dA.t().contiguous()
            run = lambda: _capi.check(lib.gbs_import(c._h, 0, C.c_void_p(dT.data_ptr()), _capi.GBS_I8, 1, sh))  # noqa
        else:
            deallocGEMMContext(c)
            c = allocGEMMContext(2048, 4096, 2048, 3, 2, False, True)
            g = torch.Generator(device=dev)
            g.manual_seed(5)
            X = torch.randn(2048, 4096, generator=g, device=dev)
            T = torch.sort(torch.randn(7, 2048, generator=g, device=dev), dim=0).values.contiguous()
            run = lambda: _capi.check(lib.gbs_import_quantize(c._h, 0, C.c_void_p(X.data_ptr()),  # noqa: E731
                                                              C.c_void_p(T.data_ptr()), 7, _capi.GBS_F32, 0, sh))
    elif case == "expand":
        c, dA, dB = ctx_of("gemm_2048x4096x2048_u3s2")
        aT, bT = dA.t().contiguous(), dB.t().contiguous()

        def run():  # column-major imports write no digits: the forward expands them first
            _capi.check(lib.gbs_import(c._h, 0, C.c_void_p(aT.data_ptr()), _capi.GBS_I8, 1, sh))
            _capi.check(lib.gbs_import(c._h, 1, C.c_void_p(bT.data_ptr()), _capi.GBS_I8, 1, sh))
            _capi.check(lib.gbs_gemm(c._h, sh))
    elif case in ("group", "group_small"):
        from gemmbitserial_gb300.grouped import Group
        mix = datagen.grouped_mix() if case == "group" else datagen.grouped_mix(seed=datagen.SEED_BASE + 77, count=96)
        gen = torch.Generator(device=dev)
        gen.manual_seed(4321)
        ops = [(datagen.torch_operand(gen, M, K, wA, eA, dev), datagen.torch_operand(gen, N, K, wB, eB, dev))
               for (M, K, N, wA, eA, wB, eB) in mix]
        ctxs = [allocGEMMContext(M, K, N, wA, wB, eA != "u", eB != "u") for (M, K, N, wA, eA, wB, eB) in mix]
        grp = Group(ctxs)

        def run():
            grp.import_([a for a, _ in ops], [b for _, b in ops], stream=s)
            grp.gemm(stream=s)
    else:  # adjoint
        M, K, N = 4096, 2048, 2048
        A = datagen.operand(datagen.SEED_BASE + 50, M, K, 2, "u")
        B = datagen.operand(datagen.SEED_BASE + 51, N, K, 1, "b")
        dC = torch.from_numpy(datagen.normal_f32(datagen.SEED_BASE + 52, (N, M))).to(dev)
        c = allocGEMMContext(M, K, N, 2, 1, False, True)
        with torch.cuda.stream(s):
            c.lhs.importRegular(torch.from_numpy(A).to(dev), stream=s)
            c.rhs.importRegular(torch.from_numpy(B).to(dev), stream=s)
        dA = torch.empty(M, K, device=dev)
        dB = torch.empty(N, K, device=dev)
        run = lambda: _capi.check(lib.gbs_adjoint(c._h, C.c_void_p(dC.data_ptr()), C.c_void_p(dA.data_ptr()),  # noqa
                                                  C.c_void_p(dB.data_ptr()), sh))
    s.synchronize()
    with torch.cuda.stream(s):
        for _ in range(1 + args.reps):
            run()
    s.synchronize()
    assert lib.gbs_debug_tc_error() == 0
    print("ok", case, flush=True)


if __name__ == "__main__":
    main()
