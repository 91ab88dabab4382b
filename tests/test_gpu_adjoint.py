"""FP32 adjoint (dA = dC.B, dB = dC^T.A from the packed planes) against a
float64 oracle and against exact unit-step finite differences.

Error metrics (both stated, both must stay below 1e-6):
  normwise    max|x - x64| / max|x64|
  elementwise max over entries of |x - x64| / sum|terms|   (sum|terms| = |dC| . |B| etc.)
"""
import ctypes as C

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    return gbs_lib


@pytest.fixture(params=["tc", "simt"])
def adjoint_pipe(request, monkeypatch):
    """GBS_ADJOINT_PIPE: the tensor-core adjoint (default) or the CUDA-core FP32 kernel."""
    if request.param == "tc":
        monkeypatch.delenv("GBS_ADJOINT_PIPE", raising=False)
    else:
        monkeypatch.setenv("GBS_ADJOINT_PIPE", "simt")
    return request.param


def run_adjoint(A, B, wA, eA, wB, eB, dC):
    import torch
    M, K = A.shape
    N = B.shape[0]
    ctx = allocGEMMContext(M, K, N, wA, wB, eA != "u", eB != "u")
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        d = torch.from_numpy(dC).cuda()
        dA = torch.empty(M, K, dtype=torch.float32, device="cuda")
        dB = torch.empty(N, K, dtype=torch.float32, device="cuda")
        _capi.check(_capi.load().gbs_adjoint(ctx._h, C.c_void_p(d.data_ptr()), C.c_void_p(dA.data_ptr()),
                                             C.c_void_p(dB.data_ptr()), None))
        torch.cuda.synchronize()
        return dA.cpu().numpy(), dB.cpu().numpy()
    finally:
        deallocGEMMContext(ctx)


def errors(x, x64, scale):
    normwise = float(np.max(np.abs(x - x64)) / max(np.max(np.abs(x64)), 1e-300))
    elementwise = float(np.max(np.abs(x - x64) / np.maximum(scale, 1e-300)))
    return normwise, elementwise


def check(A, B, wA, eA, wB, eB, dC):
    Av = O.decode_values(A, wA, eA != "u")
    Bv = O.decode_values(B, wB, eB != "u")
    dA, dB = run_adjoint(A, B, wA, eA, wB, eB, dC)
    dA64, dB64 = O.adjoint_fp64(dC, Av, Bv)
    sA = np.abs(dC.astype(np.float64)).T @ np.abs(Bv.astype(np.float64))
    sB = np.abs(dC.astype(np.float64)) @ np.abs(Av.astype(np.float64))
    ea = errors(dA.astype(np.float64), dA64, sA)
    eb = errors(dB.astype(np.float64), dB64, sB)
    return ea, eb


@pytest.mark.parametrize("enc", [(2, "u", 1, "b"), (3, "u", 2, "s"), (1, "b", 1, "b"), (1, "b", 4, "s"),
                                 (4, "s", 3, "u"), (8, "s", 8, "u"), (1, "u", 1, "u")])
def test_adjoint_matches_fp64(enc, adjoint_pipe):
    wA, eA, wB, eB = enc
    rng = np.random.default_rng(wA * 10 + wB)
    for (M, K, N) in [(96, 320, 80), (130, 1000, 257), (1, 64, 3), (300, 131, 7), (257, 700, 333)]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wA, eA)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wB, eB)
        dC = datagen.normal_f32(int(rng.integers(1 << 30)), (N, M))
        (na, ea), (nb, eb) = check(A, B, wA, eA, wB, eB, dC)
        assert na < TOL and ea < TOL and nb < TOL and eb < TOL, (enc, (M, K, N), na, ea, nb, eb)


def test_adjoint_qat_layer_full_size(adjoint_pipe):
    """The quantised-MLP layer: A 4096 x 2048 2-bit unsigned, B 2048 x 2048 bipolar, dC ~ N(0,1)."""
    M, K, N = 4096, 2048, 2048
    A = datagen.operand(datagen.SEED_BASE + 50, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 51, N, K, 1, "b")
    dC = datagen.normal_f32(datagen.SEED_BASE + 52, (N, M))
    (na, ea), (nb, eb) = check(A, B, 2, "u", 1, "b", dC)
    print(f"{adjoint_pipe}: dA normwise {na:.3e} elementwise {ea:.3e}; dB normwise {nb:.3e} elementwise {eb:.3e}")
    assert max(na, ea, nb, eb) < TOL


def test_adjoint_unit_step_finite_differences(adjoint_pipe):
    """L = sum dC * C is bilinear: one unit step of A[m,k] changes L by exactly dA[m,k]
    (a step of 2 for a bipolar entry changes it by 2*dB[n,k])."""
    import torch
    M, K, N = 64, 448, 48
    wA, eA, wB, eB = 2, "u", 1, "b"
    A = datagen.operand(datagen.SEED_BASE + 60, M, K, wA, eA)
    B = datagen.operand(datagen.SEED_BASE + 61, N, K, wB, eB)
    dC = datagen.normal_f32(datagen.SEED_BASE + 62, (N, M))
    dA, dB = run_adjoint(A, B, wA, eA, wB, eB, dC)

    def loss(A_, B_):
        ctx = allocGEMMContext(M, K, N, wA, wB, eA != "u", eB != "u")
        ctx.lhs.importRegular(A_)
        ctx.rhs.importRegular(B_)
        gemmBitSerial(ctx)
        res = ctx.res.reshape(N, M).astype(np.float64)
        deallocGEMMContext(ctx)
        return float((dC.astype(np.float64) * res).sum())

    L0 = loss(A, B)
    rng = np.random.default_rng(1)
    for _ in range(6):
        m, k = int(rng.integers(M)), int(rng.integers(K))
        step = -1 if A[m, k] == 3 else 1  # stay inside the 2-bit unsigned range
        A2 = A.copy()
        A2[m, k] += step
        fd = (loss(A2, B) - L0) / step
        assert abs(fd - dA[m, k]) <= 1e-5 * max(1.0, abs(fd)), (m, k, fd, dA[m, k])
        n, k = int(rng.integers(N)), int(rng.integers(K))
        B2 = B.copy()
        B2[n, k] = -B[n, k]  # bipolar: a step of +-2
        fd = (loss(A, B2) - L0) / (B2[n, k] - B[n, k])
        assert abs(fd - dB[n, k]) <= 1e-5 * max(1.0, abs(fd)), (n, k, fd, dB[n, k])


def test_autograd_binding():
    """torch.autograd through the binding matches float64 autograd of B @ A^T."""
    import torch
    from bitserial_autograd import BitSerialMatmul
    M, K, N = 40, 200, 24
    A = torch.from_numpy(datagen.operand(datagen.SEED_BASE + 70, M, K, 3, "s")).cuda().float()
    B = torch.from_numpy(datagen.operand(datagen.SEED_BASE + 71, N, K, 2, "u")).cuda().float()
    g = torch.randn(N, M, device="cuda", dtype=torch.float64)
    A1, B1 = A.clone().requires_grad_(True), B.clone().requires_grad_(True)
    out = BitSerialMatmul.apply(A1, B1, 3, True, 2, False)
    (out.double() * g).sum().backward()
    A2, B2 = A.double().requires_grad_(True), B.double().requires_grad_(True)
    ref = B2 @ A2.T
    (ref * g).sum().backward()
    assert torch.equal(out.double(), ref.detach())
    assert torch.allclose(A1.grad.double(), A2.grad, rtol=0, atol=1e-5 * float(A2.grad.abs().max()))
    assert torch.allclose(B1.grad.double(), B2.grad, rtol=0, atol=1e-5 * float(B2.grad.abs().max()))


def test_adjoint_rejects_host_pointers(lib):
    A = np.ones((4, 64), np.int8)
    ctx = allocGEMMContext(4, 64, 4, 1, 1, 0, 0)
    ctx.lhs.importRegular(A)
    ctx.rhs.importRegular(A)
    host = np.zeros((4, 64), np.float32)
    rc = lib.gbs_adjoint(ctx._h, C.c_void_p(host.ctypes.data), C.c_void_p(host.ctypes.data), None, None)
    assert rc == _capi.GBS_EINVAL
    deallocGEMMContext(ctx)


def test_adjoint_rejects_misaligned_pointers(lib):
    """dC, dA and dB must be 16-byte aligned (the kernels move 4 floats at a time): a pointer 4 bytes
    into a device buffer is refused on the host.  The outputs that would be written stay NULL or
    aligned-to-4 views, so even a missing check could not launch a misaligned vector access."""
    import torch
    M, K, N = 64, 128, 32
    A = datagen.operand(datagen.SEED_BASE + 90, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 91, N, K, 1, "b")
    ctx = allocGEMMContext(M, K, N, 2, 1, False, True)
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        d = torch.zeros(N * M + 4, dtype=torch.float32, device="cuda")
        out = torch.zeros(M * K + 4, dtype=torch.float32, device="cuda")
        rc = lib.gbs_adjoint(ctx._h, C.c_void_p(d.data_ptr() + 4), None, None, None)
        assert rc == _capi.GBS_EINVAL and b"aligned" in _capi.load().gbs_last_error()
        rc = lib.gbs_adjoint(ctx._h, C.c_void_p(d.data_ptr()), C.c_void_p(out.data_ptr() + 4), None, None)
        assert rc == _capi.GBS_EINVAL
        torch.cuda.synchronize()
    finally:
        deallocGEMMContext(ctx)


def test_adjoint_cache_follows_reimport(adjoint_pipe):
    """The tensor-core adjoint caches its transposed operand values; a new import replaces them."""
    import torch
    M, K, N = 200, 384, 130
    A1 = datagen.operand(datagen.SEED_BASE + 80, M, K, 3, "s")
    A2 = datagen.operand(datagen.SEED_BASE + 81, M, K, 3, "s")
    B1 = datagen.operand(datagen.SEED_BASE + 82, N, K, 2, "u")
    B2 = datagen.operand(datagen.SEED_BASE + 83, N, K, 2, "u")
    dC = datagen.normal_f32(datagen.SEED_BASE + 84, (N, M))
    ctx = allocGEMMContext(M, K, N, 3, 2, True, False)
    try:
        d = torch.from_numpy(dC).cuda()
        dA = torch.empty(M, K, device="cuda")
        dB = torch.empty(N, K, device="cuda")
        for A, B in [(A1, B1), (A2, B1), (A2, B2)]:
            ctx.lhs.importRegular(A)
            ctx.rhs.importRegular(B)
            _capi.check(_capi.load().gbs_adjoint(ctx._h, C.c_void_p(d.data_ptr()), C.c_void_p(dA.data_ptr()),
                                                 C.c_void_p(dB.data_ptr()), None))
            torch.cuda.synchronize()
            dA64, dB64 = O.adjoint_fp64(dC, O.decode_values(A, 3, True), O.decode_values(B, 2, False))
            assert np.max(np.abs(dA.cpu().numpy() - dA64)) <= 1e-6 * np.max(np.abs(dA64))
            assert np.max(np.abs(dB.cpu().numpy() - dB64)) <= 1e-6 * np.max(np.abs(dB64))
    finally:
        deallocGEMMContext(ctx)
