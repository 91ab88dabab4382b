"""Seeded, platform-independent synthetic inputs for the bit-serial GEMM.

All values come from a splitmix64 stream (one 64-bit draw per element), so the
same seed gives the same matrices on x86 and Arm.  Integer draws use the
multiply-shift map ``lo + ((r >> 32) * span) >> 32``.

The named workloads mirror the reference's benchmark shapes and encodings:
the rhs is always supplied transposed (N x K row-major, i.e. B column-major),
as ``gemmbitserial`` requires (README.md:9-10, arch-generic.hpp:165-168).
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 0x6762730000

_G = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """``n`` consecutive splitmix64 outputs of stream ``seed`` starting at ``offset``."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform_int(seed: int, shape, lo: int, hi: int, dtype=np.int8) -> np.ndarray:
    """Integers uniform in [lo, hi] (inclusive)."""
    n = int(np.prod(shape))
    out = np.empty(n, dtype=dtype)
    span = np.uint64(hi - lo + 1)
    step = 1 << 22
    for o in range(0, n, step):
        r = splitmix64(seed, min(step, n - o), o) >> np.uint64(32)
        out[o:o + len(r)] = (np.int64(lo) + ((r * span) >> np.uint64(32)).astype(np.int64)).astype(dtype)
    return out.reshape(shape)


def bipolar(seed: int, shape, dtype=np.int8) -> np.ndarray:
    """Values in {-1, +1}, each +1 with probability 1/2."""
    return (uniform_int(seed, shape, 0, 1, np.int8) * 2 - 1).astype(dtype)


def normal_f32(seed: int, shape) -> np.ndarray:
    """Standard normal float32 values (Box-Muller over two uniform streams)."""
    n = int(np.prod(shape))
    u1 = ((splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) + 1.0) * (1.0 / 9007199254740992.0)
    u2 = (splitmix64(seed ^ 0x5A5A5A5A, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return z.astype(np.float32).reshape(shape)


def operand(seed: int, rows: int, cols: int, bits: int, enc: str, dtype=np.int8) -> np.ndarray:
    """A rows x cols operand with ``bits``-bit values in encoding ``enc``.

    enc: 'u' unsigned [0, 2^bits-1]; 's' signed [-2^(bits-1), 2^(bits-1)-1];
    'b' bipolar {-1,+1} (1-bit signed in the reference's sense).
    """
    if enc == "b":
        return bipolar(seed, (rows, cols), dtype)
    if enc == "s":
        return uniform_int(seed, (rows, cols), -(1 << (bits - 1)), (1 << (bits - 1)) - 1, dtype)
    return uniform_int(seed, (rows, cols), 0, (1 << bits) - 1, dtype)


# Named workloads.  Each entry: M, K, N, (wA, encA), (wB, encB).
WORKLOADS = {
    # 1-bit unsigned {0,1}, Bernoulli(0.5) bits.
    "gemm_8x8192x8_u1u1": (8, 8192, 8, (1, "u"), (1, "u")),
    # lhs 3-bit unsigned [0,7], rhs 2-bit signed [-2,1].
    "gemm_2048x4096x2048_u3s2": (2048, 4096, 2048, (3, "u"), (2, "s")),
    # binary-net layer, both operands bipolar {-1,+1}.
    "gemm_256x9216x4096_bpbp": (256, 9216, 4096, (1, "b"), (1, "b")),
    # bipolar activations times 4-bit signed [-8,7] weights.
    "gemm_256x9216x4096_bps4": (256, 9216, 4096, (1, "b"), (4, "s")),
    # forward of the adjoint layer: 2-bit unsigned activations, bipolar weights.
    "gemm_4096x2048x2048_u2bp": (4096, 2048, 2048, (2, "u"), (1, "b")),
    # the headline shape at 8-bit signed x 8-bit signed (wider than one e4m3 digit).
    "gemm_2048x4096x2048_s8s8": (2048, 4096, 2048, (8, "s"), (8, "s")),
}


# The reference's CaffeNet chain (benchmark.cpp:174-237): (M, K, N) of its 8
# GEMMs (conv layers as GEMMs, then the fully connected layers as GEMVs), all
# 2-bit unsigned weights (lhs) x 2-bit unsigned activations (rhs).
CAFFENET = [(96, 363, 3025), (256, 2400, 729), (384, 2304, 169), (384, 3456, 169),
            (256, 3456, 169), (4096, 9216, 1), (4096, 4096, 1), (1000, 4096, 1)]


def caffenet_mix():
    """The CaffeNet chain as a problem mix: (M, K, N, wA, encA, wB, encB)."""
    return [(M, K, N, 2, "u", 2, "u") for (M, K, N) in CAFFENET]


def workload(name: str, seed_index: int = 0):
    """Return (M, K, N, wA, sA, wB, sB, A, B) for a named workload; A is M x K, B is N x K (int8)."""
    M, K, N, (wA, eA), (wB, eB) = WORKLOADS[name]
    seed = SEED_BASE + seed_index
    A = operand(seed, M, K, wA, eA)
    B = operand(seed + 0x100, N, K, wB, eB)
    return M, K, N, wA, eA != "u", wB, eB != "u", A, B


def grouped_mix(seed: int = SEED_BASE + 4, count: int = 512, m_max: int = 256, k_words=(4, 128),
                n_range=(64, 4096)):
    """The grouped-GEMM problem mix: a list of (M, K, N, wA, encA, wB, encB).

    M = round(exp(U(0, ln m_max))) in [1, m_max] (log-uniform); K = 64 * U{k_words};
    N = U{n_range}; wA in {1, 2, 4}, wB in {1, 2, 3, 4}; encoding u / s / b with
    equal probability.  A bipolar draw forces w = 1.  A signed draw with w = 1
    becomes w = 2, because a 1-bit signed operand is bipolar by definition in
    gemmbitserial (gemmbitserial.hpp:74-76).
    """
    r = splitmix64(seed, count * 8).reshape(count, 8) >> np.uint64(11)
    u = r.astype(np.float64) / float(1 << 53)
    out = []
    for i in range(count):
        M = int(min(m_max, max(1, round(np.exp(u[i, 0] * np.log(m_max))))))
        K = 64 * (k_words[0] + int(u[i, 1] * (k_words[1] - k_words[0] + 1)))
        N = n_range[0] + int(u[i, 2] * (n_range[1] - n_range[0] + 1))
        wA = (1, 2, 4)[int(u[i, 3] * 3)]
        wB = (1, 2, 3, 4)[int(u[i, 4] * 4)]
        eA = "usb"[int(u[i, 5] * 3)]
        eB = "usb"[int(u[i, 6] * 3)]
        if eA == "b":
            wA = 1
        elif eA == "s" and wA == 1:
            wA = 2
        if eB == "b":
            wB = 1
        elif eB == "s" and wB == 1:
            wB = 2
        out.append((M, K, N, wA, eA, wB, eB))
    return out


def torch_operand(gen, rows: int, cols: int, bits: int, enc: str, device):
    """A rows x cols int8 CUDA tensor with the distribution of operand(), drawn by a torch generator."""
    import torch
    if enc == "b":
        return (torch.randint(0, 2, (rows, cols), generator=gen, device=device, dtype=torch.int8) * 2 - 1)
    if enc == "s":
        lo, hi = -(1 << (bits - 1)), (1 << (bits - 1)) - 1
    else:
        lo, hi = 0, (1 << bits) - 1
    return torch.randint(lo, hi + 1, (rows, cols), generator=gen, device=device, dtype=torch.int16).to(torch.int8)
