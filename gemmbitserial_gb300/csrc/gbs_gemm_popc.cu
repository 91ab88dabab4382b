// gbs_gemm_popc.cu -- forward bit-serial GEMM on the CUDA cores (LOP3 + POPC).
//
// Computes, for every plane pair (i, j), popc(A_i[m] AND B_j[n]) (XOR for
// bipolar x bipolar) and folds the weights of gemmBitSerial_generic_usingBinary
// (arch-generic.hpp:169-193: +-2^(i+j), negative for a signed MSB plane,
// doubled for bipolar x regular), the bipolar x regular accumulator seed
// (-rowsum, arch-generic.hpp:45-71) and the bipolar x bipolar correction
// (ncols - 2*xor, arch-generic.hpp:255-259) into one int32 epilogue.  All
// arithmetic is modulo 2^32, as the reference's int32 accumulators.
//
// Two kernels:
//  * gemm_popc_tiled: 64 x 64 output tile per 256-thread CTA, 4 x 4 outputs
//    per thread, planes staged through shared memory by cp.async in K chunks
//    (double buffered).  Thread (tx, ty) owns lhs rows tx + 16i and rhs rows
//    ty + 16j, so a half-warp stores 16 consecutive results of the
//    transposed output row.
//  * gemm_popc_skinny: one warp per output element, lanes stride over the K
//    words; for matrix-vector and other small-output shapes.
#include "gbs_internal.h"

namespace gbs {
namespace {

constexpr int BM = 64, BN = 64, NT = 256;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool pred) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = pred ? 16 : 0;  // src-size 0 zero-fills the destination
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <bool XOR>
__device__ __forceinline__ uint32_t pc2(ulonglong2 a, ulonglong2 b) {
  if (XOR) return __popcll(a.x ^ b.x) + __popcll(a.y ^ b.y);
  return __popcll(a.x & b.x) + __popcll(a.y & b.y);
}

template <bool XOR, int KC>
__global__ void __launch_bounds__(NT, 2) gemm_popc_tiled(GemmShape g, Epilogue e) {
  constexpr int LDW = KC + 2;  // padded row stride (words): conflict-free 16-byte reads
  const int wa = g.wa, wb = g.wb;
  extern __shared__ __align__(16) uint64_t smem[];
  const int stage_words = (wa * BM + wb * BN) * LDW;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const uint64_t m0 = (uint64_t)blockIdx.x * BM, n0 = (uint64_t)blockIdx.y * BN;
  const uint64_t wpr = g.wpr;
  const int nchunks = (int)((wpr + KC - 1) / KC);

  auto load_stage = [&](int st, uint64_t k0) {
    uint64_t *s = smem + st * stage_words;
    const int per_row = KC / 2;  // 16-byte pieces per row
    const int a_pieces = wa * BM * per_row, all = a_pieces + wb * BN * per_row;
    for (int idx = tid; idx < all; idx += NT) {
      const bool isA = idx < a_pieces;
      const int li = isA ? idx : idx - a_pieces;
      const int plane = li / (BM * per_row), rem = li % (BM * per_row);
      const int row = rem / per_row, p = rem % per_row;
      const uint64_t k = k0 + 2 * p;
      const uint64_t *src = isA ? g.A + plane * g.a_plane + (m0 + row) * wpr
                                : g.B + plane * g.b_plane + (n0 + row) * wpr;
      uint64_t *dst = s + (isA ? 0 : wa * BM * LDW) + (plane * BM + row) * LDW + 2 * p;
      const bool ok = k < wpr;
      cp_async16(dst, ok ? src + k : src, ok);
    }
  };

  uint32_t acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0u;

  if (nchunks > 0) {
    load_stage(0, 0);
    cp_commit();
  }
  for (int c = 0; c < nchunks; c++) {
    if (c + 1 < nchunks) {
      load_stage((c + 1) & 1, (uint64_t)(c + 1) * KC);
      cp_commit();
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const uint64_t *sa = smem + (c & 1) * stage_words;
    const uint64_t *sb = sa + wa * BM * LDW;
#pragma unroll 1
    for (int i = 0; i < wa; i++) {
#pragma unroll 1
      for (int j = 0; j < wb; j++) {
        uint32_t t[4][4];
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
          for (int n = 0; n < 4; n++) t[m][n] = 0u;
        const uint64_t *pa = sa + (i * BM + tx) * LDW;
        const uint64_t *pb = sb + (j * BN + ty) * LDW;
#pragma unroll 2
        for (int kp = 0; kp < KC / 2; kp++) {
          ulonglong2 a[4], b[4];
#pragma unroll
          for (int m = 0; m < 4; m++) a[m] = *reinterpret_cast<const ulonglong2 *>(pa + m * 16 * LDW + 2 * kp);
#pragma unroll
          for (int n = 0; n < 4; n++) b[n] = *reinterpret_cast<const ulonglong2 *>(pb + n * 16 * LDW + 2 * kp);
#pragma unroll
          for (int m = 0; m < 4; m++)
#pragma unroll
            for (int n = 0; n < 4; n++) t[m][n] += pc2<XOR>(a[m], b[n]);
        }
        const uint32_t al = (uint32_t)e.alpha[i][j];
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
          for (int n = 0; n < 4; n++) acc[m][n] += t[m][n] * al;
      }
    }
    __syncthreads();
  }

#pragma unroll
  for (int n = 0; n < 4; n++) {
    const uint64_t gn = n0 + ty + 16 * n;
    if (gn >= g.N) continue;
    const uint32_t bn = e.c0 - (e.rb ? (uint32_t)e.rb[gn] : 0u);
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const uint64_t gm = m0 + tx + 16 * m;
      if (gm >= g.M) continue;
      const uint32_t v = acc[m][n] + bn - (e.ra ? (uint32_t)e.ra[gm] : 0u);
      g.C[gn * g.M + gm] = (int32_t)v;
    }
  }
}

// One warp per output (m, n); lanes stride over the K words.
__global__ void __launch_bounds__(256) gemm_popc_skinny(GemmShape g, Epilogue e) {
  const uint64_t o = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (o >= g.M * g.N) return;  // warp-uniform
  const uint64_t n = o / g.M, m = o % g.M;
  uint32_t acc = 0;
  for (int i = 0; i < g.wa; i++) {
    const uint64_t *a = g.A + i * g.a_plane + m * g.wpr;
    for (int j = 0; j < g.wb; j++) {
      const uint64_t *b = g.B + j * g.b_plane + n * g.wpr;
      uint32_t cnt = 0;
      if (e.use_xor) {
        for (uint64_t w = lane; w < g.wpr; w += 32) cnt += __popcll(a[w] ^ b[w]);
      } else {
        for (uint64_t w = lane; w < g.wpr; w += 32) cnt += __popcll(a[w] & b[w]);
      }
      acc += cnt * (uint32_t)e.alpha[i][j];
    }
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if (lane == 0) {
    uint32_t v = acc + e.c0 - (e.ra ? (uint32_t)e.ra[m] : 0u) - (e.rb ? (uint32_t)e.rb[n] : 0u);
    g.C[n * g.M + m] = (int32_t)v;
  }
}

template <bool XOR, int KC>
cudaError_t run_tiled(const GemmShape &g, const Epilogue &e, cudaStream_t s) {
  const size_t smem = 2ull * (g.wa * BM + g.wb * BN) * (KC + 2) * sizeof(uint64_t);
  auto kern = gemm_popc_tiled<XOR, KC>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  dim3 grid((unsigned)((g.M + BM - 1) / BM), (unsigned)((g.N + BN - 1) / BN));
  kern<<<grid, NT, smem, s>>>(g, e);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gemm_popc(const GemmShape &g, const Epilogue &e, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  const bool skinny = (g.M * g.N <= 32768) || g.M < 16 || g.N < 16;
  if (skinny) {
    const uint64_t threads = g.M * g.N * 32;
    gemm_popc_skinny<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(g, e);
    count_launch();
    return cudaGetLastError();
  }
  if (e.use_xor) return run_tiled<true, 16>(g, e, s);
  const int planes = g.wa + g.wb;
  if (planes <= 6) return run_tiled<false, 16>(g, e, s);
  if (planes <= 12) return run_tiled<false, 8>(g, e, s);
  return run_tiled<false, 4>(g, e, s);
}

}  // namespace gbs
