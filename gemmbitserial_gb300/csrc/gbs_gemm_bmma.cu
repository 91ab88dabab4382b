// gbs_gemm_bmma.cu -- forward bit-serial GEMM on the tensor pipe
// (mma.sync.m16n8k256 b1, AND + popcount, s32 accumulate).
//
// Same contract as the CUDA-core kernel (gbs_gemm_popc.cu): per plane pair
// (i, j) the MMA produces popc(A_i[m] AND B_j[n]) over a K chunk, which is
// folded into the int32 accumulator with the weight alpha[i][j].  Bipolar x
// bipolar uses AND with the identity xor = pa + pb - 2*and (the host passes
// alpha = 4 and the bipolar row sums), because b1 XOR.popc issues at half the
// AND rate on this GPU.
//
// CTA tile 128 (lhs rows) x 64 (rhs rows), 8 warps as 4 x 2, warp tile
// 32 x 32 (2 m16 x 4 n8 MMA tiles), K chunk 512 bits (two k256 steps), planes
// staged by cp.async into a 2-stage ring.  Shared rows are 64 bytes; the
// 16-byte chunk c of row r sits at chunk c ^ ((r >> 1) & 3), which makes every
// ldmatrix phase (8 rows x 16 bytes) hit distinct banks.
#include "gbs_internal.h"

namespace gbs {
namespace {

constexpr int BM = 128, BN = 64, KW = 8, NT = 256;  // KW: 64-bit words per chunk row
constexpr int ROWB = KW * 8;                        // bytes per staged row

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void *gmem, bool pred) {
  int sz = pred ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ uint32_t swz(int row, int chunk) {
  return (uint32_t)(row * ROWB + ((chunk ^ ((row >> 1) & 3)) << 4));
}
__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void bmma(int (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.and.popc {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(NT, 2) gemm_bmma_kernel(GemmShape g, Epilogue e) {
  extern __shared__ __align__(128) uint8_t smem[];
  const int wa = g.wa, wb = g.wb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;  // warp tile origin: rows 32*wm, cols 32*wn
  const uint64_t m0 = (uint64_t)blockIdx.x * BM, n0 = (uint64_t)blockIdx.y * BN;
  const uint64_t wpr = g.wpr;
  const int nchunks = (int)((wpr + KW - 1) / KW);
  const uint32_t a_tile = BM * ROWB, b_tile = BN * ROWB;
  const uint32_t stage_bytes = wa * a_tile + wb * b_tile;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);

  auto load_stage = [&](int st, uint64_t k0) {
    const uint32_t s = sbase + st * stage_bytes;
    const int a_pieces = wa * BM * (KW / 2), all = a_pieces + wb * BN * (KW / 2);
    for (int idx = tid; idx < all; idx += NT) {
      const bool isA = idx < a_pieces;
      const int li = isA ? idx : idx - a_pieces;
      const int rows = isA ? BM : BN;
      const int plane = li / (rows * (KW / 2)), rem = li % (rows * (KW / 2));
      const int row = rem / (KW / 2), c = rem % (KW / 2);
      const uint64_t k = k0 + 2 * c;
      const uint64_t grow = (isA ? m0 : n0) + row;
      const uint64_t *base = isA ? g.A + plane * g.a_plane : g.B + plane * g.b_plane;
      const uint32_t dst = s + (isA ? plane * a_tile : wa * a_tile + plane * b_tile) + swz(row, c);
      const bool ok = k < wpr && grow < (isA ? g.a_rows : g.b_rows);
      cp_async16(dst, ok ? base + grow * wpr + k : base, ok);
    }
  };

  uint32_t acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[i][j][r] = 0u;

  // per-lane ldmatrix row/chunk selectors
  const int q = lane >> 3, r8 = lane & 7;
  const int a_row = wm * 32 + (q & 1) * 8 + r8, a_chunk = q >> 1;  // + 16 rows for the 2nd m16 tile
  const int b_row = wn * 32 + (q >> 1) * 8 + r8, b_chunk = q & 1;  // + 16 rows for n8 tiles 2, 3

  if (nchunks > 0) {
    load_stage(0, 0);
    asm volatile("cp.async.commit_group;\n" ::);
  }
  for (int ch = 0; ch < nchunks; ch++) {
    if (ch + 1 < nchunks) {
      load_stage((ch + 1) & 1, (uint64_t)(ch + 1) * KW);
      asm volatile("cp.async.commit_group;\n" ::);
      asm volatile("cp.async.wait_group 1;\n" ::);
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::);
    }
    __syncthreads();
    const uint32_t s = sbase + (ch & 1) * stage_bytes;
#pragma unroll 1
    for (int i = 0; i < wa; i++) {
      uint32_t af[2][2][4];  // [k step][m16 tile][reg]
      const uint32_t at = s + i * a_tile;
#pragma unroll
      for (int ks = 0; ks < 2; ks++)
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
          ldsm_x4(at + swz(a_row + mt * 16, ks * 2 + a_chunk), af[ks][mt][0], af[ks][mt][1], af[ks][mt][2],
                  af[ks][mt][3]);
#pragma unroll 1
      for (int j = 0; j < wb; j++) {
        const uint32_t bt = s + wa * a_tile + j * b_tile;
        int t[2][4][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
          for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int r = 0; r < 4; r++) t[mt][nt][r] = 0;
#pragma unroll
        for (int ks = 0; ks < 2; ks++) {
          uint32_t bf[2][4];  // [n16 pair][b0 n, b1 n, b0 n+8, b1 n+8]
#pragma unroll
          for (int np = 0; np < 2; np++)
            ldsm_x4(bt + swz(b_row + np * 16, ks * 2 + b_chunk), bf[np][0], bf[np][1], bf[np][2], bf[np][3]);
#pragma unroll
          for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
              bmma(t[mt][nt], af[ks][mt], bf[nt >> 1][(nt & 1) * 2], bf[nt >> 1][(nt & 1) * 2 + 1]);
        }
        const uint32_t al = (uint32_t)e.alpha[i][j];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
          for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[mt][nt][r] += (uint32_t)t[mt][nt][r] * al;
      }
    }
    __syncthreads();
  }

  // epilogue: c0/c1 -> (row g, cols 2c, 2c+1), c2/c3 -> (row g+8, same cols)
  const int gq = lane >> 2, cq = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const uint64_t gm = m0 + wm * 32 + mt * 16 + gq + (r >> 1) * 8;
        const uint64_t gn = n0 + wn * 32 + nt * 8 + cq * 2 + (r & 1);
        if (gm < g.M && gn < g.N) {
          const uint32_t v = acc[mt][nt][r] + e.c0 - (e.ra ? (uint32_t)e.ra[gm] : 0u) -
                             (e.rb ? (uint32_t)e.rb[gn] : 0u);
          g.C[gn * g.M + gm] = (int32_t)v;
        }
      }
}

}  // namespace

bool bmma_supported(int wa, int wb, int) { return wa >= 1 && wa <= kMaxBits && wb >= 1 && wb <= kMaxBits; }

cudaError_t launch_gemm_bmma(const GemmShape &g, const Epilogue &e, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  const size_t smem = 2ull * (g.wa * BM + g.wb * BN) * ROWB;
  cudaError_t err = cudaFuncSetAttribute(gemm_bmma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  dim3 grid((unsigned)((g.M + BM - 1) / BM), (unsigned)((g.N + BN - 1) / BN));
  gemm_bmma_kernel<<<grid, NT, smem, s>>>(g, e);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs
