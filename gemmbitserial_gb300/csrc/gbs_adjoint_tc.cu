// gbs_adjoint_tc.cu -- the FP32 adjoint of the bit-serial GEMM on the
// 5th-generation tensor cores, with an exact bf16 split of dC.
//
// No reference counterpart (the reference has no backward pass).  With the
// forward res[n, m] = sum_k A[m, k] * B[n, k] and an FP32 upstream gradient
// dC in the result layout dC[n*M + m]:
//   dA[m, k] = sum_n dC[n, m] * B[n, k]      (M x K, row-major)
//   dB[n, k] = sum_m dC[n, m] * A[m, k]      (N x K, row-major)
// where A and B are the values the planes encode (gemmbitserial.hpp:313-333):
// sum_j s_j 2^j bit_j, s_j = -1 for a signed MSB plane; 2*bit - 1 for bipolar.
//
// Exactness of the operands: every value has at most 8 significant bits, so
// it is exact in bf16.  dC is split as dC = hi + mid + lo with hi = bf16(dC),
// mid = bf16(dC - hi), lo = bf16(dC - hi - mid); each residual is exact in
// fp32 and the three bf16 terms carry all 24 bits of the fp32 significand.
// Every product (8 x 8 significant bits) is exact in fp32.  The tensor core
// accumulates hi*V in one fp32 TMEM accumulator and (mid + lo)*V, 2^-8 of its
// size, in a second; the epilogue adds the two.  So the only rounding is the
// fp32 accumulation itself, done 16 products per MMA step.
//
// Both products are "Out[r, k] = sum_s X[r, s] * Vt[k, s]" with both operands
// contraction-major in HBM: pre-passes write the three splits of dC as
// [N][M] (dB: r = n, s = m) and transposed as [M][N] (dA: r = m, s = n), and
// the operand values transposed as Vt[k][s] in bf16.
//
// GEMM kernel: CTA tile 128 rows (r) x 256 columns (k), 32 values of s per
// stage in a 5-stage ring: TMA loads the three 128 x 32 split tiles and the
// 256 x 32 value tile (64-byte swizzle), warp 1 issues 6 tcgen05.mma.kind::f16
// (M=128, N=256, K=16) per stage into the two accumulators (all 512 TMEM
// columns), warps 2-5 add the accumulators and store through a padded
// shared-memory tile so that each warp store covers 128 contiguous bytes of a
// row of Out.  Every mbarrier wait is bounded.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>

#include "gbs_internal.h"
#include "gbs_tc_common.cuh"

namespace gbs {
namespace {

constexpr int kAdjThreads = 192;
constexpr uint32_t kAdjScratchFloats = 32 * 33;          // per epilogue warp

// Ring: 32 values of s per stage (64-byte rows, 64-byte swizzle), 5 stages of
// 40 KB.  Two stages of 64 values (80 KB, 128-byte rows) hold the same bytes
// but free them half as often; that ring ran the GEMMs latency-bound, 15 %
// slower per adjoint.
constexpr int kAdjKs = 32;
constexpr int kAdjStages = 5;
constexpr uint32_t kAdjSplitBytes = 128 * kAdjKs * 2;  // 128 rows x 32 bf16
constexpr uint32_t kAdjValBytes = 256 * kAdjKs * 2;    // 256 rows x 32 bf16
constexpr uint32_t kAdjStageBytes = 3 * kAdjSplitBytes + kAdjValBytes;

constexpr size_t adj_smem_bytes() {
  return 1024 + kAdjStages * kAdjStageBytes + 4 * kAdjScratchFloats * 4 + 8 * (2 * kAdjStages + 2) + 16;
}
static_assert(adj_smem_bytes() <= 232448, "shared memory per CTA");

struct AdjTcArgs {
  float *out;  // R x K row-major
  uint32_t R, K, nstages;
  uint32_t idesc;
};

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}

__global__ void __launch_bounds__(kAdjThreads, 1)
    adjoint_tc_kernel(const __grid_constant__ CUtensorMap tmHi, const __grid_constant__ CUtensorMap tmMid,
                      const __grid_constant__ CUtensorMap tmLo, const __grid_constant__ CUtensorMap tmV, AdjTcArgs a,
                      uint32_t *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float *scratch = reinterpret_cast<float *>(smem + kAdjStages * kAdjStageBytes);
  uint64_t *bars = reinterpret_cast<uint64_t *>(scratch + 4 * kAdjScratchFloats);
  const uint32_t full = smem_u32(bars), empty = full + 8 * kAdjStages, acc_full = empty + 8 * kAdjStages;
  const uint32_t mma_done = acc_full + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kAdjStages + 2);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint32_t r0 = blockIdx.x * 128, k0 = blockIdx.y * 256;

  if (tid == 0) {
    for (int i = 0; i < kAdjStages; i++) {
      mbar_init(full + 8 * i, 1);
      mbar_init(empty + 8 * i, 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;  // columns [0, 256): hi accumulator; [256, 512): mid + lo

  if (warp == 0) {
    if (lane == 0) {
      uint32_t issued = 0;
      for (uint32_t k = 0; k < a.nstages; k++) {
        const uint32_t s = k % kAdjStages, use = k / kAdjStages;
        if (use > 0 && !mbar_wait_err(empty + 8 * s, (use - 1) & 1, abort_flag, err)) break;
        mbar_expect_tx(full + 8 * s, kAdjStageBytes);
        const uint32_t dst = smem_u32(smem + s * kAdjStageBytes);
        const int x = (int)(k * kAdjKs);
        tma_load_2d(dst, &tmHi, x, (int)r0, full + 8 * s);
        tma_load_2d(dst + kAdjSplitBytes, &tmMid, x, (int)r0, full + 8 * s);
        tma_load_2d(dst + 2 * kAdjSplitBytes, &tmLo, x, (int)r0, full + 8 * s);
        tma_load_2d(dst + 3 * kAdjSplitBytes, &tmV, x, (int)k0, full + 8 * s);
        issued = k + 1;
      }
      if (*abort_flag)
        for (uint32_t k = (issued > (uint32_t)kAdjStages ? issued - kAdjStages : 0); k < issued; k++)
          mbar_drain_err(full + 8 * (k % kAdjStages), (k / kAdjStages) & 1, err);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      for (uint32_t k = 0; k < a.nstages && ok; k++) {
        const uint32_t s = k % kAdjStages;
        if (!mbar_wait_err(full + 8 * s, (k / kAdjStages) & 1, abort_flag, err)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = smem_u32(smem + s * kAdjStageBytes), vb = base + 3 * kAdjSplitBytes;
#pragma unroll
        for (int kk = 0; kk < kAdjKs / 16; kk++) {  // K = 16 per MMA: 32 bytes along the row
          const uint64_t bd = sw64_desc(vb + kk * 32);
          const uint32_t first = (k | kk) != 0;
          mma_bf16(tmem, sw64_desc(base + kk * 32), bd, a.idesc, first);
          mma_bf16(tmem + 256, sw64_desc(base + kAdjSplitBytes + kk * 32), bd, a.idesc, first);
          mma_bf16(tmem + 256, sw64_desc(base + 2 * kAdjSplitBytes + kk * 32), bd, a.idesc, 1u);
        }
        mma_commit(empty + 8 * s);
      }
      if (ok) {
        mma_commit(acc_full);
      } else {  // issued MMAs finish before TMEM is freed
        mma_commit(mma_done);
        mbar_drain_err(mma_done, 0, err);
      }
    }
  } else {
    if (__all_sync(0xffffffffu, mbar_wait_err(acc_full, 0, abort_flag, err))) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int q = warp & 3;
      float *sc = scratch + (warp - 2) * kAdjScratchFloats;  // [32 rows][33]
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (uint32_t c = 0; c < 256; c += 32) {
        uint32_t hi[32], lo[32];
        tmem_ld32(taddr + c, hi);
        tmem_ld32(taddr + 256 + c, lo);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; j++) sc[lane * 33 + j] = __uint_as_float(hi[j]) + __uint_as_float(lo[j]);
        __syncwarp();
        // rows r0 + 32q .. +31 of this column block: one base pointer, a fixed
        // row stride, no per-element predicate when all 32 rows exist
        const uint32_t col = k0 + c + lane, row0 = r0 + q * 32;
        if (col < a.K) {
          float *p = a.out + (uint64_t)row0 * a.K + col;
          const uint64_t K = a.K;
          if (row0 + 32 <= a.R) {
#pragma unroll 8
            for (int i = 0; i < 32; i++) p[(uint64_t)i * K] = sc[i * 33 + lane];
          } else {
#pragma unroll 4
            for (int i = 0; i < 32; i++)
              if (row0 + i < a.R) p[(uint64_t)i * K] = sc[i * 33 + lane];
          }
        }
        __syncwarp();
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  }
}

// ------------------------------------------------------------ pre-passes
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
  h = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(h);
  m = __float2bfloat16_rn(r1);
  l = __float2bfloat16_rn(r1 - __bfloat162float(m));
}

// dC [N][M] -> hi/mid/lo in both orientations: [N][pM] (rows n) and [M][pN]
// (rows m).  A block takes 64 x 64 elements: 16 consecutive m per thread in,
// 16 consecutive n per thread out of the transposed tile, 16-byte stores.
// 16 bf16 values, packed two per word (element 2i in the low half of w[i]).
__device__ __forceinline__ void store16(__nv_bfloat16 *dst, const uint32_t (&w)[8], uint32_t valid) {
  if (valid >= 16) {
    reinterpret_cast<uint4 *>(dst)[0] = make_uint4(w[0], w[1], w[2], w[3]);
    reinterpret_cast<uint4 *>(dst)[1] = make_uint4(w[4], w[5], w[6], w[7]);
  } else {
    unsigned short *d16 = reinterpret_cast<unsigned short *>(dst);
#pragma unroll
    for (int j = 0; j < 16; j++)
      if ((uint32_t)j < valid) d16[j] = (unsigned short)(w[j >> 1] >> (16 * (j & 1)));
  }
}

__device__ __forceinline__ uint32_t bf16_bits(__nv_bfloat16 x) { return (uint32_t)__bfloat16_as_ushort(x); }

// The three split terms of 16 values, packed for store16.
__device__ __forceinline__ void split16(const float (&x)[16], uint32_t (&h)[8], uint32_t (&m)[8], uint32_t (&l)[8]) {
#pragma unroll
  for (int i = 0; i < 8; i++) {
    __nv_bfloat16 h0, m0, l0, h1, m1, l1;
    split3(x[2 * i], h0, m0, l0);
    split3(x[2 * i + 1], h1, m1, l1);
    h[i] = bf16_bits(h0) | (bf16_bits(h1) << 16);
    m[i] = bf16_bits(m0) | (bf16_bits(m1) << 16);
    l[i] = bf16_bits(l0) | (bf16_bits(l1) << 16);
  }
}

__global__ void __launch_bounds__(256) split_kernel(const float *__restrict__ dC, uint32_t N, uint32_t M, uint32_t pM,
                                                    uint32_t pN, int want_d, int want_t,
                                                    __nv_bfloat16 *__restrict__ dh, __nv_bfloat16 *__restrict__ dm,
                                                    __nv_bfloat16 *__restrict__ dl, __nv_bfloat16 *__restrict__ th,
                                                    __nv_bfloat16 *__restrict__ tm, __nv_bfloat16 *__restrict__ tl) {
  __shared__ float t[64][65];
  const uint32_t m0 = blockIdx.x * 64;
  const int row = threadIdx.x >> 2, part = threadIdx.x & 3;
  for (uint32_t n0 = blockIdx.y * 64; n0 < N; n0 += gridDim.y * 64) {
    {
      const uint32_t n = n0 + row, mb = m0 + 16 * part;
      float x[16];
      const uint32_t valid = (n < N && mb < M) ? min(16u, M - mb) : 0u;
      if (valid == 16 && (M & 3) == 0) {
        const float4 *src = reinterpret_cast<const float4 *>(dC + (uint64_t)n * M + mb);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const float4 v = src[i];
          x[4 * i] = v.x; x[4 * i + 1] = v.y; x[4 * i + 2] = v.z; x[4 * i + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++) x[j] = (uint32_t)j < valid ? dC[(uint64_t)n * M + mb + j] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < 16; j++) t[row][16 * part + j] = x[j];
      if (want_d && valid) {
        uint32_t h[8], m[8], l[8];
        split16(x, h, m, l);
        const uint64_t o = (uint64_t)n * pM + mb;
        store16(dh + o, h, valid);
        store16(dm + o, m, valid);
        store16(dl + o, l, valid);
      }
    }
    __syncthreads();
    if (want_t) {
      const uint32_t m = m0 + row, nb = n0 + 16 * part;
      const uint32_t valid = (m < M && nb < N) ? min(16u, N - nb) : 0u;
      if (valid) {
        float x[16];
#pragma unroll
        for (int j = 0; j < 16; j++) x[j] = t[16 * part + j][row];
        uint32_t h[8], md[8], l[8];
        split16(x, h, md, l);
        const uint64_t o = (uint64_t)m * pN + nb;
        store16(th + o, h, valid);
        store16(tm + o, md, valid);
        store16(tl + o, l, valid);
      }
    }
    __syncthreads();
  }
}

// Operand values, transposed: planes (rows s < S, columns k < K) -> Vt[k][s]
// in bf16 with row pitch pS.  A block decodes 64 rows x 64 columns (one plane
// word per row) through shared memory; threads store 16 consecutive s.
__global__ void __launch_bounds__(256) values_t_kernel(const uint64_t *__restrict__ planes, uint64_t plane_words,
                                                       uint64_t wpr, int nbits, int neg_msb, int bipolar, uint32_t S,
                                                       uint32_t K, uint32_t pS, __nv_bfloat16 *__restrict__ vt) {
  __shared__ __align__(16) __nv_bfloat16 t[64][72];  // [k][s], 144-byte rows
  const uint32_t kw = blockIdx.x;
  const int hi = threadIdx.x >> 2, part = threadIdx.x & 3;
  for (uint32_t s0 = blockIdx.y * 64; s0 < S; s0 += gridDim.y * 64) {
    {
      const uint32_t s = s0 + hi;  // this thread: row s, columns 16*part .. +16 of word kw
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = 0.f;
      if (s < S) {
        for (int b = 0; b < nbits; b++) {
          const uint32_t bits = (uint32_t)(planes[b * plane_words + (uint64_t)s * wpr + kw] >> (16 * part)) & 0xFFFFu;
          const float w = bipolar ? 2.f : (b == neg_msb ? -(float)(1 << b) : (float)(1 << b));
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] += ((bits >> j) & 1u) ? w : 0.f;
        }
        if (bipolar) {
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] -= 1.f;
        }
      }
#pragma unroll
      for (int j = 0; j < 16; j++) t[16 * part + j][hi] = __float2bfloat16_rn(v[j]);
    }
    __syncthreads();
    {
      const uint32_t k = kw * 64 + hi, sb = s0 + 16 * part;  // this thread: row k, s = sb .. +16
      const uint32_t valid = (k < K && sb < S) ? min(16u, S - sb) : 0u;
      if (valid) {
        const uint4 *src = reinterpret_cast<const uint4 *>(&t[hi][16 * part]);
        const uint4 a0 = src[0], a1 = src[1];
        const uint32_t o[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        store16(vt + (uint64_t)k * pS + sb, o, valid);
      }
    }
    __syncthreads();
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn adj_encode_fn() {
  static std::atomic<EncodeTiledFn> fn{nullptr};  // racing first calls store the same value
  EncodeTiledFn f = fn.load(std::memory_order_relaxed);
  if (!f) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess) {
      f = (EncodeTiledFn)p;
      fn.store(f, std::memory_order_relaxed);
    } else {
      cudaGetLastError();
    }
  }
  return f;
}

// 2-D bf16 map over [rows][cols] (row pitch `pitch` elements), box 32 x box_rows
// (64-byte rows), 64-byte swizzle.
bool bf16_map(CUtensorMap *map, const void *base, uint64_t cols, uint64_t rows, uint64_t pitch, uint32_t box_rows) {
  EncodeTiledFn fn = adj_encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {pitch * 2};
  cuuint32_t box[2] = {(cuuint32_t)kAdjKs, box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

uint64_t pitch8(uint64_t x) { return (x + 7) / 8 * 8; }

}  // namespace

// Workspace of a context's tensor-core adjoint: the splits of dC in both
// orientations and both operands' transposed values, with their tensor maps.
struct AdjPlan {
  __nv_bfloat16 *ws = nullptr;
  __nv_bfloat16 *split_d[3] = {};  // [N][pM]  (dB)
  __nv_bfloat16 *split_t[3] = {};  // [M][pN]  (dA)
  __nv_bfloat16 *vt_b = nullptr;   // B values [K][pN] (dA)
  __nv_bfloat16 *vt_a = nullptr;   // A values [K][pM] (dB)
  CUtensorMap map_d[3], map_t[3], map_vb, map_va;
  // dB runs on a second, high-priority stream, forked from and joined back to
  // the caller's, so that dA's kernels fill the SMs dB's leave idle
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

void adj_plan_free(AdjPlan *p) {
  if (!p) return;
  if (p->ws) cudaFree(p->ws);
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->join) cudaEventDestroy(p->join);
  if (p->side) cudaStreamDestroy(p->side);
  delete p;
}

bool adjoint_tc_available() { return adj_encode_fn() != nullptr; }

namespace {

int build_plan(gbs_ctx *c) {
  const uint64_t M = c->lhs.nrows, N = c->rhs.nrows, K = c->lhs.ncols;
  const uint64_t pM = pitch8(M), pN = pitch8(N);
  const uint64_t n_d = N * pM, n_t = M * pN, n_vb = K * pN, n_va = K * pM;
  AdjPlan *p = new AdjPlan();
  const size_t bytes = (3 * n_d + 3 * n_t + n_vb + n_va + 64) * sizeof(__nv_bfloat16);
  if (dev_alloc((void **)&p->ws, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return fail(GBS_ENOMEM, "gbs_adjoint: workspace allocation failed");
  }
  // every array starts on a 128-byte boundary
  uint8_t *q = reinterpret_cast<uint8_t *>(p->ws);
  auto take = [&](uint64_t elems) {
    __nv_bfloat16 *r = reinterpret_cast<__nv_bfloat16 *>(q);
    q += (elems * 2 + 127) / 128 * 128;
    return r;
  };
  for (int i = 0; i < 3; i++) p->split_d[i] = take(n_d);
  for (int i = 0; i < 3; i++) p->split_t[i] = take(n_t);
  p->vt_b = take(n_vb);
  p->vt_a = take(n_va);
  bool ok = true;
  for (int i = 0; i < 3; i++) {
    ok = ok && bf16_map(&p->map_d[i], p->split_d[i], M, N, pM, 128);  // dB: rows n, contraction m
    ok = ok && bf16_map(&p->map_t[i], p->split_t[i], N, M, pN, 128);  // dA: rows m, contraction n
  }
  ok = ok && bf16_map(&p->map_vb, p->vt_b, N, K, pN, 256);
  ok = ok && bf16_map(&p->map_va, p->vt_a, M, K, pM, 256);
  if (!ok) {
    adj_plan_free(p);
    return fail(GBS_EUNSUPPORTED, "gbs_adjoint: tensor map encoding failed");
  }
  // the side stream runs dB, whose tiles contract over M (twice as many
  // stages as dA's at the benchmark shape): at the highest priority its
  // long tiles are placed first and dA's shorter ones fill around them
  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&p->side, cudaStreamNonBlocking, greatest);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    adj_plan_free(p);
    return cuda_fail(e, "gbs_adjoint: stream/event creation");
  }
  c->adj = p;
  return GBS_OK;
}

cudaError_t launch_values_t(const Mat &op, __nv_bfloat16 *vt, uint64_t pS, cudaStream_t s) {
  const int neg = (op.issigned && !op.bipolar()) ? (int)op.nbits - 1 : -1;
  dim3 grid((unsigned)op.wpr(), (unsigned)std::min<uint64_t>((op.nrows + 63) / 64, 65535));
  values_t_kernel<<<grid, 256, 0, s>>>(op.planes, op.nrows_a * op.wpr(), op.wpr(), (int)op.nbits, neg,
                                       op.bipolar() ? 1 : 0, (uint32_t)op.nrows, (uint32_t)op.ncols, (uint32_t)pS, vt);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_gemm(const CUtensorMap (&split)[3], const CUtensorMap &vmap, uint64_t R, uint64_t S, uint64_t K,
                        float *out, cudaStream_t s) {
  AdjTcArgs a;
  a.out = out;
  a.R = (uint32_t)R;
  a.K = (uint32_t)K;
  a.nstages = (uint32_t)((S + kAdjKs - 1) / kAdjKs);
  // kind::f16: D fp32, A and B bf16, both K-major, M = 128, N = 256
  a.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
  uint32_t *err = tc_error_ptr();
  if (!err) return cudaErrorInvalidSymbol;
  cudaError_t e =
      cudaFuncSetAttribute(adjoint_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_smem_bytes());
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((R + 127) / 128), (unsigned)((K + 255) / 256));
  adjoint_tc_kernel<<<grid, kAdjThreads, adj_smem_bytes(), s>>>(split[0], split[1], split[2], vmap, a, err);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

// dA = dC . B and dB = dC^T . A on the tensor cores (either output may be null).
int adjoint_tc(gbs_ctx *c, const float *dC, float *dA, float *dB, cudaStream_t s) {
  const uint64_t M = c->lhs.nrows, N = c->rhs.nrows, K = c->lhs.ncols;
  if (M * K + N * K == 0) return GBS_OK;
  if (M == 0 || N == 0) {  // an empty contraction: zero gradients
    cudaError_t e = cudaSuccess;
    if (dA && M && K) e = cudaMemsetAsync(dA, 0, M * K * 4, s);
    if (e == cudaSuccess && dB && N && K) e = cudaMemsetAsync(dB, 0, N * K * 4, s);
    return e == cudaSuccess ? GBS_OK : cuda_fail(e, "gbs_adjoint: memset");
  }
  if (!c->adj) {
    const int rc = build_plan(c);
    if (rc != GBS_OK) return rc;
  }
  AdjPlan &p = *c->adj;
  const uint64_t pM = pitch8(M), pN = pitch8(N);
  dim3 sg((unsigned)((M + 63) / 64), (unsigned)std::min<uint64_t>((N + 63) / 64, 65535));
  cudaError_t e = cudaSuccess;
  // dB on the high-priority side stream, enqueued first: its split of dC,
  // A's values, the GEMM
  if (dB) {
    e = cudaEventRecord(p.fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p.side, p.fork, 0);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_adjoint: stream fork");
    split_kernel<<<sg, 256, 0, p.side>>>(dC, (uint32_t)N, (uint32_t)M, (uint32_t)pM, (uint32_t)pN, 1, 0, p.split_d[0],
                                         p.split_d[1], p.split_d[2], p.split_t[0], p.split_t[1], p.split_t[2]);
    count_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess && !c->vt_valid[0]) {  // operand values: rebuilt only after an import
      e = launch_values_t(c->lhs, p.vt_a, pM, p.side);
      c->vt_valid[0] = e == cudaSuccess;
    }
    if (e == cudaSuccess) e = launch_gemm(p.map_d, p.map_va, N, M, K, dB, p.side);
    if (e == cudaSuccess) e = cudaEventRecord(p.join, p.side);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_adjoint: dB kernels");
  }
  // dA on the caller's stream: its split of dC (transposed), B's values, the GEMM
  if (dA) {
    split_kernel<<<sg, 256, 0, s>>>(dC, (uint32_t)N, (uint32_t)M, (uint32_t)pM, (uint32_t)pN, 0, 1, p.split_d[0],
                                    p.split_d[1], p.split_d[2], p.split_t[0], p.split_t[1], p.split_t[2]);
    count_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess && !c->vt_valid[1]) {
      e = launch_values_t(c->rhs, p.vt_b, pN, s);
      c->vt_valid[1] = e == cudaSuccess;
    }
    if (e == cudaSuccess) e = launch_gemm(p.map_t, p.map_vb, M, N, K, dA, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_adjoint: dA kernels");
  }
  if (dB) {
    e = cudaStreamWaitEvent(s, p.join, 0);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_adjoint: stream join");
  }
  return GBS_OK;
}

}  // namespace gbs
