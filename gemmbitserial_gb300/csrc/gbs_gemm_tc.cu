// gbs_gemm_tc.cu -- forward bit-serial GEMM on the 5th-generation tensor cores
// (tcgen05.mma, TMEM accumulator, TMA staging).
//
// Every plane pair (i, j) is evaluated on the tensor pipe as a product of
// 0/1 matrices: a set bit of lhs plane i becomes the fp8 (e4m3) value
// s_i * 2^i and a set bit of rhs plane j becomes t_j * 2^j (s, t = -1 for a
// signed MSB plane, gemmbitserial.hpp:313-333 / arch-generic.hpp:179-192), a
// clear bit becomes 0; a bipolar plane becomes +-1.  One fp32 accumulator in
// TMEM then sums all wA x wB plane-pair products, i.e. the AND + popcount of
// every plane pair weighted by +-2^(i+j) -- and, because bipolar values are
// +-1 directly, the bipolar corrections of arch-generic.hpp:45-71, 255-259
// need no epilogue term.  Every product and partial sum is an integer, exact
// in fp32 while |sum| < 2^24; the host only selects this kernel when
// K * max|a| * max|b| < 2^24, so the int32 result is bit-exact.
//
// CTA: one 128 x 128 output tile; K advances 128 bits per stage.
//   warp 0     TMA producer: packed planes of the stage (wA + wB boxes of
//              128 rows x 16 bytes) into a 4-slot ring, mbarrier complete_tx
//   warp 1     allocates 128 TMEM columns; lane 0 issues tcgen05.mma
//              (M=128, N=128, K=32 e4m3) for every plane pair and K step,
//              tcgen05.commit frees operand slots and finally signals the
//              accumulator
//   warps 2-9  decode packed bits into the operand ring (128-byte-swizzled,
//              K-major canonical layout), then run the epilogue:
//              tcgen05.ld 32 lanes x 32 columns, fp32 -> int32, coalesced
//              stores of the transposed result res[n*M + m]
// Every mbarrier wait is bounded: on timeout the CTA raises g_tc_error,
// stops issuing work, waits (bounded) for what it issued and frees TMEM.
#include <cuda.h>

#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>

#include "gbs_internal.h"
#include "gbs_tc_common.cuh"

namespace gbs {

static __device__ uint32_t g_tc_error;

namespace {

constexpr int kBM = 128;
constexpr int kRowB = 128;          // bytes per operand row per stage (128 e4m3 values of K)
constexpr int kPkRowB = 16;         // packed bytes per row per plane per stage (128 bits)
constexpr int kDecWarps = 12;  // warps 2..13 decode; warps 2..9 also run the epilogue
constexpr int kThreads = 64 + 32 * kDecWarps;
constexpr int kPkSlots = 4;

// How the planes of one operand become e4m3 operand tiles.  DIGIT mode: one
// tile whose value is the whole few-bit number (all planes at once, so one
// MMA covers every plane pair).  PAIR mode: one tile per plane holding
// {0, +-2^i}.  A tile's value for a given code (its planes' bits, plane
// first+b as bit b) is tab byte [code]: 16 entries, 4 per word.
struct TcOperand {
  int ntiles;
  int first[4], count[4];
  uint32_t tab[4][4];
  int bip;  // bipolar operand: columns past K must decode to 0, not -1
};

struct TcArgs {
  int32_t *C;
  uint64_t M, N, K;
  uint32_t nstages;         // K stages of 128 bits
  uint32_t a_rows, b_rows;  // padded rows per plane (TMA row coordinate of plane i = i * rows + tile row)
  int wa, wb, no;
  uint32_t idesc;
  TcOperand A, B;
};
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag) {
  return mbar_wait_err(bar, parity, abort_flag, &g_tc_error);
}
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) { mbar_drain_err(bar, parity, &g_tc_error); }
// mbar_wait with a given number of rounds (the test hook's short limit)
__device__ __forceinline__ bool mbar_wait_rounds(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                                 uint32_t rounds) {
  for (uint32_t it = 0; it < rounds; ++it) {
    if (mbar_try(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  *abort_flag = 1;
  atomicOr(&g_tc_error, 1u);
  return false;
}

// One tile row of one stage: CNT planes (16 bytes each, `pstride` apart) ->
// 128 e4m3 bytes written as 8 swizzled 16-byte chunks.  Columns at or past
// `kvalid` are forced to 0 (needed for bipolar operands, whose zero padding
// bits would otherwise decode to -1).
template <int CNT>
__device__ __forceinline__ void decode_row(const uint8_t *src, uint32_t pstride, const uint32_t (&tab)[4],
                                           uint8_t *dst, int row, int kvalid) {
  uint32_t w[CNT][4];
#pragma unroll
  for (int p = 0; p < CNT; p++) {
    const uint4 v = *reinterpret_cast<const uint4 *>(src + p * pstride);
    w[p][0] = v.x; w[p][1] = v.y; w[p][2] = v.z; w[p][3] = v.w;
  }
  const uint32_t v0 = tab[0] & 0xFFu, v1 = (tab[0] >> 8) & 0xFFu;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    uint32_t pw[4];
#pragma unroll
    for (int p = 0; p < 4; p++) pw[p] = p < CNT ? w[p][c >> 1] : 0u;
    uint32_t q[4];
#pragma unroll
    for (int n = 0; n < 4; n++) {
      const int sh = 16 * (c & 1) + 4 * n;
      if (CNT == 1) {
        const uint32_t sp = decode4<1>(pw, sh, tab);
        q[n] = sp * v1 + (sp ^ 0x01010101u) * v0;
      } else {
        q[n] = decode4<CNT>(pw, sh, tab);
      }
    }
    if (kvalid < 128) {
#pragma unroll
      for (int n = 0; n < 4; n++) {
        const int c0 = 16 * c + 4 * n;
        if (c0 + 4 > kvalid) q[n] &= c0 >= kvalid ? 0u : (0xFFFFFFFFu >> (8 * (4 - (kvalid - c0))));
      }
    }
    *reinterpret_cast<uint4 *>(dst + ((c ^ (row & 7)) << 4)) = make_uint4(q[0], q[1], q[2], q[3]);
  }
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntA = a.A.ntiles, ntB = a.B.ntiles;
  const uint32_t a_tile = kBM * kRowB, b_tile = BN * kRowB;
  const uint32_t op_stage = ntA * a_tile + ntB * b_tile;
  const uint32_t pk_a = kBM * kPkRowB, pk_b = BN * kPkRowB;  // packed bytes of one plane per stage
  const uint32_t pk_stage = a.wa * pk_a + a.wb * pk_b;
  uint8_t *op_ring = smem;
  uint8_t *pk_ring = op_ring + a.no * op_stage;
  uint64_t *bars = reinterpret_cast<uint64_t *>(pk_ring + kPkSlots * pk_stage);
  // barriers: pk_full[4], pk_empty[4], op_full[no], op_empty[no], acc_full, mma_done
  const uint32_t pk_full = smem_u32(bars), pk_empty = pk_full + 8 * kPkSlots;
  const uint32_t op_full = pk_empty + 8 * kPkSlots, op_empty = op_full + 8 * a.no;
  const uint32_t acc_full = op_empty + 8 * a.no, mma_done = acc_full + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kPkSlots + 2 * a.no + 2);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint64_t m0 = (uint64_t)blockIdx.x * kBM, n0 = (uint64_t)blockIdx.y * BN;

  if (tid == 0) {
    for (int i = 0; i < kPkSlots; i++) {
      mbar_init(pk_full + 8 * i, 1);                // producer's expect_tx + TMA bytes
      mbar_init(pk_empty + 8 * i, 32 * kDecWarps);  // every decoder thread has read the slot
    }
    for (int i = 0; i < a.no; i++) {
      mbar_init(op_full + 8 * i, 32 * kDecWarps);   // every decoder thread has written its chunks
      mbar_init(op_empty + 8 * i, 1);               // tcgen05.commit of the MMAs that read the slot
    }
    mbar_init(acc_full, 1);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer: 128-row boxes (two per rhs plane when BN = 256)
    if (lane == 0) {
      uint32_t issued = 0;
      for (uint32_t k = 0; k < a.nstages; k++) {
        const uint32_t s = k % kPkSlots, use = k / kPkSlots;
        if (use > 0 && !mbar_wait(pk_empty + 8 * s, (use - 1) & 1, abort_flag)) break;
        mbar_expect_tx(pk_full + 8 * s, pk_stage);
        const uint32_t dst = smem_u32(pk_ring + s * pk_stage);
        for (int i = 0; i < a.wa; i++)
          tma_load_2d(dst + i * pk_a, &tmA, (int)(2 * k), (int)(i * a.a_rows + m0), pk_full + 8 * s);
        for (int j = 0; j < a.wb; j++)
          for (int h = 0; h < BN / 128; h++)
            tma_load_2d(dst + a.wa * pk_a + j * pk_b + h * 128 * kPkRowB, &tmB, (int)(2 * k),
                        (int)(j * a.b_rows + n0 + 128 * h), pk_full + 8 * s);
        issued = k + 1;
      }
      if (*abort_flag) {  // let issued copies land before the CTA can exit
        for (uint32_t k = (issued > kPkSlots ? issued - kPkSlots : 0); k < issued; k++)
          mbar_drain(pk_full + 8 * (k % kPkSlots), (k / kPkSlots) & 1);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer: every (lhs tile, rhs tile) pair, 4 K steps of 32
    if (lane == 0) {
      bool ok = true;
      for (uint32_t k = 0; k < a.nstages && ok; k++) {
        const uint32_t o = k % a.no;
        if (!mbar_wait(op_full + 8 * o, (k / a.no) & 1, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = smem_u32(op_ring + o * op_stage);
        for (int i = 0; i < ntA; i++)
          for (int j = 0; j < ntB; j++)
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
              const uint64_t ad = sw128_desc(base + i * a_tile + kk * 32);
              const uint64_t bd = sw128_desc(base + ntA * a_tile + j * b_tile + kk * 32);
              mma_f8(tmem, ad, bd, a.idesc, (k | i | j | kk) != 0);
            }
        mma_commit(op_empty + 8 * o);
      }
      mma_commit(ok ? acc_full : mma_done);
      if (!ok) mbar_drain(mma_done, 0);  // issued MMAs finish before TMEM is freed
    }
  } else {
    // ---------------- decoders: each thread owns whole tile rows (all 8 chunks of 16 columns)
    const int d = tid - 64;
    const int rowsA = ntA * kBM, rows = rowsA + ntB * BN;
    for (uint32_t k = 0; k < a.nstages; k++) {
      const uint32_t s = k % kPkSlots, o = k % a.no;
      if (!mbar_wait(pk_full + 8 * s, (k / kPkSlots) & 1, abort_flag)) break;
      if (k >= (uint32_t)a.no && !mbar_wait(op_empty + 8 * o, ((k / a.no) - 1) & 1, abort_flag)) break;
      const uint8_t *pk = pk_ring + s * pk_stage;
      uint8_t *op = op_ring + o * op_stage;
      // columns of this stage past the real K (only the last stage can have any)
      const int kvalid = (uint64_t)k * 128 + 128 > a.K ? (int)(a.K - (uint64_t)k * 128) : 128;
      for (int r = d; r < rows; r += 32 * kDecWarps) {
        const bool isA = r < rowsA;
        const int rr = isA ? r : r - rowsA;
        const int t = isA ? rr >> 7 : rr / BN, row = isA ? rr & 127 : rr % BN;
        const TcOperand &P = isA ? a.A : a.B;
        const uint8_t *src = isA ? pk + P.first[t] * pk_a : pk + a.wa * pk_a + P.first[t] * pk_b;
        const uint32_t pstride = isA ? pk_a : pk_b;
        uint8_t *dst = op + (isA ? t * a_tile : ntA * a_tile + t * b_tile) + row * kRowB;
        const uint32_t tab[4] = {P.tab[t][0], P.tab[t][1], P.tab[t][2], P.tab[t][3]};
        switch (P.count[t]) {
          case 1: decode_row<1>(src + row * kPkRowB, pstride, tab, dst, row, P.bip ? kvalid : 128); break;
          case 2: decode_row<2>(src + row * kPkRowB, pstride, tab, dst, row, P.bip ? kvalid : 128); break;
          case 3: decode_row<3>(src + row * kPkRowB, pstride, tab, dst, row, P.bip ? kvalid : 128); break;
          default: decode_row<4>(src + row * kPkRowB, pstride, tab, dst, row, P.bip ? kvalid : 128); break;
        }
      }
      // generic-proxy writes become visible to tcgen05.mma (async proxy) via fence + mbarrier release
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(op_full + 8 * o);
      mbar_arrive(pk_empty + 8 * s);
    }
    // epilogue (warps 2..9): warp w reads TMEM lanes 32*(w%4)..+31 (output rows), half of
    // the columns.  The decision is warp-uniform because tcgen05.ld is a whole-warp instruction.
    if (warp < 10 && __all_sync(0xffffffffu, mbar_wait(acc_full, 0, abort_flag))) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int quarter = warp & 3, half = (warp - 2) >> 2;
      const uint64_t gm = m0 + quarter * 32 + lane;
#pragma unroll 1
      for (int cb = 0; cb < BN / 64; cb++) {
        const int col = half * (BN / 2) + cb * 32;
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)col;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
              "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
              "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
              "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        int32_t o[32];
#pragma unroll
        for (int j = 0; j < 32; j++) o[j] = __float2int_rn(__uint_as_float(v[j]));
        store_result_cols<32>(a.C, a.M, a.N, gm, n0 + col, o);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(BN));
  }
}

// ---------------------------------------------------------------- HBM digit path
// TMA-fed GEMM on digit matrices: 128 x BN output tile per CTA.
//   warp 0     TMA: A box 128 rows x 128 bytes, B boxes 128 rows x 128 bytes
//              (BN/128 of them), 128-byte swizzle = the MMA's K-major layout
//   warp 1     TMEM allocation; lane 0 issues 4 tcgen05.mma (K = 32) per stage
//   warps 2-9  epilogue: TMEM -> int32 -> res[n*M + m]
constexpr int kTmaStagesMax = 4;
constexpr int kTmaThreads = 320;

struct TmaArgs {
  int32_t *C;
  uint64_t M, N;
  uint32_t nstages;
  uint32_t idesc;
  int stages;
  int splits;  // SM-pair kernel: K chunks per output tile, one SM pair each (1, 2 or 4)
  // SM-pair kernel, test hook: 0 normally; otherwise nothing is loaded or
  // multiplied and the waits give up after this many rounds, so the kernel
  // takes its abort path (error bit, drains, TMEM freed) and returns
  uint32_t wait_limit;
};

template <int BN>
__global__ void __launch_bounds__(kTmaThreads, 1)
    gemm_tc_tma_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TmaArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t a_bytes = kBM * kRowB, b_bytes = BN * kRowB, stage_bytes = a_bytes + b_bytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + a.stages * stage_bytes);
  const uint32_t full = smem_u32(bars), empty = full + 8 * a.stages, acc_full = empty + 8 * a.stages;
  const uint32_t mma_done = acc_full + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * a.stages + 2);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint64_t m0 = (uint64_t)blockIdx.x * kBM, n0 = (uint64_t)blockIdx.y * BN;

  if (tid == 0) {
    for (int i = 0; i < a.stages; i++) {
      mbar_init(full + 8 * i, 1);
      mbar_init(empty + 8 * i, 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t issued = 0;
      for (uint32_t k = 0; k < a.nstages; k++) {
        const uint32_t s = k % a.stages, use = k / a.stages;
        if (use > 0 && !mbar_wait(empty + 8 * s, (use - 1) & 1, abort_flag)) break;
        mbar_expect_tx(full + 8 * s, stage_bytes);
        const uint32_t dst = smem_u32(smem + s * stage_bytes);
        tma_load_digits(dst, &tmA, (int)k, (uint32_t)m0, full + 8 * s);
        for (int h = 0; h < BN / 128; h++)
          tma_load_digits(dst + a_bytes + h * 128 * kRowB, &tmB, (int)k, (uint32_t)(n0 + 128 * h), full + 8 * s);
        issued = k + 1;
      }
      if (*abort_flag) {
        for (uint32_t k = (issued > (uint32_t)a.stages ? issued - a.stages : 0); k < issued; k++)
          mbar_drain(full + 8 * (k % a.stages), (k / a.stages) & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      for (uint32_t k = 0; k < a.nstages && ok; k++) {
        const uint32_t s = k % a.stages;
        if (!mbar_wait(full + 8 * s, (k / a.stages) & 1, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = smem_u32(smem + s * stage_bytes);
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
          mma_f8(tmem, sw128_desc(base + kk * 32), sw128_desc(base + a_bytes + kk * 32), a.idesc, (k | kk) != 0);
        mma_commit(empty + 8 * s);
      }
      mma_commit(ok ? acc_full : mma_done);
      if (!ok) mbar_drain(mma_done, 0);
    }
  } else {
    if (__all_sync(0xffffffffu, mbar_wait(acc_full, 0, abort_flag))) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int quarter = warp & 3, half = (warp - 2) >> 2;
      const uint64_t gm = m0 + quarter * 32 + lane;
#pragma unroll 1
      for (int cb = 0; cb < BN / 64; cb++) {
        const int col = half * (BN / 2) + cb * 32;
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)col;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
              "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
              "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
              "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        int32_t o[32];
#pragma unroll
        for (int j = 0; j < 32; j++) o[j] = __float2int_rn(__uint_as_float(v[j]));
        store_result_cols<32>(a.C, a.M, a.N, gm, n0 + col, o);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(BN));
  }
}

// Pair kernel: a cluster of two CTAs on two SMs computes one 256 x BN
// output tile (BN = 256 or 128) with tcgen05.mma.cta_group::2 (M = 256,
// N = BN, K = 32).  CTA rank r holds A rows [m0 + 128r, +128) and B rows
// [n0 + BN/2 r, +BN/2) of every stage and accumulates its 128 result rows x
// BN columns in its own TMEM; at BN = 256 each SM receives 32 KB per
// 128-digit stage for the math a 1-SM 128 x 256 tile does with 48 KB.  The
// 128-column tiles double the tile count for shapes with few tiles.
//   warp 0     in the leader: TMA of both CTAs' halves of every stage onto
//              the leader's full barrier (the peer's into its shared memory)
//   warp 1     TMEM allocation (both CTAs, collectively); in the leader, lane
//              0 issues the MMAs and commits to the empty / accumulator
//              barriers of both CTAs (multicast)
//   warps 2-5  epilogue of this CTA's 128 rows
// A cluster barrier closes the kernel, so no CTA frees TMEM or exits while
// its peer may still signal its barriers or write its accumulator.
constexpr int kPairStagesMax = 9;
constexpr size_t kPairSmemCap = 227 * 1024;  // the per-block dynamic shared memory limit
constexpr int kPairThreads = 192;
constexpr uint32_t kPairHalfBytes = 128 * kRowB;  // 128 rows x 128 digits

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t map_to_rank(uint32_t smem_addr, uint32_t rank) {
  uint32_t d;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(smem_addr), "r"(rank));
  return d;
}
// tma_load_digits for an SM pair: completes on `bar`, the leader CTA's barrier.
__device__ __forceinline__ void tma_load_digits_pair(uint32_t dst, const CUtensorMap *map, int k, uint32_t row,
                                                     uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2 [%0], [%1, {%2, "
      "%3, %4, %5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(k), "r"((int)(row >> 4)), "r"(bar)
      : "memory");
}
// L2 prefetch of the box tma_load_digits(_pair) would load (a hint: no data
// lands in shared memory and no barrier is signalled).
__device__ __forceinline__ void tma_prefetch_digits(const CUtensorMap *map, int k, uint32_t row) {
  asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(0), "r"(0), "r"(k), "r"((int)(row >> 4))
               : "memory");
}
__device__ __forceinline__ void mma_f8_pair(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
// arrives on `bar` in both CTAs of the pair whose ranks are the set bits of `mask`
__device__ __forceinline__ void mma_commit_pair(uint32_t bar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
      "h"(mask)
      : "memory");
}
// Generic address of the same shared-memory location in CTA `rank` of the
// cluster: plain loads through it can be batched by the compiler.
template <typename T>
__device__ __forceinline__ const T *cluster_ptr(const T *p, uint32_t rank) {
  uint64_t d;
  asm("mapa.u64 %0, %1, %2;" : "=l"(d) : "l"(reinterpret_cast<uint64_t>(p)), "r"(rank));
  return reinterpret_cast<const T *>(d);
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
// Waits for this thread's TMEM loads; the registers they fill are operands,
// so no use of them can be scheduled before the wait.
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&v)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                 "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15]),
                 "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]), "+r"(v[22]),
                 "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]), "+r"(v[29]),
                 "+r"(v[30]), "+r"(v[31])
               :
               : "memory");
}
// Marks registers a TMEM load filled as produced after the tcgen05.wait::ld
// issued just before (volatile asm keeps its place in program order): for
// several loads in flight behind one wait.
__device__ __forceinline__ void tmem_after_wait(uint32_t (&v)[32]) {
  asm volatile(""
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                 "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15]),
                 "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]), "+r"(v[22]),
                 "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]), "+r"(v[29]),
                 "+r"(v[30]), "+r"(v[31])
               :
               : "memory");
}
// 32 columns n0 .. n0+31 of result row m from fp32 accumulator bits.
__device__ __forceinline__ void store_cols(const TmaArgs &a, const uint32_t (&v)[32], uint64_t gm, uint64_t n0) {
  int32_t o[32];
#pragma unroll
  for (int j = 0; j < 32; j++) o[j] = __float2int_rn(__uint_as_float(v[j]));
  store_result_cols<32>(a.C, a.M, a.N, gm, n0, o);
}

template <int SPLITS, int BN>
__global__ void __launch_bounds__(kPairThreads, 1)
    gemm_tc_pair_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TmaArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = cluster_rank();
  // ranks 2p and 2p+1 form the SM pair of K chunk p; the even one leads
  const uint32_t peer = rank & 1u, split = rank >> 1, lead = rank & ~1u;
  const uint16_t pair_mask = (uint16_t)(3u << lead);
  constexpr uint32_t kBHalf = (BN / 2) * kRowB;  // this CTA's BN/2 rows of the B tile
  const uint32_t stage_bytes = kPairHalfBytes + kBHalf;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + a.stages * stage_bytes);
  const uint32_t full = smem_u32(bars), empty = full + 8 * a.stages, acc_full = empty + 8 * a.stages;
  const uint32_t mma_done = acc_full + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * a.stages + 2);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint64_t pair_m0 = (uint64_t)(blockIdx.x / (2 * SPLITS)) * 256, n0 = (uint64_t)blockIdx.y * BN;
  const uint64_t m0 = pair_m0 + 128 * peer;
  const uint32_t k_lo = split * a.nstages / SPLITS, k_hi = (split + 1) * a.nstages / SPLITS;
  const uint32_t nk = k_hi - k_lo;
  bool tile_done = false;  // epilogue warps: the accumulator is complete
  griddep_launch_dependents();
  if (tid == 0 && a.wait_limit == 0) {  // descriptors towards the TMA unit before the first load needs them
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
  }
  if (tid == 64 && peer == 0 && a.wait_limit == 0) {
    // an epilogue thread (idle until the accumulator is done) sends the first
    // three stages towards L2 while setup runs and the previous kernel
    // finishes: about 50 ns per hint, within the setup's own time (issued
    // from the setup thread for the whole ring, they held up its barrier
    // initialisation by 1-2 us)
    const uint32_t pre = nk < 3u ? nk : 3u;
    for (uint32_t k = 0; k < pre; k++) {
      tma_prefetch_digits(&tmA, (int)(k_lo + k), (uint32_t)pair_m0);
      tma_prefetch_digits(&tmA, (int)(k_lo + k), (uint32_t)(pair_m0 + 128));
      tma_prefetch_digits(&tmB, (int)(k_lo + k), (uint32_t)n0);
      tma_prefetch_digits(&tmB, (int)(k_lo + k), (uint32_t)(n0 + BN / 2));
    }
  }

  if (tid == 0) {
    for (int i = 0; i < a.stages; i++) {
      mbar_init(full + 8 * i, 1);
      mbar_init(empty + 8 * i, 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  // both CTAs' barriers are initialised before either CTA signals its peer
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  griddep_wait();  // operands and result belong to the previous kernels until here

  if (warp == 0) {
    // The leader's TMA loads the stage for both CTAs: its own halves, and the
    // peer's into the peer's shared memory, all completing on the leader's
    // full barrier.  Each CTA loading its own halves onto that barrier puts a
    // cross-SM completion on every stage's critical path, which measured about
    // twice as slow per stage as the one-issuer ring.  (The test hook loads nothing.)
    if (lane == 0 && peer == 0 && a.wait_limit == 0) {
      uint32_t issued = 0;
      for (uint32_t k = 0; k < nk; k++) {
        const uint32_t s = k % a.stages, use = k / a.stages;
        if (use > 0 && !mbar_wait(empty + 8 * s, (use - 1) & 1, abort_flag)) break;
        const uint32_t fb = map_to_rank(full + 8 * s, lead);
        mbar_expect_tx(full + 8 * s, 2 * stage_bytes);
        const uint32_t dst = smem_u32(smem + s * stage_bytes), pdst = map_to_rank(dst, lead + 1);
        const int kc = (int)(k_lo + k);
        tma_load_digits_pair(dst, &tmA, kc, (uint32_t)pair_m0, fb);
        tma_load_digits_pair(dst + kPairHalfBytes, &tmB, kc, (uint32_t)n0, fb);
        tma_load_digits_pair(pdst, &tmA, kc, (uint32_t)(pair_m0 + 128), fb);
        tma_load_digits_pair(pdst + kPairHalfBytes, &tmB, kc, (uint32_t)(n0 + BN / 2), fb);
        issued = k + 1;
      }
      // after an abort, wait (bounded) for the loads the barriers still expect
      // (the peer's shared memory is written until then; the closing cluster
      // barrier keeps the peer resident)
      if (*abort_flag) {
        for (uint32_t k = (issued > (uint32_t)a.stages ? issued - a.stages : 0); k < issued; k++)
          mbar_drain(full + 8 * (k % a.stages), (k / a.stages) & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && peer == 0) {
      // test hook: nothing was loaded, so this wait runs out (no copy or MMA in flight)
      bool ok = a.wait_limit == 0 || mbar_wait_rounds(full, 0, abort_flag, a.wait_limit);
      for (uint32_t k = 0; k < nk && ok; k++) {
        const uint32_t s = k % a.stages;
        if (!mbar_wait(full + 8 * s, (k / a.stages) & 1, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = smem_u32(smem + s * stage_bytes);
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
          mma_f8_pair(tmem, sw128_desc(base + kk * 32), sw128_desc(base + kPairHalfBytes + kk * 32), a.idesc,
                      (k | kk) != 0);
        mma_commit_pair(empty + 8 * s, pair_mask);
      }
      if (ok) {
        mma_commit_pair(acc_full, pair_mask);
      } else {  // issued MMAs finish before TMEM is freed
        asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mma_done)
                     : "memory");
        mbar_drain(mma_done, 0);
      }
    }
  } else {
    tile_done = __all_sync(0xffffffffu, a.wait_limit ? mbar_wait_rounds(acc_full, 0, abort_flag, a.wait_limit)
                                                     : mbar_wait(acc_full, 0, abort_flag));
    if (tile_done) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int q = warp & 3;
      const uint64_t gm = m0 + q * 32 + lane;
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16);
      if (SPLITS == 1) {
        // four 32-column TMEM loads behind one wait: tcgen05.wait::ld waits
        // for all of a thread's loads, so the latency is paid once per 128
        // columns
#pragma unroll 1
        for (int col = 0; col < BN; col += 128) {
          uint32_t v[4][32];
#pragma unroll
          for (int i = 0; i < 4; i++) tmem_ld32(taddr + (uint32_t)(col + 32 * i), v[i]);
          tmem_wait_ld(v[0]);
#pragma unroll
          for (int i = 1; i < 4; i++) tmem_after_wait(v[i]);
#pragma unroll
          for (int i = 0; i < 4; i++) store_cols(a, v[i], gm, n0 + col + 32 * i);
        }
      } else {
        // the columns the other K chunks reduce go into the drained ring as
        // [64 column quads][128 rows][4 columns] fp32: each lane (row) writes,
        // and later reads remotely, 16 bytes per quad, a warp 512 contiguous
        // bytes; this chunk's own columns stay in TMEM
        float4 *part = reinterpret_cast<float4 *>(smem) + q * 32 + lane;
        const uint32_t own0 = split * (BN / SPLITS), own1 = own0 + BN / SPLITS;
#pragma unroll 1
        for (uint32_t col = 0; col < BN; col += 32) {
          if (col >= own0 && col < own1) continue;
          uint32_t v[32];
          tmem_ld32(taddr + (uint32_t)col, v);
          tmem_wait_ld(v);
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            part[((col + j) >> 2) * 128] = make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]),
                                                       __uint_as_float(v[j + 2]), __uint_as_float(v[j + 3]));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  if constexpr (SPLITS > 1) {
    // Split-K reduction over distributed shared memory: the CTA of chunk p sums
    // columns [p*BN/S, (p+1)*BN/S) of its 128 rows over the S partial tiles
    // (integers below 2^24: the fp32 sums are exact) and stores them; a warp's
    // remote loads and its stores each cover 32 consecutive rows of a column.
    if (warp >= 2 && tile_done) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int q = warp & 3;
      const uint32_t row = (uint32_t)(q * 32 + lane), cols = BN / SPLITS, c0 = split * cols;
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + c0;
      const uint64_t gm = m0 + row;
      const float4 *mine = reinterpret_cast<const float4 *>(smem) + (c0 >> 2) * 128 + row;
      const float4 *src[SPLITS - 1];
#pragma unroll
      for (int qq = 1; qq < SPLITS; qq++) src[qq - 1] = cluster_ptr(mine, 2 * ((split + qq) % SPLITS) + peer);
      // 32 columns at a time: the other chunks' partials (remote loads issued
      // first), then this chunk's own from TMEM
#pragma unroll 1
      for (uint32_t cb = 0; cb < cols; cb += 32) {
        float4 raw[SPLITS - 1][8];
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
          for (int qq = 0; qq < SPLITS - 1; qq++) raw[qq][i] = src[qq][((cb >> 2) + i) * 128];
        uint32_t v[32];
        tmem_ld32(taddr + cb, v);
        tmem_wait_ld(v);
        int32_t o[32];
#pragma unroll
        for (int i = 0; i < 32; i++) {
          float acc = __uint_as_float(v[i]);
#pragma unroll
          for (int qq = 0; qq < SPLITS - 1; qq++) {
            const float4 r4 = raw[qq][i >> 2];
            acc += (i & 3) == 0 ? r4.x : (i & 3) == 1 ? r4.y : (i & 3) == 2 ? r4.z : r4.w;
          }
          o[i] = __float2int_rn(acc);
        }
        store_result_cols<32>(a.C, a.M, a.N, gm, n0 + c0 + cb, o);
      }
    }
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(BN));
  }
}

// Persistent SM-pair kernel, 256 x 256 tiles, for grids of more tiles than
// the GPU has SM pairs: each 2-CTA cluster p of P loops over tiles p, p + P,
// ...  and accumulates its j-th tile in TMEM buffer j & 1 (2 x 256 columns),
// so the epilogue of one tile overlaps the MMAs of the next instead of a
// second wave repeating launch, setup and the first load.  The operand ring
// runs on across tiles; the leader's TMA loads both CTAs' halves as in
// gemm_tc_pair_kernel.  Barriers (same offsets in both CTAs): full / empty
// of the ring; acc_full[2], committed (multicast) by the MMA thread when a
// tile's accumulator is complete; acc_empty[2] in the leader, where the 4
// epilogue warps of both CTAs (the peer's remotely) arrive once they have
// read a buffer, before the MMAs may write it again.
__global__ void __launch_bounds__(kPairThreads, 1)
    gemm_tc_pair_persistent_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                                   TmaArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t peer = cluster_rank() & 1u;  // clusters of 2: rank 0 leads
  constexpr uint16_t kPairMask = 3;
  constexpr uint32_t stage_bytes = 2 * kPairHalfBytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + a.stages * stage_bytes);
  const uint32_t full = smem_u32(bars), empty = full + 8 * a.stages, acc_full = empty + 8 * a.stages;
  const uint32_t acc_empty = acc_full + 16, mma_done = acc_empty + 16;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * a.stages + 5);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint32_t npairs = gridDim.x >> 1, pid = blockIdx.x >> 1;
  // tiles in M-fastest order (tile t = row block t % mt of column block t / mt): the pairs running at
  // once write whole columns of the M-major result, which measured ~2.5x faster than N-fastest
  const uint32_t mt = (uint32_t)((a.M + 255) / 256), ntiles = mt * (uint32_t)((a.N + 255) / 256), nk = a.nstages;
  griddep_launch_dependents();

  if (tid == 0) {
    for (int i = 0; i < a.stages; i++) {
      mbar_init(full + 8 * i, 1);
      mbar_init(empty + 8 * i, 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(acc_full + 8 * b, 1);
      mbar_init(acc_empty + 8 * b, 8);  // 4 epilogue warps x 2 CTAs
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  griddep_wait();  // operands and result belong to the previous kernels until here

  if (warp == 0) {
    if (lane == 0 && peer == 0) {  // the leader's TMA: both CTAs' halves of every stage
      uint32_t g = 0;
      bool stop = false;
      for (uint32_t t = pid; t < ntiles && !stop; t += npairs) {
        const uint32_t m0 = (t % mt) * 256u, n0 = (t / mt) * 256u;
        for (uint32_t k = 0; k < nk; k++, g++) {
          const uint32_t s = g % a.stages, use = g / a.stages;
          if (use > 0 && !mbar_wait(empty + 8 * s, (use - 1) & 1, abort_flag)) {
            stop = true;
            break;
          }
          const uint32_t fb = map_to_rank(full + 8 * s, 0);
          mbar_expect_tx(full + 8 * s, 2 * stage_bytes);
          const uint32_t dst = smem_u32(smem + s * stage_bytes), pdst = map_to_rank(dst, 1);
          tma_load_digits_pair(dst, &tmA, (int)k, m0, fb);
          tma_load_digits_pair(dst + kPairHalfBytes, &tmB, (int)k, n0, fb);
          tma_load_digits_pair(pdst, &tmA, (int)k, m0 + 128, fb);
          tma_load_digits_pair(pdst + kPairHalfBytes, &tmB, (int)k, n0 + 128, fb);
        }
      }
      if (*abort_flag)  // wait (bounded) for the loads the barriers still expect
        for (uint32_t q = (g > (uint32_t)a.stages ? g - a.stages : 0); q < g; q++)
          mbar_drain(full + 8 * (q % a.stages), (q / a.stages) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0 && peer == 0) {  // the leader issues the pair's MMAs
      bool ok = true;
      uint32_t g = 0, j = 0;
      for (uint32_t t = pid; t < ntiles && ok; t += npairs, j++) {
        const uint32_t b = j & 1u, dacc = tmem + b * 256u;
        if (j >= 2 && !mbar_wait(acc_empty + 8 * b, ((j >> 1) - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (uint32_t k = 0; k < nk; k++, g++) {
          const uint32_t s = g % a.stages;
          if (!mbar_wait(full + 8 * s, (g / a.stages) & 1, abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t base = smem_u32(smem + s * stage_bytes);
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            mma_f8_pair(dacc, sw128_desc(base + kk * 32), sw128_desc(base + kPairHalfBytes + kk * 32), a.idesc,
                        (k | kk) != 0);
          mma_commit_pair(empty + 8 * s, kPairMask);
        }
        if (ok) mma_commit_pair(acc_full + 8 * b, kPairMask);
      }
      if (!ok) {  // issued MMAs finish before TMEM is freed
        asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mma_done)
                     : "memory");
        mbar_drain(mma_done, 0);
      }
    }
  } else {  // epilogue: this CTA's 128 rows of every tile
    const int q = warp & 3;
    uint32_t j = 0;
    for (uint32_t t = pid; t < ntiles; t += npairs, j++) {
      const uint32_t b = j & 1u;
      if (!__all_sync(0xffffffffu, mbar_wait(acc_full + 8 * b, (j >> 1) & 1, abort_flag))) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint64_t gm = (uint64_t)(t % mt) * 256u + 128u * peer + (uint32_t)(q * 32 + lane);
      const uint64_t n0 = (uint64_t)(t / mt) * 256u;
      const uint32_t taddr = tmem + b * 256u + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (int col = 0; col < 256; col += 128) {  // four TMEM loads behind one wait
        uint32_t v[4][32];
#pragma unroll
        for (int i = 0; i < 4; i++) tmem_ld32(taddr + (uint32_t)(col + 32 * i), v[i]);
        tmem_wait_ld(v[0]);
#pragma unroll
        for (int i = 1; i < 4; i++) tmem_after_wait(v[i]);
#pragma unroll
        for (int i = 0; i < 4; i++) store_cols(a, v[i], gm, n0 + col + 32 * i);
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) {  // this warp is done with the buffer: tell the leader's MMA thread
        if (peer == 0) {
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(acc_empty + 8 * b) : "memory");
        } else {
          const uint32_t rb = map_to_rank(acc_empty + 8 * b, 0);
          asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(rb) : "memory");
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(512));
  }
}

// ---------------------------------------------------------------- stream-K SM pairs
// Stream-K pair kernel: the (256 x 256 tile, 128-digit K stage) units of the
// whole GEMM are split evenly over P SM pairs (2-CTA clusters), so all pairs
// run the same number of stages whatever the tile count.  Pair p owns units
// [p U / P, (p+1) U / P), tiles M-fastest, and walks them from the top down
// in segments of one tile each; segment j accumulates in TMEM buffer j & 1 so
// its epilogue overlaps the next segment's MMAs.  A tile split over pairs is
// finished by the pair holding its last stage (the tail): with the descending
// walk that is the tile's last segment in time, while every other share of it
// is the first segment of a lower pair, done early and stored as an fp32
// partial in that pair's workspace slot.  The tail's epilogue waits
// (bounded) for those partials' flags -- only ever on lower pairs, which
// were dispatched first and wait on nobody before publishing -- and adds them
// (integers below 2^24: exact).  Flags carry the launch's epoch, so the
// workspace needs no reset.  Loads, MMAs and the TMEM buffers' handshakes are
// those of gemm_tc_pair_persistent_kernel.  Measured on 2048 x 4096 x 2048
// (64 tiles): over all 76 pairs it ran 28 us against 21 us for one tile per
// pair -- a split tile's partial store, flag and reload cost more than the
// five stages the even split saves -- so the built-in rule does not take it;
// it is a tuner candidate (variant 515).
struct SkArgs {
  int32_t *C;
  float *ws;        // [pairs][256 columns][256 rows] fp32 partial tiles
  uint32_t *flags;  // [pairs][2 CTAs][4 warps]: epoch once that warp's partial rows are stored
  uint64_t M, N;
  uint32_t nk;      // K stages per tile
  uint32_t mt;      // 256-row tiles along M
  uint32_t units;   // tiles * nk
  uint32_t epoch;
  uint32_t idesc;
  int stages;
};

struct SkSeg {
  uint32_t t, k0, k1;  // tile, stages [k0, k1)
};
// Next segment of the descending walk from u down to u0 (false when done).
__device__ __forceinline__ bool sk_next(uint32_t &u, uint32_t u0, uint32_t nk, SkSeg &sg) {
  if (u <= u0) return false;
  const uint32_t t = (u - 1) / nk, base = t * nk;
  sg.t = t;
  sg.k1 = u - base;
  sg.k0 = u0 > base ? u0 - base : 0u;
  u = base + sg.k0;
  return true;
}
__device__ __forceinline__ uint32_t sk_u0(uint32_t p, uint32_t units, uint32_t pairs) {
  return (uint32_t)(((uint64_t)p * units) / pairs);
}
// Bounded wait for a flag word to reach `epoch` (acquire: the partial it
// guards is visible after it); false after the limit.
__device__ __forceinline__ bool sk_wait_flag(const uint32_t *f, uint32_t epoch) {
  for (uint32_t it = 0; it < kTcWaitLimit; ++it) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
    if (v == epoch) return true;
    __nanosleep(64);
  }
  return false;
}

__global__ void __launch_bounds__(kPairThreads, 1)
    gemm_tc_pair_streamk_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                                SkArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  griddep_launch_dependents();
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t peer = cluster_rank() & 1u;  // clusters of 2: rank 0 leads
  constexpr uint16_t kPairMask = 3;
  constexpr uint32_t stage_bytes = 2 * kPairHalfBytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + a.stages * stage_bytes);
  const uint32_t full = smem_u32(bars), empty = full + 8 * a.stages, acc_full = empty + 8 * a.stages;
  const uint32_t acc_empty = acc_full + 16, mma_done = acc_empty + 16;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * a.stages + 5);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint32_t npairs = gridDim.x >> 1, pid = blockIdx.x >> 1, nk = a.nk;
  const uint32_t u0 = sk_u0(pid, a.units, npairs), u1 = sk_u0(pid + 1, a.units, npairs);

  if (tid == 0) {
    for (int i = 0; i < a.stages; i++) {
      mbar_init(full + 8 * i, 1);
      mbar_init(empty + 8 * i, 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(acc_full + 8 * b, 1);
      mbar_init(acc_empty + 8 * b, 8);  // 4 epilogue warps x 2 CTAs
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  griddep_wait();  // operands, result and workspace belong to the previous kernels until here

  if (warp == 0) {
    if (lane == 0 && peer == 0) {  // the leader's TMA: both CTAs' halves of every stage
      uint32_t g = 0, u = u1;
      bool stop = false;
      SkSeg sg;
      while (!stop && sk_next(u, u0, nk, sg)) {
        const uint32_t m0 = (sg.t % a.mt) * 256u, n0 = (sg.t / a.mt) * 256u;
        for (uint32_t k = sg.k0; k < sg.k1; k++, g++) {
          const uint32_t s = g % a.stages, use = g / a.stages;
          if (use > 0 && !mbar_wait(empty + 8 * s, (use - 1) & 1, abort_flag)) {
            stop = true;
            break;
          }
          const uint32_t fb = map_to_rank(full + 8 * s, 0);
          mbar_expect_tx(full + 8 * s, 2 * stage_bytes);
          const uint32_t dst = smem_u32(smem + s * stage_bytes), pdst = map_to_rank(dst, 1);
          tma_load_digits_pair(dst, &tmA, (int)k, m0, fb);
          tma_load_digits_pair(dst + kPairHalfBytes, &tmB, (int)k, n0, fb);
          tma_load_digits_pair(pdst, &tmA, (int)k, m0 + 128, fb);
          tma_load_digits_pair(pdst + kPairHalfBytes, &tmB, (int)k, n0 + 128, fb);
        }
      }
      if (*abort_flag)  // wait (bounded) for the loads the barriers still expect
        for (uint32_t q = (g > (uint32_t)a.stages ? g - a.stages : 0); q < g; q++)
          mbar_drain(full + 8 * (q % a.stages), (q / a.stages) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0 && peer == 0) {  // the leader issues the pair's MMAs
      bool ok = true;
      uint32_t g = 0, j = 0, u = u1;
      SkSeg sg;
      while (ok && sk_next(u, u0, nk, sg)) {
        const uint32_t b = j & 1u, dacc = tmem + b * 256u;
        if (j >= 2 && !mbar_wait(acc_empty + 8 * b, ((j >> 1) - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (uint32_t k = sg.k0; k < sg.k1; k++, g++) {
          const uint32_t s = g % a.stages;
          if (!mbar_wait(full + 8 * s, (g / a.stages) & 1, abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t base = smem_u32(smem + s * stage_bytes);
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            mma_f8_pair(dacc, sw128_desc(base + kk * 32), sw128_desc(base + kPairHalfBytes + kk * 32), a.idesc,
                        (k != sg.k0 || kk != 0) ? 1u : 0u);
          mma_commit_pair(empty + 8 * s, kPairMask);
        }
        if (ok) mma_commit_pair(acc_full + 8 * b, kPairMask);
        j++;
      }
      if (!ok) {  // issued MMAs finish before TMEM is freed
        asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mma_done)
                     : "memory");
        mbar_drain(mma_done, 0);
      }
    }
  } else {  // epilogue: this CTA's 128 rows of every segment
    const int q = warp & 3;
    const uint32_t row = 128u * peer + (uint32_t)(q * 32 + lane);  // row within the 256-row tile
    uint32_t j = 0, u = u1;
    SkSeg sg;
    while (sk_next(u, u0, nk, sg)) {
      const uint32_t b = j & 1u;
      if (!__all_sync(0xffffffffu, mbar_wait(acc_full + 8 * b, (j >> 1) & 1, abort_flag))) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t taddr = tmem + b * 256u + ((uint32_t)(q * 32) << 16);
      if (sg.k1 < nk) {
        // a share of a tile a higher pair finishes: publish it as an fp32 partial
        float *w = a.ws + (size_t)pid * 65536u + row;
#pragma unroll 1
        for (int col = 0; col < 256; col += 32) {
          uint32_t v[32];
          tmem_ld32(taddr + (uint32_t)col, v);
          tmem_wait_ld(v);
#pragma unroll
          for (int i = 0; i < 32; i++) __stcg(w + (size_t)(col + i) * 256u, __uint_as_float(v[i]));
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) {
          uint32_t *f = a.flags + pid * 8u + peer * 4u + (uint32_t)q;
          asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(f), "r"(a.epoch) : "memory");
        }
      } else {
        // this pair finishes the tile: add the partials of the lower pairs holding stages [0, k0)
        const uint64_t gm = (uint64_t)(sg.t % a.mt) * 256u + row;
        const uint64_t n0 = (uint64_t)(sg.t / a.mt) * 256u;
        const uint32_t base = sg.t * nk;
        uint32_t qlo = pid;  // contributors are pairs [qlo, pid)
        bool ok = true;
        for (uint32_t lo = sg.k0; lo > 0 && qlo > 0;) {
          qlo--;
          ok = ok && sk_wait_flag(a.flags + qlo * 8u + peer * 4u + (uint32_t)q, a.epoch);
          const uint32_t uq = sk_u0(qlo, a.units, npairs);
          lo = uq > base ? uq - base : 0u;
        }
        if (!__all_sync(0xffffffffu, ok)) {
          if (lane == 0) atomicOr(&g_tc_error, 4u);
          *abort_flag = 1;
        }
#pragma unroll 1
        for (int col = 0; col < 256; col += 32) {
          uint32_t v[32];
          tmem_ld32(taddr + (uint32_t)col, v);
          tmem_wait_ld(v);
          float acc[32];
#pragma unroll
          for (int i = 0; i < 32; i++) acc[i] = __uint_as_float(v[i]);
          for (uint32_t qq = qlo; qq < pid; qq++) {
            const float *w = a.ws + (size_t)qq * 65536u + (size_t)col * 256u + row;
#pragma unroll
            for (int i = 0; i < 32; i++) acc[i] += __ldcg(w + (size_t)i * 256u);
          }
          int32_t o[32];
#pragma unroll
          for (int i = 0; i < 32; i++) o[i] = __float2int_rn(acc[i]);
          store_result_cols<32>(a.C, a.M, a.N, gm, n0 + (uint64_t)col, o);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) {  // this warp is done with the buffer: tell the leader's MMA thread
        if (peer == 0) {
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(acc_empty + 8 * b) : "memory");
        } else {
          const uint32_t rb = map_to_rank(acc_empty + 8 * b, 0);
          asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(rb) : "memory");
        }
      }
      j++;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(512));
  }
}

// Throughput probe: one CTA per SM, one thread issuing back-to-back
// tcgen05.mma (M=128, N=256) from fixed zeroed shared tiles; KIND 0 = e4m3
// (K=32), KIND 1 = bf16 (K=16).  A commit + bounded wait closes every 64
// MMAs.  The issue loop holds nothing but the MMAs: one thread's issue rate
// is close to the tensor core's, and a runtime branch per MMA measurably
// lowered the rate it reported.
template <int KIND>
__global__ void __launch_bounds__(128, 1) peak_tc_kernel(int iters) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 48 * 1024);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1);
  for (int i = threadIdx.x; i < 48 * 1024 / 16; i += blockDim.x)
    reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_u32(smem), b0 = a0 + 16 * 1024;
    const uint32_t idesc = (1u << 4) | (KIND ? ((1u << 7) | (1u << 10)) : 0u) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
    uint32_t phase = 0;
    for (int it = 0; it < iters; it++) {
#pragma unroll 1
      for (int rep = 0; rep < 16; rep++)
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
          const uint64_t ad = sw128_desc(a0 + kk * 32), bd = sw128_desc(b0 + kk * 32);
          if constexpr (KIND == 1)
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(idesc), "r"(1u));
          else
            mma_f8(tmem, ad, bd, idesc, 1u);
        }
      mma_commit(smem_u32(bar));
      bool done = false;
      for (uint32_t w = 0; w < kTcWaitLimit && !done; ++w) done = mbar_try(smem_u32(bar), phase);
      if (!done) {  // wait (bounded) once more for the MMAs in flight: TMEM is freed below
        atomicOr(&g_tc_error, 2u);
        mbar_drain(smem_u32(bar), phase);
        break;
      }
      phase ^= 1;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
  }
}

// e4m3 byte of a small integer (|v| <= 16 is exact: 3 mantissa bits below 2^4).
uint32_t e4m3_int(int v) {
  if (v == 0) return 0u;
  const uint32_t sign = v < 0 ? 0x80u : 0u;
  int m = v < 0 ? -v : v, e = 0;
  while ((m >> (e + 1)) != 0) e++;
  const int frac = (m - (1 << e)) << (3 - e);  // exact for e <= 3, zero for m = 16
  return sign | (uint32_t)((e + 7) << 3) | (uint32_t)(e <= 3 ? frac : 0);
}

// Value of code `code` (bit b = plane first+b) for planes [first, first+count) of operand m.
int code_value(const Mat &m, int first, int count, int code) {
  if (m.bipolar()) return (code & 1) ? 1 : -1;
  int v = 0;
  for (int b = 0; b < count; b++)
    if ((code >> b) & 1) {
      const int plane = first + b;
      const int w = 1 << plane;
      v += (m.issigned && plane == (int)m.nbits - 1) ? -w : w;
    }
  return v;
}

TcOperand make_operand(const Mat &m, bool digits) {
  TcOperand op;
  memset(&op, 0, sizeof(op));
  op.bip = m.bipolar() ? 1 : 0;
  op.ntiles = digits ? 1 : (int)m.nbits;
  for (int t = 0; t < op.ntiles; t++) {
    op.first[t] = digits ? 0 : t;
    op.count[t] = digits ? (int)m.nbits : 1;
    for (int code = 0; code < (1 << op.count[t]); code++)
      op.tab[t][code >> 2] |= e4m3_int(code_value(m, op.first[t], op.count[t], code)) << (8 * (code & 3));
  }
  return op;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The process-wide lookups below are idempotent: threads that race on a
// first call store the same value, so relaxed atomics suffice.
EncodeTiledFn encode_fn() {
  static std::atomic<EncodeTiledFn> fn{nullptr};
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

// Tensor map over all planes of one operand: 2-D u64 [nbits * nrows_a][wpr], box 128 rows x 2 words.
bool make_plane_map(CUtensorMap *map, const Mat &m) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {m.wpr(), m.nbits * m.nrows_a};
  cuuint64_t strides[1] = {m.wpr() * 8};
  cuuint32_t box[2] = {2, 128};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, m.planes, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

uint64_t max_abs(const Mat &m) {
  if (m.bipolar()) return 1;
  return m.issigned ? (1ull << (m.nbits - 1)) : ((1ull << m.nbits) - 1);
}

constexpr size_t kSmemCap = 225 * 1024;

size_t tc_smem(int ntA, int ntB, int wa, int wb, int bn, int no) {
  const size_t op_stage = (size_t)ntA * kBM * kRowB + (size_t)ntB * bn * kRowB;
  const size_t pk_stage = (size_t)wa * kBM * kPkRowB + (size_t)wb * bn * kPkRowB;
  return 1024 + no * op_stage + kPkSlots * pk_stage + 8 * (2 * kPkSlots + 2 * no + 2) + 16;
}

}  // namespace

// Map of a digit matrix (rows x cols, 16-row blocks: digit_offset) as the
// 4-D tensor [rows/16][cols/128][16][128] bytes; a box is box_rows rows (a
// multiple of 16, <= 256) of one 128-digit column chunk, 128-byte swizzled.
bool tc_map_u8(void *map, const uint8_t *base, uint64_t cols, uint64_t rows, uint32_t box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || box_rows == 0 || box_rows > 256 || box_rows % 16 || cols % 128 || rows % 16) return false;
  cuuint64_t dims[4] = {128, 16, cols / 128, rows / 16};
  cuuint64_t strides[3] = {128, 2048, (cols / 128) * 2048};
  cuuint32_t box[4] = {128, 16, 1, box_rows / 16};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  return fn(reinterpret_cast<CUtensorMap *>(map), CU_TENSOR_MAP_DATA_TYPE_UINT8, 4, (void *)base, dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Map of a nibble matrix (rows x cols codes, blocks of nibble_offset) as the
// 4-D tensor [rows/16][cols/128][16][64] bytes; a box is 256 rows of one
// 128-column chunk, 64-byte swizzled.
bool tc_map_nibbles(void *map, const uint8_t *base, uint64_t cols, uint64_t rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || cols % 128 || rows % 256 || rows == 0) return false;
  cuuint64_t dims[4] = {64, 16, cols / 128, rows / 16};
  cuuint64_t strides[3] = {64, 1024, (cols / 128) * 1024};
  cuuint32_t box[4] = {64, 16, 1, 16};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  return fn(reinterpret_cast<CUtensorMap *>(map), CU_TENSOR_MAP_DATA_TYPE_UINT8, 4, (void *)base, dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void tc_digit_table(const Mat &m, uint32_t tab[4]) {
  const TcOperand op = make_operand(m, true);
  for (int i = 0; i < 4; i++) tab[i] = op.tab[0][i];
}

uint64_t tc_max_abs(const Mat &m) { return max_abs(m); }

bool tc_encoder_available() { return encode_fn() != nullptr; }

// A tensor-core pipe is exact for a context when every partial sum stays an
// integer below 2^24 in fp32 and each operand's values fit e4m3 exactly (at
// most 4 bits).  The shared-memory variants also need every plane of a stage
// in their operand ring (at most 5 planes in total) and rows of whole 128-bit
// stages (an even number of plane words).
bool tc_exact(const gbs_ctx *c, int pipe) {
  const Mat &A = c->lhs, &B = c->rhs;
  if (A.nbits > 4 || B.nbits > 4 || A.nrows == 0 || B.nrows == 0 || A.ncols == 0) return false;
  if ((pipe == GBS_PIPE_TC_PAIRS || pipe == GBS_PIPE_TC_SMEM) && A.nbits + B.nbits > 5) return false;
  // the shared-memory variants load the planes in 2-word (128-bit) stages by TMA: rows of an even word count
  if ((pipe == GBS_PIPE_TC_PAIRS || pipe == GBS_PIPE_TC_SMEM) && (A.wpr() & 1)) return false;
  if ((double)A.ncols * (double)max_abs(A) * (double)max_abs(B) >= 16777216.0) return false;
  if (A.nrows_a * A.nbits > (1ull << 31) || B.nrows_a * B.nbits > (1ull << 31) || A.ncols_a >= (1ull << 31))
    return false;
  return encode_fn() != nullptr;
}

cudaError_t launch_gemm_tc(gbs_ctx *c, cudaStream_t s, bool digits, int bn_req) {
  if (!c->tc_maps_ready) {
    if (!make_plane_map(reinterpret_cast<CUtensorMap *>(c->tc_map_a), c->lhs) ||
        !make_plane_map(reinterpret_cast<CUtensorMap *>(c->tc_map_b), c->rhs))
      return cudaErrorInvalidValue;
    c->tc_maps_ready = true;
  }
  const Mat &A = c->lhs, &B = c->rhs;
  TcArgs a;
  memset(&a, 0, sizeof(a));
  a.C = result_ptr(c);
  a.M = A.nrows;
  a.N = B.nrows;
  a.K = A.ncols;
  a.nstages = (uint32_t)(A.wpr() / 2);
  a.a_rows = (uint32_t)A.nrows_a;
  a.b_rows = (uint32_t)B.nrows_a;
  a.wa = (int)A.nbits;
  a.wb = (int)B.nbits;
  a.A = make_operand(A, digits);
  a.B = make_operand(B, digits);
  const int bn = (bn_req == 128 || bn_req == 256) ? bn_req : ((digits && a.N > 128) ? 256 : 128);
  // kind::f8f6f4: D fp32, A and B e4m3, both K-major, M = 128, N = bn
  a.idesc = (1u << 4) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
  int no = 4;
  while (no > 1 && tc_smem(a.A.ntiles, a.B.ntiles, a.wa, a.wb, bn, no) > kSmemCap) no--;
  a.no = no;
  const size_t smem = tc_smem(a.A.ntiles, a.B.ntiles, a.wa, a.wb, bn, no);
  if (smem > kSmemCap) return cudaErrorInvalidConfiguration;
  const CUtensorMap &ma = *reinterpret_cast<const CUtensorMap *>(c->tc_map_a);
  const CUtensorMap &mb = *reinterpret_cast<const CUtensorMap *>(c->tc_map_b);
  cudaError_t e;
  if (bn == 256) {
    e = cudaFuncSetAttribute(gemm_tc_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.M + kBM - 1) / kBM), (unsigned)((a.N + 255) / 256));
    gemm_tc_kernel<256><<<grid, kThreads, smem, s>>>(ma, mb, a);
  } else {
    e = cudaFuncSetAttribute(gemm_tc_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.M + kBM - 1) / kBM), (unsigned)((a.N + 127) / 128));
    gemm_tc_kernel<128><<<grid, kThreads, smem, s>>>(ma, mb, a);
  }
  count_launch();
  return cudaGetLastError();
}

namespace {

// Tensor map over a digit matrix ([drows][dcols] in 16-row blocks), box_rows x 128 digits, 128-byte swizzle.
bool make_digit_map(CUtensorMap *map, const uint8_t *digits, const Mat &m, uint32_t box_rows = 128) {
  return tc_map_u8(map, digits, m.dcols, m.drows, box_rows);
}

cudaError_t expand_side(gbs_ctx *c, int side, cudaStream_t s) {
  cudaError_t e = ensure_digit_buffer(c, side);
  if (e != cudaSuccess) return e;
  e = launch_expand(make_expand_job(side ? c->rhs : c->lhs, c->digits[side]), s);
  if (e == cudaSuccess) c->digits_valid[side] = true;
  return e;
}

cudaError_t expand_nibble_side(gbs_ctx *c, int side, cudaStream_t s) {
  cudaError_t e = ensure_nibble_buffer(c, side);
  if (e != cudaSuccess) return e;
  e = launch_expand(make_nibble_job(side ? c->rhs : c->lhs, c->nibbles[side]), s);
  if (e == cudaSuccess) c->nibbles_valid[side] = true;
  return e;
}

}  // namespace

namespace {

int sm_count_cached() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  int n = cache[dev].load(std::memory_order_relaxed);
  if (!n) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) cudaGetLastError();
    n = v > 0 ? v : 1;
    cache[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

// Stages of the pair kernel's ring for BN-column tiles, and its shared memory.
int pair_stages(int bn) {
  const size_t stage_bytes = kPairHalfBytes + (size_t)(bn / 2) * kRowB;
  int stages = kPairStagesMax;
  while (stages > 2 && 1024 + stages * stage_bytes + 8 * (2 * stages + 2) + 16 > kPairSmemCap) stages--;
  return stages;
}
size_t pair_smem_bytes(int bn) {
  const int stages = pair_stages(bn);
  return 1024 + stages * (kPairHalfBytes + (size_t)(bn / 2) * kRowB) + 8 * (2 * stages + 2) + 16;
}

// Calls f with the kernel instance of `splits` and `bn` (1/2/4 x 256/128).
template <typename F>
cudaError_t with_pair_kernel(int splits, int bn, F f) {
  if (bn == 128) {
    if (splits == 4) return f(gemm_tc_pair_kernel<4, 128>);
    if (splits == 2) return f(gemm_tc_pair_kernel<2, 128>);
    return f(gemm_tc_pair_kernel<1, 128>);
  }
  if (splits == 4) return f(gemm_tc_pair_kernel<4, 256>);
  if (splits == 2) return f(gemm_tc_pair_kernel<2, 256>);
  return f(gemm_tc_pair_kernel<1, 256>);
}

// Programmatic stream serialization for a launch on `s`: on unless GBS_PDL=0,
// the stream is the legacy default stream (which synchronises with others) or
// the stream is being captured (graph launches keep plain edges).
bool pdl_for(cudaStream_t s) {
  if (!pdl_enabled() || s == nullptr) return false;
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return st == cudaStreamCaptureStatusNone;
}

void pair_launch_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute (&attr)[2], int splits, int bn, size_t smem,
                        cudaStream_t s) {
  with_pair_kernel(splits, bn, [&](auto kern) {
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  cfg = cudaLaunchConfig_t{};
  cfg.blockDim = dim3(kPairThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2 * splits;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_for(s) ? 2 : 1;
}

// Clusters of 2 * splits CTAs that fit the GPU at once (they are placed within
// one GPC each), cached per device.
int pair_max_clusters(int splits, int bn) {
  static std::atomic<int> cache[64][5][2];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  std::atomic<int> &slot = cache[dev][splits][bn == 128 ? 1 : 0];
  int v = slot.load(std::memory_order_relaxed);
  if (v == 0) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    pair_launch_config(cfg, attr, splits, bn, pair_smem_bytes(bn), nullptr);
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(2 * splits, 1, 1);
    int n = 0;
    cudaError_t e = with_pair_kernel(splits, bn, [&](auto kern) { return cudaOccupancyMaxActiveClusters(&n, kern, &cfg); });
    if (e != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    v = n > 0 ? n : -1;
    slot.store(v, std::memory_order_relaxed);
  }
  return v > 0 ? v : 0;
}

// K split of a grid of `tiles` pair tiles: the largest of 4 or 2 that keeps
// >= 8 stages per chunk and fits one wave, else 1.
int pair_splits(uint64_t tiles, uint32_t nstages, int bn) {
  for (int cand : {4, 2})
    if (nstages / cand >= 8 && tiles <= (uint64_t)pair_max_clusters(cand, bn)) return cand;
  return 1;
}

// Shared memory of the persistent and stream-K pair kernels (256-column
// tiles, two TMEM accumulators) and their ring depth.
int pair_loop_stages() {
  int stages = pair_stages(256);
  while (stages > 2 && 1024 + (size_t)stages * 2 * kPairHalfBytes + 8 * (2 * stages + 5) + 16 > kPairSmemCap) stages--;
  return stages;
}
size_t pair_loop_smem(int stages) { return 1024 + (size_t)stages * 2 * kPairHalfBytes + 8 * (2 * stages + 5) + 16; }

// SM pairs the stream-K kernel can hold at once (its clusters of 2 are placed
// within one GPC each), cached per device; every pair of a launch must be
// resident together, since a tile's last pair waits for lower pairs' partials.
int streamk_max_pairs() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    const size_t smem = pair_loop_smem(pair_loop_stages());
    int n = 0;
    if (cudaFuncSetAttribute(gemm_tc_pair_streamk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
        cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 2;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(2);
      cfg.blockDim = dim3(kPairThreads);
      cfg.dynamicSmemBytes = smem;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      if (cudaOccupancyMaxActiveClusters(&n, gemm_tc_pair_streamk_kernel, &cfg) != cudaSuccess) n = 0;
    }
    cudaGetLastError();
    v = n > 0 ? n : -1;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v > 0 ? v : 0;
}

// Minimum K stages per pair for a stream-K launch: fewer pairs than the GPU
// holds when the whole GEMM has too few units to give each pair this many.
constexpr uint32_t kStreamKMinUnits = 8;

// Launches the stream-K pair kernel over the context's digit matrices
// (maps ready); allocates its workspace on first use.
cudaError_t launch_pair_streamk(gbs_ctx *c, cudaStream_t s, const TmaArgs &ta) {
  const uint64_t mt = (ta.M + 255) / 256, nt = (ta.N + 255) / 256;
  const uint64_t units = mt * nt * ta.nstages;
  const int maxp = streamk_max_pairs();
  if (maxp <= 0 || units == 0 || units > 0xFFFFFFFFull) return cudaErrorInvalidConfiguration;
  const uint32_t pairs =
      (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)maxp, units / kStreamKMinUnits));
  if (c->sk_pairs < pairs) {
    if (c->sk_ws) cudaFree(c->sk_ws);
    if (c->sk_flags) cudaFree(c->sk_flags);
    c->sk_ws = nullptr;
    c->sk_flags = nullptr;
    c->sk_pairs = 0;
    cudaError_t e = dev_alloc((void **)&c->sk_ws, (size_t)pairs * 65536 * sizeof(float));
    if (e == cudaSuccess) e = dev_alloc((void **)&c->sk_flags, (size_t)pairs * 8 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(c->sk_flags, 0, (size_t)pairs * 8 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    c->sk_pairs = pairs;
    c->sk_epoch = 0;
  }
  if (++c->sk_epoch == 0) c->sk_epoch = 1;  // flags start at 0: epoch 0 is never a live launch
  SkArgs a;
  memset(&a, 0, sizeof(a));
  a.C = ta.C;
  a.ws = c->sk_ws;
  a.flags = c->sk_flags;
  a.M = ta.M;
  a.N = ta.N;
  a.nk = ta.nstages;
  a.mt = (uint32_t)mt;
  a.units = (uint32_t)units;
  a.epoch = c->sk_epoch;
  a.idesc = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
  a.stages = pair_loop_stages();
  const size_t smem = pair_loop_smem(a.stages);
  cudaError_t e =
      cudaFuncSetAttribute(gemm_tc_pair_streamk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim = dim3(2 * pairs);
  cfg.blockDim = dim3(kPairThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_for(s) ? 2 : 1;
  const CUtensorMap &ma = *reinterpret_cast<const CUtensorMap *>(c->tc_map_da);
  const CUtensorMap &mb = *reinterpret_cast<const CUtensorMap *>(c->tc_map_db);
  e = cudaLaunchKernelEx(&cfg, gemm_tc_pair_streamk_kernel, ma, mb, a);
  count_launch();
  c->last_pair_bn = 256;
  c->last_pair_splits = 1;
  c->last_pair_persistent = false;
  c->last_pair_streamk = (int)pairs;
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace

// GBS_PDL=0 in the environment launches the tensor-core kernels without
// programmatic stream serialization (read once per process).
bool pdl_enabled() {
  static const bool on = [] {
    const char *v = getenv("GBS_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

cudaError_t launch_gemm_tc_hbm(gbs_ctx *c, cudaStream_t s, int bn_req) {
  if (bn_req < 0 && (c->lhs.nrows < 256 || c->rhs.nrows < 256)) {
    // a side of fewer than 256 rows: the persistent kernel over a one-problem
    // plan (larger side as the MMA's 128-row operand, MMA N down to 16)
    if (!c->plan1_ready) {
      if (!c->plan1) c->plan1 = new TcgPlan();
      gbs_ctx *one[1] = {c};
      if (tcg_plan_build(c->plan1, one, 1) != GBS_OK) return cudaErrorInvalidValue;
      c->plan1_ready = true;
    }
    for (int side = 0; side < 2; side++) {  // the digit and nibble matrices the plan reads
      cudaError_t e = cudaSuccess;
      if (((c->plan1->sides[0] >> side) & 1) && !c->digits_valid[side]) e = expand_side(c, side, s);
      if (e == cudaSuccess && ((c->plan1->sides[0] >> (2 + side)) & 1) && !c->nibbles_valid[side])
        e = expand_nibble_side(c, side, s);
      if (e != cudaSuccess) return e;
    }
    uint32_t *err = tc_error_ptr();
    if (!err) return cudaErrorInvalidSymbol;
    return tcg_gemm(*c->plan1, err, s, c->out);
  }
  for (int side = 0; side < 2; side++)
    if (!c->digits_valid[side]) {
      cudaError_t e = expand_side(c, side, s);
      if (e != cudaSuccess) return e;
    }
  if (!c->digit_maps_ready) {
    if (!make_digit_map(reinterpret_cast<CUtensorMap *>(c->tc_map_da), c->digits[0], c->lhs) ||
        !make_digit_map(reinterpret_cast<CUtensorMap *>(c->tc_map_db), c->digits[1], c->rhs))
      return cudaErrorInvalidValue;
    c->digit_maps_ready = true;
  }
  TmaArgs a;
  memset(&a, 0, sizeof(a));
  a.C = result_ptr(c);
  a.M = c->lhs.nrows;
  a.N = c->rhs.nrows;
  a.nstages = (uint32_t)(c->lhs.dcols / 128);
  if (bn_req == kPairVariantStreamK) return launch_pair_streamk(c, s, a);
  if (bn_req == kPairVariant || bn_req == kPairVariant128 || bn_req == kPairVariantPersistent || bn_req < 0 ||
      pair_split_variant(bn_req)) {
    // 256 x BN tiles on SM pairs
    // Tile width and K split.  A split sums partials over distributed shared
    // memory, which costs more the more chunks there are: candidates in order
    // of preference, the first that keeps at least half the SM pairs busy in
    // one wave wins, else the one that keeps the most busy.  (An M=256 N=128
    // pair MMA takes as long as an N=256 one, so narrow tiles only pay where
    // they replace a wider split.)
    const uint64_t mt = (a.M + 255) / 256;
    int bn = bn_req == kPairVariant128 ? 128 : 256;
    int splits = pair_splits(mt * ((a.N + bn - 1) / bn), a.nstages, bn);
    if (pair_split_variant(bn_req)) {  // tile width and K split both forced (a tuner candidate)
      bn = bn_req / 10;
      splits = bn_req % 10;
      const uint64_t tiles = mt * ((a.N + bn - 1) / bn);
      if (splits > 1 && (a.nstages < (uint32_t)splits || tiles > (uint64_t)pair_max_clusters(splits, bn)))
        splits = 1;  // every K chunk needs a stage, and all clusters of the grid must fit at once
    }
    if (bn_req < 0) {
      const uint64_t pairs = (uint64_t)sm_count_cached() / 2;
      static const int cand[6][2] = {{256, 1}, {256, 2}, {128, 1}, {128, 2}, {256, 4}, {128, 4}};
      uint64_t best_used = 0;
      for (const auto &cv : cand) {
        const int cb = cv[0], cs = cv[1];
        const uint64_t tiles = mt * ((a.N + cb - 1) / cb);
        if (cs > 1 && (a.nstages / cs < 8 || tiles > (uint64_t)pair_max_clusters(cs, cb))) continue;
        const uint64_t used = std::min<uint64_t>(tiles * cs, pairs);
        if (used > best_used) {
          best_used = used;
          bn = cb;
          splits = cs;
        }
        if (2 * used >= pairs) break;
      }
    }
    if (bn == 128 && !c->digit_map_b64_ready) {
      if (!make_digit_map(reinterpret_cast<CUtensorMap *>(c->tc_map_db64), c->digits[1], c->rhs, 64))
        return cudaErrorInvalidValue;
      c->digit_map_b64_ready = true;
    }
    a.splits = splits;
    a.idesc = (1u << 4) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
    // More 256 x 256 tiles than one wave holds: the persistent kernel, whose
    // pairs loop over tiles with two TMEM accumulators, so each tile's
    // epilogue overlaps the next tile's MMAs instead of a second wave
    // repeating launch, setup and the first load (variant 514 forces it, with
    // about three tiles per pair)
    const uint64_t ntiles = mt * ((a.N + 255) / 256);
    const uint64_t fit = (uint64_t)std::max(1, pair_max_clusters(1, 256));
    if (bn_req == kPairVariantPersistent || (bn_req < 0 && bn == 256 && splits == 1 && ntiles > fit)) {
      a.splits = 1;
      a.idesc = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
      a.stages = pair_stages(256);
      size_t smem = 1024 + (size_t)a.stages * 2 * kPairHalfBytes + 8 * (2 * a.stages + 5) + 16;
      while (smem > kPairSmemCap && a.stages > 2) {
        a.stages--;
        smem = 1024 + (size_t)a.stages * 2 * kPairHalfBytes + 8 * (2 * a.stages + 5) + 16;
      }
      const uint64_t npairs =
          bn_req == kPairVariantPersistent ? std::max<uint64_t>(1, (ntiles + 2) / 3) : std::min(ntiles, fit);
      cudaError_t e = cudaFuncSetAttribute(gemm_tc_pair_persistent_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      cudaLaunchConfig_t cfg;
      cfg = cudaLaunchConfig_t{};
      cudaLaunchAttribute attr[2];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 2;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[1].val.programmaticStreamSerializationAllowed = 1;
      cfg.gridDim = dim3((unsigned)(2 * npairs));
      cfg.blockDim = dim3(kPairThreads);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cfg.attrs = attr;
      cfg.numAttrs = pdl_for(s) ? 2 : 1;
      if (!c->digit_maps_ready) return cudaErrorInvalidValue;
      const CUtensorMap &ma = *reinterpret_cast<const CUtensorMap *>(c->tc_map_da);
      const CUtensorMap &mb = *reinterpret_cast<const CUtensorMap *>(c->tc_map_db);
      e = cudaLaunchKernelEx(&cfg, gemm_tc_pair_persistent_kernel, ma, mb, a);
      count_launch();
      c->last_pair_bn = 256;
      c->last_pair_splits = 1;
      c->last_pair_persistent = true;
      c->last_pair_streamk = 0;
      return e != cudaSuccess ? e : cudaGetLastError();
    }
    a.stages = pair_stages(bn);
    a.wait_limit = c->debug_wait_limit;
    const size_t smem = pair_smem_bytes(bn);
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    pair_launch_config(cfg, attr, a.splits, bn, smem, s);
    cfg.gridDim = dim3((unsigned)(2 * a.splits * mt), (unsigned)((a.N + bn - 1) / bn));
    const CUtensorMap &ma = *reinterpret_cast<const CUtensorMap *>(c->tc_map_da);
    const CUtensorMap &mb = *reinterpret_cast<const CUtensorMap *>(bn == 128 ? c->tc_map_db64 : c->tc_map_db);
    cudaError_t e = with_pair_kernel(a.splits, bn, [&](auto kern) { return cudaLaunchKernelEx(&cfg, kern, ma, mb, a); });
    count_launch();
    c->last_pair_bn = bn;
    c->last_pair_splits = a.splits;
    c->last_pair_persistent = false;
    c->last_pair_streamk = 0;
    return e != cudaSuccess ? e : cudaGetLastError();
  }
  const int bn = (bn_req == 128 || bn_req == 256) ? bn_req : (a.N > 128 ? 256 : 128);
  a.idesc = (1u << 4) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
  const size_t stage_bytes = (size_t)(kBM + bn) * kRowB;
  int stages = kTmaStagesMax;
  while (stages > 2 && 1024 + stages * stage_bytes + 8 * (2 * stages + 2) + 16 > kSmemCap) stages--;
  a.stages = stages;
  const size_t smem = 1024 + stages * stage_bytes + 8 * (2 * stages + 2) + 16;
  const CUtensorMap &ma = *reinterpret_cast<const CUtensorMap *>(c->tc_map_da);
  const CUtensorMap &mb = *reinterpret_cast<const CUtensorMap *>(c->tc_map_db);
  cudaError_t e;
  if (bn == 256) {
    e = cudaFuncSetAttribute(gemm_tc_tma_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.M + kBM - 1) / kBM), (unsigned)((a.N + 255) / 256));
    gemm_tc_tma_kernel<256><<<grid, kTmaThreads, smem, s>>>(ma, mb, a);
  } else {
    e = cudaFuncSetAttribute(gemm_tc_tma_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.M + kBM - 1) / kBM), (unsigned)((a.N + 127) / 128));
    gemm_tc_tma_kernel<128><<<grid, kTmaThreads, smem, s>>>(ma, mb, a);
  }
  count_launch();
  return cudaGetLastError();
}

// tcgen05 MMA rate in FLOP/s (2 per multiply-add) for e4m3 and bf16 at full
// SM clock: the best of several ~0.2 ms bursts, each too short for the power
// limit to pull the clock down (longer loops settle ~25 % lower on a
// 1.4 kW GB300).  The kernels it is the ceiling of run for tens of
// microseconds at a time, at full clock.
int tc_peaks(double *f8, double *bf16) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 1024 + 48 * 1024 + 64;
  cudaError_t e = cudaFuncSetAttribute(peak_tc_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(peak_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_tc_peaks");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double out[2] = {0, 0};
  // rate from the difference of a short and a long burst (launch cost cancels),
  // best of several, with idle gaps so the power draw stays low between them
  const int lo = 20, hi = 60;
  for (int kind = 0; kind < 2; kind++) {
    auto launch = [&](int iters) {
      if (kind) peak_tc_kernel<1><<<sms, 128, smem>>>(iters);
      else peak_tc_kernel<0><<<sms, 128, smem>>>(iters);
    };
    launch(4);
    cudaDeviceSynchronize();
    float best[2] = {1e30f, 1e30f};
    for (int r = 0; r < 6; r++)
      for (int v = 0; v < 2; v++) {
        std::this_thread::sleep_for(std::chrono::milliseconds(1));
        cudaEventRecord(e0);
        launch(v ? hi : lo);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best[v] = std::min(best[v], ms);
      }
    const double k = kind ? 16.0 : 32.0, dt = (double)(best[1] - best[0]);
    out[kind] = dt > 0 ? 2.0 * sms * (double)(hi - lo) * 64.0 * 128.0 * 256.0 * k / (dt * 1e-3) : 0.0;
  }
  count_launch(26);
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_tc_peaks");
  if (f8) *f8 = out[0];
  if (bf16) *bf16 = out[1];
  return GBS_OK;
}

uint32_t *tc_error_ptr() {
  static std::atomic<uint32_t *> addr[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  uint32_t *a = addr[dev].load(std::memory_order_relaxed);
  if (!a) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tc_error) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    a = static_cast<uint32_t *>(p);
    addr[dev].store(a, std::memory_order_relaxed);
  }
  return a;
}

uint32_t tc_error_word() {
  uint32_t v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(v)) != cudaSuccess) {
    cudaGetLastError();
    return 0xFFFFFFFFu;
  }
  return v;
}

}  // namespace gbs

using namespace gbs;

// Test hook of the tensor-core kernels' bounded waits: one launch of the
// SM-pair kernel that loads and multiplies nothing, so its first wait gives up
// after `rounds` try_wait rounds; the kernel then takes its abort path (error
// bit, bounded drains, TMEM freed, clean exit) and the host reads the error.
extern "C" int gbs_debug_tc_timeout(gbs_ctx *c, uint32_t rounds, void *stream) {
  if (!c || rounds == 0) return fail(GBS_EINVAL, "gbs_debug_tc_timeout: NULL context or zero rounds");
  if (!c->lhs.imported || !c->rhs.imported) return fail(GBS_ESTATE, "gbs_debug_tc_timeout: import both operands first");
  if (!tc_exact(c, GBS_PIPE_TC) || c->lhs.nrows < 256 || c->rhs.nrows < 256)
    return fail(GBS_EUNSUPPORTED, "gbs_debug_tc_timeout: needs a context the SM-pair kernel runs (M, N >= 256)");
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(c->device) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "gbs_debug_tc_timeout: cudaSetDevice");
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t zero = 0;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(zero));
  const int saved_pipe = c->pipe, saved_variant = c->variant;
  int rc = GBS_OK;
  if (e == cudaSuccess) {
    c->pipe = GBS_PIPE_TC;
    c->variant = 2561;  // one 256 x 256 tile per SM pair, no K split
    c->debug_wait_limit = rounds;
    rc = gbs_gemm(c, stream);
    c->debug_wait_limit = 0;
    c->pipe = saved_pipe;
    c->variant = saved_variant;
    e = cudaStreamSynchronize(s);
  }
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&err, g_tc_error, sizeof(err));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(zero));
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_debug_tc_timeout");
  if (rc != GBS_OK) return rc;
  if (err) return fail(GBS_ETIMEOUT, "gbs_debug_tc_timeout: the kernel's bounded wait gave up (error bits " +
                                         std::to_string(err) + "); it drained, freed TMEM and returned");
  return fail(GBS_EINVAL, "gbs_debug_tc_timeout: the wait did not run out");
}

