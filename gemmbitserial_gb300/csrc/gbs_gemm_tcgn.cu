// gbs_gemm_tcgn.cu -- persistent tensor-core GEMM over a table of problems
// whose larger operand is streamed as 4-bit codes and decoded to e4m3
// digits in shared memory.
//
// The reference multiplies bit planes pairwise, AND + popcount weighted by
// +-2^(i+j) (arch-generic.hpp:179-192), over a host loop of problems
// (benchmark.cpp:192-206).  The digit kernel (gbs_gemm_tcg.cu) reads both
// operands as one-byte e4m3 digits (each element's whole value), which for
// the memory-bound problems of a group (one side of at most a few hundred
// rows) streams one byte per element of the larger side.  Here the larger
// side is stored as a "nibble matrix" -- each element's plane code in 4 bits
// -- and expanded in shared memory: a byte-permute lookup turns four codes
// into four exact e4m3 values in one instruction (codes of up to 3 bits; six
// for 4-bit codes), so the kernel reads half the bytes and decodes ~0.5
// instructions per element.  (Decoding the bit planes themselves, a bit
// transposition, measured ~3.7 instructions per element: issue-bound.)
//
// Roles: the smaller side is the MMA's M operand ("MMA-A": 128-row tiles of
// its digit matrix, TMA), the larger side its N operand ("MMA-B": 256-row
// tiles, decoded), so one tcgen05.mma covers 256 rows of the larger side.
// Products and partial sums are exact integers in the fp32 accumulator while
// K * max|a| * max|b| < 2^24, the same bound as the digit kernel.
//
// Nibble matrix layout: [drows/16][dcols/128] blocks of 16 rows x 64 bytes
// (128 codes per row, the even column in the low nibble), read through a 4-D
// tensor map whose box is 256 rows of one 128-column chunk with 64-byte
// swizzle (the decoders' 16-byte reads are then free of bank conflicts).
//
// Warps: 0 nibble loads (lane 0); 1 TMEM allocation and MMA issue (lane 0);
// 2 MMA-A digit loads (lane 0); 3-6 epilogue of tile j while the MMAs of tile
// j + 1 run; 7-22 decoders, half a row of the 256-row stage per thread.  Every
// mbarrier wait is bounded; on timeout the CTA sets a bit in the caller's
// error word, stops issuing, drains what it issued and frees TMEM.
#include <algorithm>

#include "gbs_internal.h"
#include "gbs_tc_common.cuh"

namespace gbs {
namespace {

constexpr int kNbDecWarps = 16;  // 512 decoder threads: half a row (64 codes) of the 256-row MMA-B stage each
constexpr int kNbDec0 = 7;      // first decoder warp
constexpr int kNbThreads = 32 * (kNbDec0 + kNbDecWarps);
constexpr int kNbASlots = 4;  // MMA-A digit stages, 128 rows x 128 digits
constexpr int kNbNSlots = 4;  // nibble stages, 256 rows x 64 bytes
constexpr int kNbBSlots = 3;  // decoded MMA-B stages, 256 rows x 128 digits
constexpr uint32_t kNbASlotBytes = 128 * 128;
constexpr uint32_t kNbNSlotBytes = 256 * 64;
constexpr uint32_t kNbBSlotBytes = 256 * 128;
constexpr uint32_t kNbAccCols = 256;
constexpr int kNbBars = 2 * (kNbASlots + kNbNSlots + kNbBSlots) + 2 * 2 + 1;
constexpr size_t kNbSmem = 1024 + kNbASlots * kNbASlotBytes + kNbNSlots * kNbNSlotBytes +
                           kNbBSlots * kNbBSlotBytes + 8 * kNbBars + 16;
static_assert(kNbSmem <= 227 * 1024, "nibble kernel shared memory");

__device__ __forceinline__ uint32_t snake(uint32_t j, uint32_t b, uint32_t G) {
  return j * G + ((j & 1u) ? G - 1u - b : b);
}

__device__ __forceinline__ bool ntile_ok(const TcgTile &t, const TcgProblem &P, uint32_t nprob) {
  return t.p < nprob && P.nk > 0 && (t.r + 1) * 128u <= P.a_rows && (t.c + 1) * 256u <= P.b_rows &&
         P.a_bytes >= 2048u && P.a_bytes <= kNbASlotBytes && P.a_bytes % 2048u == 0;
}

// prmt.b32 in its generic mode: result byte i is source byte s[4i+2:4i] of
// {b, a}, or that byte's sign replicated when s[4i+3] is set.
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}

// e4m3 bytes of the 4 codes in the low 16 bits of x (nibble i = column i).
template <bool W4>
__device__ __forceinline__ uint32_t lut4(uint32_t x, const uint32_t (&tab)[4]) {
  if (!W4) return prmt(tab[0], tab[1], x);  // codes 0..7: the selectors' sign bits are clear
  const uint32_t sel = x & 0x7777u;
  const uint32_t lo = prmt(tab[0], tab[1], sel), hi = prmt(tab[2], tab[3], sel);
  // 0xFF in byte i when code i >= 8: its bit 3 is the sign bit of byte 0/1 of x << 4 (codes 0, 2)
  // or of x (codes 1, 3)
  const uint32_t m = prmt(x << 4, x, 0xD9C8u);
  return (lo & ~m) | (hi & m);
}

// Half `half` of one row of the MMA-B stage: 32 of its 64 bytes of codes
// (16-byte chunks 64-byte swizzled) -> 64 of its 128 e4m3 bytes (16-byte
// chunks 128-byte swizzled, the MMA's K-major layout).
template <bool W4>
__device__ __forceinline__ void decode_half_row(const uint8_t *src, uint8_t *dst, uint32_t row, uint32_t half,
                                                const uint32_t (&tab)[4]) {
#pragma unroll
  for (uint32_t jj = 0; jj < 2; jj++) {  // codes of columns 32j .. 32j + 31
    const uint32_t j = 2 * half + jj;
    const uint4 v = *reinterpret_cast<const uint4 *>(src + ((j ^ ((row >> 1) & 3u)) << 4));
    const uint4 d0 = make_uint4(lut4<W4>(v.x, tab), lut4<W4>(v.x >> 16, tab), lut4<W4>(v.y, tab),
                                lut4<W4>(v.y >> 16, tab));
    const uint4 d1 = make_uint4(lut4<W4>(v.z, tab), lut4<W4>(v.z >> 16, tab), lut4<W4>(v.w, tab),
                                lut4<W4>(v.w >> 16, tab));
    *reinterpret_cast<uint4 *>(dst + (((2 * j) ^ (row & 7u)) << 4)) = d0;
    *reinterpret_cast<uint4 *>(dst + (((2 * j + 1) ^ (row & 7u)) << 4)) = d1;
  }
}

// 16 accumulator columns of the warp's 32 TMEM lanes, without the wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
// Marks registers filled by TMEM loads as produced after the tcgen05.wait::ld
// issued just before (volatile asm keeps its place in program order), so no
// use of them is scheduled ahead of the wait.
__device__ __forceinline__ void regs_after_wait(uint32_t (&v)[16]) {
  asm volatile(""
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                 "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
               :
               : "memory");
}

// Rows [row, row + 256) x codes [128 k, 128 k + 128) of a nibble matrix: the
// box lands as 256 rows x 64 bytes, 64-byte swizzled.
__device__ __forceinline__ void tma_load_nibbles(uint32_t dst, const CUtensorMap *map, int k, uint32_t row,
                                                 uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(k), "r"((int)(row >> 4)), "r"(bar)
      : "memory");
}

__global__ void __launch_bounds__(kNbThreads, 1)
    gemm_tcgn_kernel(const TcgProblem *__restrict__ probs, const CUtensorMap *__restrict__ maps,
                     const TcgTile *__restrict__ tiles, uint32_t ntiles, uint32_t nprob, uint32_t *err,
                     int32_t *out0) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *aring = smem;
  uint8_t *bring = aring + kNbASlots * kNbASlotBytes;
  uint8_t *nring = bring + kNbBSlots * kNbBSlotBytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(nring + kNbNSlots * kNbNSlotBytes);
  const uint32_t a_full = smem_u32(bars), a_empty = a_full + 8 * kNbASlots;
  const uint32_t n_full = a_empty + 8 * kNbASlots, n_empty = n_full + 8 * kNbNSlots;
  const uint32_t b_full = n_empty + 8 * kNbNSlots, b_empty = b_full + 8 * kNbBSlots;
  const uint32_t acc_full = b_empty + 8 * kNbBSlots, acc_empty = acc_full + 16, mma_done = acc_empty + 16;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kNbBars);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t G = gridDim.x, b = blockIdx.x;

  if (tid == 0) {
    for (int i = 0; i < kNbASlots; i++) {
      mbar_init(a_full + 8 * i, 1);
      mbar_init(a_empty + 8 * i, 1);
    }
    for (int i = 0; i < kNbNSlots; i++) {
      mbar_init(n_full + 8 * i, 1);
      mbar_init(n_empty + 8 * i, kNbDecWarps);  // every decoder warp has read the stage
    }
    for (int i = 0; i < kNbBSlots; i++) {
      mbar_init(b_full + 8 * i, kNbDecWarps);  // every decoder warp has written its rows
      mbar_init(b_empty + 8 * i, 1);           // tcgen05.commit of the MMAs that read the slot
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(acc_full + 8 * i, 1);
      mbar_init(acc_empty + 8 * i, 4);  // one arrival per epilogue warp
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(2 * kNbAccCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 || warp == 2) {
    // ---------------- TMA: warp 0 the nibble stages (MMA-B), warp 2 the digit stages (MMA-A)
    if (lane == 0) {
      const bool nib = warp == 0;
      const int slots = nib ? kNbNSlots : kNbASlots;
      const uint32_t full = nib ? n_full : a_full, empty = nib ? n_empty : a_empty;
      uint8_t *ring = nib ? nring : aring;
      uint32_t it = 0;
      bool stop = false;
      for (uint32_t j = 0; !stop; j++) {
        const uint32_t t = snake(j, b, G);
        if (t >= ntiles) break;
        const TcgTile tl = tiles[t];
        if (tl.p >= nprob) continue;
        const TcgProblem P = probs[tl.p];
        if (!ntile_ok(tl, P, nprob)) continue;
        const CUtensorMap *m = maps + 2 * tl.p + (nib ? 1 : 0);
        const uint32_t bytes = nib ? kNbNSlotBytes : P.a_bytes;
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
        for (uint32_t k = 0; k < P.nk; k++, it++) {
          const uint32_t s = it % slots, use = it / slots;
          if (use > 0 && !mbar_wait_err(empty + 8 * s, (use - 1) & 1, abort_flag, err)) {
            stop = true;
            break;
          }
          mbar_expect_tx(full + 8 * s, bytes);
          const uint32_t dst = smem_u32(ring + s * (nib ? kNbNSlotBytes : kNbASlotBytes));
          if (nib) tma_load_nibbles(dst, m, (int)k, tl.c * 256u, full + 8 * s);
          else tma_load_digits(dst, m, (int)k, tl.r * 128u, full + 8 * s);
        }
      }
      if (*abort_flag)  // let issued copies land before the CTA can exit
        for (uint32_t q = (it > (uint32_t)slots ? it - slots : 0); q < it; q++)
          mbar_drain_err(full + 8 * (q % slots), (q / slots) & 1, err);
    }
  } else if (warp == 1) {
    // ---------------- MMA issue: 4 x (M = 128, N = 256, K = 32) per stage
    if (lane == 0) {
      uint32_t it = 0, jt = 0;
      bool ok = true;
      for (uint32_t j = 0; ok; j++) {
        const uint32_t t = snake(j, b, G);
        if (t >= ntiles) break;
        const TcgTile tl = tiles[t];
        if (tl.p >= nprob) continue;
        const TcgProblem P = probs[tl.p];
        if (!ntile_ok(tl, P, nprob)) continue;
        const uint32_t acc = jt & 1, use = jt >> 1;
        if (use > 0 && !mbar_wait_err(acc_empty + 8 * acc, (use - 1) & 1, abort_flag, err)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t d = tmem + acc * kNbAccCols;
        for (uint32_t k = 0; k < P.nk; k++, it++) {
          const uint32_t as = it % kNbASlots, bs = it % kNbBSlots;
          if (!mbar_wait_err(a_full + 8 * as, (it / kNbASlots) & 1, abort_flag, err) ||
              !mbar_wait_err(b_full + 8 * bs, (it / kNbBSlots) & 1, abort_flag, err)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t abase = smem_u32(aring + as * kNbASlotBytes), bbase = smem_u32(bring + bs * kNbBSlotBytes);
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            mma_f8(d, sw128_desc(abase + kk * 32), sw128_desc(bbase + kk * 32), P.idesc, (k | kk) != 0);
          mma_commit(a_empty + 8 * as);
          mma_commit(b_empty + 8 * bs);
        }
        if (!ok) break;
        mma_commit(acc_full + 8 * acc);
        jt++;
      }
      if (!ok) {  // issued MMAs finish before TMEM is freed
        mma_commit(mma_done);
        mbar_drain_err(mma_done, 0, err);
      }
    }
  } else if (warp < kNbDec0) {
    // ---------------- epilogue: TMEM lanes 32q .. 32q+31 (MMA-A rows) belong to this warp
    const int q = warp & 3;
    uint32_t jt = 0;
    for (uint32_t j = 0;; j++) {
      const uint32_t t = snake(j, b, G);
      if (t >= ntiles) break;
      const TcgTile tl = tiles[t];
      TcgProblem P;
      if (tl.p < nprob) P = probs[tl.p];
      if (tl.p >= nprob || !ntile_ok(tl, P, nprob)) {
        if (warp == 3 && lane == 0) atomicOr(err, 4u);
        continue;
      }
      if (out0 && tl.p == 0) P.C = out0;  // the caller's result buffer for problem 0
      const uint32_t acc = jt & 1, use = jt >> 1;
      if (!__all_sync(0xffffffffu, mbar_wait_err(acc_full + 8 * acc, use & 1, abort_flag, err))) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t row = tl.r * 128u + (uint32_t)(q * 32 + lane);  // an MMA-A row
      const uint32_t taddr = tmem + acc * kNbAccCols + ((uint32_t)(q * 32) << 16);
      const uint32_t nb = P.swap ? P.M : P.N;  // rows of MMA-B (the tile's columns)
      const uint32_t ncols = min(256u, nb - min(nb, tl.c * 256u));
      // a warp whose 32 accumulator rows all lie past the smaller side's rows stores nothing:
      // it skips the TMEM loads too (in a group most smaller sides have a few dozen rows)
      const uint32_t arows = P.swap ? P.N : P.M;
      const bool live = tl.r * 128u + (uint32_t)(q * 32) < arows;
#pragma unroll 1
      for (uint32_t col = 0; live && col < ncols; col += 32) {
        // two 16-column loads behind one wait (columns up to col + 31 < 256 stay inside the
        // accumulator; only the stores are bounded by ncols)
        uint32_t v[2][16];
#pragma unroll
        for (int h = 0; h < 2; h++) tmem_ld16(taddr + col + 16 * h, v[h]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int h = 0; h < 2; h++) regs_after_wait(v[h]);
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const uint32_t c0 = tl.c * 256u + col + 16u * h;
          if (col + 16u * h >= ncols) break;
          int32_t o[16];
#pragma unroll
          for (int i = 0; i < 16; i++) o[i] = __float2int_rn(__uint_as_float(v[h][i]));
          if (!P.swap) {  // row = m, column = n: lanes write 32 consecutive m of one n
            store_result_cols<16>(P.C, P.M, P.N, row, c0, o);
          } else if (row < P.N) {  // row = n, column = m: each lane writes a run of its result row
            int32_t *dst = P.C + (uint64_t)row * P.M + c0;
            if ((P.M & 3u) == 0) {
#pragma unroll
              for (int i = 0; i < 16; i += 4)
                if (c0 + i < P.M) *reinterpret_cast<int4 *>(dst + i) = make_int4(o[i], o[i + 1], o[i + 2], o[i + 3]);
            } else {
#pragma unroll
              for (int i = 0; i < 16; i++)
                if (c0 + i < P.M) dst[i] = o[i];
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty + 8 * acc);
      jt++;
    }
  } else {
    // ---------------- decoders: thread -> row `row` of every 256-row MMA-B stage
    const uint32_t row = (uint32_t)(tid - 32 * kNbDec0) & 255u, half = (uint32_t)(tid - 32 * kNbDec0) >> 8;
    uint32_t it = 0;
    bool ok = true;
    for (uint32_t j = 0; ok; j++) {
      const uint32_t t = snake(j, b, G);
      if (t >= ntiles) break;
      const TcgTile tl = tiles[t];
      if (tl.p >= nprob) continue;
      const TcgProblem P = probs[tl.p];
      if (!ntile_ok(tl, P, nprob)) continue;
      const uint32_t tab[4] = {P.tab[0], P.tab[1], P.tab[2], P.tab[3]};
      for (uint32_t k = 0; k < P.nk; k++, it++) {
        const uint32_t ns = it % kNbNSlots, bs = it % kNbBSlots;
        // every lane waits (and acquires); the decisions are warp-uniform for the warp barriers below
        if (!__all_sync(0xffffffffu, mbar_wait_err(n_full + 8 * ns, (it / kNbNSlots) & 1, abort_flag, err)) ||
            (it >= (uint32_t)kNbBSlots &&
             !__all_sync(0xffffffffu, mbar_wait_err(b_empty + 8 * bs, ((it / kNbBSlots) - 1) & 1, abort_flag, err)))) {
          ok = false;
          break;
        }
        const uint8_t *src = nring + ns * kNbNSlotBytes + row * 64u;
        uint8_t *dst = bring + bs * kNbBSlotBytes + row * 128u;
        if (P.w4) decode_half_row<true>(src, dst, row, half, tab);
        else decode_half_row<false>(src, dst, row, half, tab);
        // generic-proxy writes become visible to tcgen05.mma (async proxy): each thread's
        // proxy fence, the warp's barrier, then one mbarrier arrival (release) per warp
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(b_full + 8 * bs);
          mbar_arrive(n_empty + 8 * ns);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(2 * kNbAccCols));
  }
}

}  // namespace

cudaError_t tcgn_prepare() {
  return cudaFuncSetAttribute(gemm_tcgn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNbSmem);
}

cudaError_t tcgn_gemm(const TcgPlan &plan, uint32_t *err, cudaStream_t s, int32_t *out0) {
  if (!plan.ntiles) return cudaSuccess;
  gemm_tcgn_kernel<<<plan.grid, kNbThreads, kNbSmem, s>>>(
      plan.d_probs, reinterpret_cast<const CUtensorMap *>(plan.d_maps), plan.d_tiles, plan.ntiles, plan.nprob, err,
      out0);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs
