// gbs_gemm_tcg.cu -- persistent tensor-core GEMM over a table of problems,
// and the planes -> e4m3 digit expansion that feeds it.
//
// The reference evaluates a list of GEMMs as a host loop of gemmBitSerial
// calls (benchmark.cpp:192-206); each call is AND + popcount over every plane
// pair weighted by +-2^(i+j) (arch-generic.hpp:179-192), with the bipolar
// corrections of arch-generic.hpp:45-71.  Here every operand of a problem is
// first expanded to an e4m3 "digit" matrix whose byte is the element's whole
// few-bit value (bipolar: +-1; columns past K and rows past nrows: 0), so one
// fp8 tcgen05.mma over digits covers all plane pairs and all corrections at
// once.  Products and partial sums are integers, exact in the fp32 TMEM
// accumulator while K * max|a| * max|b| < 2^24 (the eligibility rule), so
// the int32 result is bit-exact.
//
// Kernel: one CTA per SM walks its share of a cost-sorted tile table (snake
// order, no atomics).  A tile is 128 rows of the MMA-A operand x bn rows of
// the MMA-B operand; per problem the larger side is MMA-A ("swap" when that
// is the rhs), so a problem with few lhs rows uses an MMA N as small as 16
// instead of padding M to 128.
//   warp 0     lane 0: TMA producer -- A box 128 x 128 bytes and B box
//              bn x 128 bytes per stage, 128-byte swizzle, into a 4-slot ring
//              that runs across tile boundaries
//   warp 1     allocates all 512 TMEM columns (two 256-column accumulators);
//              lane 0 issues 4 tcgen05.mma (K = 32) per stage and commits the
//              accumulator of each tile
//   warps 2-5  epilogue of tile j while the MMAs of tile j+1 run: tcgen05.ld
//              32 lanes x 16 columns, fp32 -> int32, stores into res[n*M + m]
// Every mbarrier wait is bounded; on timeout the CTA sets a bit in the
// caller's error word, stops issuing, drains what it issued and frees TMEM.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gbs_internal.h"
#include "gbs_tc_common.cuh"

namespace gbs {
namespace {

constexpr int kTgStages = 4;
constexpr uint32_t kTgABytes = 128 * 128;           // MMA-A box: 128 rows x 128 digits
constexpr uint32_t kTgSlotBytes = kTgABytes + 256 * 128;  // + MMA-B box of up to 256 rows
constexpr int kTgThreads = 192;
constexpr uint32_t kTgAccCols = 256;

constexpr size_t tcg_smem_bytes() { return 1024 + kTgStages * kTgSlotBytes + 8 * (2 * kTgStages + 5) + 16; }

// Tile j of CTA b among G CTAs: rounds of G consecutive table entries, every
// other round walked backwards, so each CTA's share of a cost-sorted table
// sums to nearly the same cost.
__device__ __forceinline__ uint32_t snake_tile(uint32_t j, uint32_t b, uint32_t G) {
  return j * G + ((j & 1u) ? G - 1u - b : b);
}

__device__ __forceinline__ bool tile_ok(const TcgTile &t, const TcgProblem &P, uint32_t nprob) {
  return t.p < nprob && P.bn >= 16 && P.bn <= 256 && (P.bn & 15u) == 0 && P.nk > 0 &&
         (t.r + 1) * 128u <= P.a_rows && (t.c + 1) * P.bn <= P.b_rows;
}

__global__ void __launch_bounds__(kTgThreads, 1)
    gemm_tcg_kernel(const TcgProblem *__restrict__ probs, const CUtensorMap *__restrict__ maps,
                    const TcgTile *__restrict__ tiles, uint32_t ntiles, uint32_t nprob, uint32_t *err,
                    int32_t *out0) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTgStages * kTgSlotBytes);
  const uint32_t full = smem_u32(bars), empty = full + 8 * kTgStages, acc_full = empty + 8 * kTgStages;
  const uint32_t acc_empty = acc_full + 16, mma_done = acc_empty + 16;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kTgStages + 5);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint32_t G = gridDim.x, b = blockIdx.x;

  if (tid == 0) {
    for (int i = 0; i < kTgStages; i++) {
      mbar_init(full + 8 * i, 1);
      mbar_init(empty + 8 * i, 1);
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
                 "n"(2 * kTgAccCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t it = 0;  // stage loads issued
      bool stop = false;
      for (uint32_t j = 0; !stop; j++) {
        const uint32_t t = snake_tile(j, b, G);
        if (t >= ntiles) break;
        const TcgTile tl = tiles[t];
        if (tl.p >= nprob) continue;
        const TcgProblem P = probs[tl.p];
        if (!tile_ok(tl, P, nprob)) continue;
        const CUtensorMap *ma = maps + 2 * tl.p, *mb = ma + 1;
        // the maps were written by a host copy: order them for the tensor-map proxy
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(ma) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(mb) : "memory");
        const uint32_t bytes = kTgABytes + P.bn * 128u;
        for (uint32_t k = 0; k < P.nk; k++, it++) {
          const uint32_t s = it % kTgStages, use = it / kTgStages;
          if (use > 0 && !mbar_wait_err(empty + 8 * s, (use - 1) & 1, abort_flag, err)) {
            stop = true;
            break;
          }
          mbar_expect_tx(full + 8 * s, bytes);
          const uint32_t dst = smem_u32(smem + s * kTgSlotBytes);
          tma_load_digits(dst, ma, (int)k, tl.r * 128, full + 8 * s);
          tma_load_digits(dst + kTgABytes, mb, (int)k, tl.c * P.bn, full + 8 * s);
        }
      }
      if (*abort_flag)
        for (uint32_t q = (it > (uint32_t)kTgStages ? it - kTgStages : 0); q < it; q++)
          mbar_drain_err(full + 8 * (q % kTgStages), (q / kTgStages) & 1, err);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t it = 0, jt = 0;  // stages consumed, tiles accumulated
      bool ok = true;
      for (uint32_t j = 0; ok; j++) {
        const uint32_t t = snake_tile(j, b, G);
        if (t >= ntiles) break;
        const TcgTile tl = tiles[t];
        if (tl.p >= nprob) continue;
        const TcgProblem P = probs[tl.p];
        if (!tile_ok(tl, P, nprob)) continue;
        const uint32_t a = jt & 1, use = jt >> 1;
        if (use > 0 && !mbar_wait_err(acc_empty + 8 * a, (use - 1) & 1, abort_flag, err)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t d = tmem + a * kTgAccCols;
        for (uint32_t k = 0; k < P.nk; k++, it++) {
          const uint32_t s = it % kTgStages;
          if (!mbar_wait_err(full + 8 * s, (it / kTgStages) & 1, abort_flag, err)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t base = smem_u32(smem + s * kTgSlotBytes);
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            mma_f8(d, sw128_desc(base + kk * 32), sw128_desc(base + kTgABytes + kk * 32), P.idesc, (k | kk) != 0);
          mma_commit(empty + 8 * s);
        }
        if (!ok) break;
        mma_commit(acc_full + 8 * a);
        jt++;
      }
      if (!ok) {  // issued MMAs finish before TMEM is freed
        mma_commit(mma_done);
        mbar_drain_err(mma_done, 0, err);
      }
    }
  } else {
    const int q = warp & 3;  // TMEM lanes 32q .. 32q+31 belong to this warp
    uint32_t jt = 0;
    for (uint32_t j = 0;; j++) {
      const uint32_t t = snake_tile(j, b, G);
      if (t >= ntiles) break;
      const TcgTile tl = tiles[t];
      TcgProblem P;
      if (tl.p < nprob) P = probs[tl.p];
      if (tl.p >= nprob || !tile_ok(tl, P, nprob)) {
        if (warp == 2 && lane == 0) atomicOr(err, 4u);
        continue;
      }
      if (out0 && tl.p == 0) P.C = out0;  // the caller's result buffer for problem 0
      const uint32_t a = jt & 1, use = jt >> 1;
      if (!__all_sync(0xffffffffu, mbar_wait_err(acc_full + 8 * a, use & 1, abort_flag, err))) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t row = tl.r * 128u + (uint32_t)(q * 32 + lane);
      const uint32_t taddr = tmem + a * kTgAccCols + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (uint32_t col = 0; col < P.bn; col += 16) {
        uint32_t v[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr + col));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        int32_t o[16];
#pragma unroll
        for (int i = 0; i < 16; i++) o[i] = __float2int_rn(__uint_as_float(v[i]));
        const uint32_t c0 = tl.c * P.bn + col;
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
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty + 8 * a);
      jt++;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(2 * kTgAccCols));
  }
}

// ------------------------------------------------------------ digit expansion
// One thread writes 16 digits (one 16-byte store) of one row; chunks entirely
// past K are skipped, as are rows past nrows: the buffer is zeroed when it is
// allocated and those bytes never change.
template <int CNT>
__device__ __forceinline__ void expand_chunk(const ExpandJob &j, uint32_t r, uint32_t col0) {
  const uint64_t w = col0 >> 6;
  const int sh = (int)(col0 & 63);
  uint32_t pw[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int p = 0; p < CNT; p++) pw[p] = (uint32_t)(j.planes[(p * j.nrows_a + r) * j.wpr + w] >> (sh & 32));
  const uint32_t tab[4] = {j.tab[0], j.tab[1], j.tab[2], j.tab[3]};
  uint32_t q[4];
#pragma unroll
  for (int n = 0; n < 4; n++) {
    const int s4 = (sh & 16) + 4 * n;
    if (CNT == 1) {
      const uint32_t sp = decode4<1>(pw, s4, tab);
      q[n] = sp * ((tab[0] >> 8) & 0xFFu) + (sp ^ 0x01010101u) * (tab[0] & 0xFFu);
    } else {
      q[n] = decode4<CNT>(pw, s4, tab);
    }
    const uint32_t c0 = col0 + 4 * n;
    if (c0 + 4 > j.K) q[n] &= c0 >= j.K ? 0u : (0xFFFFFFFFu >> (8 * (4 - (j.K - c0))));
  }
  *reinterpret_cast<uint4 *>(j.digits + digit_offset(r, col0, j.dcols)) = make_uint4(q[0], q[1], q[2], q[3]);
}

// One thread writes 32 codes (one 16-byte store) of one row of a nibble
// matrix: the codes of 4 columns as bytes (plane p's nibble spread to bit p
// of each byte), then two bytes' codes into one (even column low).
template <int CNT>
__device__ __forceinline__ void expand_nibble_chunk(const ExpandJob &j, uint32_t r, uint32_t col0) {
  const uint64_t w = col0 >> 6;
  const int sh = (int)(col0 & 63);
  uint32_t pw[CNT];
#pragma unroll
  for (int p = 0; p < CNT; p++) pw[p] = (uint32_t)(j.planes[(p * j.nrows_a + r) * j.wpr + w] >> sh);
  uint32_t o[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {  // columns 8i .. 8i + 7
    uint32_t t[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      uint32_t c = 0;
#pragma unroll
      for (int p = 0; p < CNT; p++) c |= (bfe4(pw[p], 8 * i + 4 * h) * (0x00204081u << p)) & (0x01010101u << p);
      t[h] = c | (c >> 4);  // bytes 0 and 2: code pairs (even column low)
    }
    o[i] = __byte_perm(t[0], t[1], 0x6420u);
  }
  *reinterpret_cast<uint4 *>(j.digits + nibble_offset(r, col0, j.dcols)) = make_uint4(o[0], o[1], o[2], o[3]);
}

__device__ __forceinline__ void expand_thread(const ExpandJob &j, uint64_t local) {
  if (local >= (uint64_t)j.nrows * j.chunks) return;  // padding threads of the job
  uint32_t r, col0;
  if (local < 0xFFFFFFFFull) {  // 32-bit division in the common case
    r = (uint32_t)local / j.chunks;
    col0 = ((uint32_t)local - r * j.chunks) * 16u;
  } else {
    r = (uint32_t)(local / j.chunks);
    col0 = (uint32_t)(local % j.chunks) * 16u;
  }
  if (j.nib) {
    col0 *= 2;  // 32 codes per thread
    switch (j.nbits) {
      case 1: expand_nibble_chunk<1>(j, r, col0); break;
      case 2: expand_nibble_chunk<2>(j, r, col0); break;
      case 3: expand_nibble_chunk<3>(j, r, col0); break;
      default: expand_nibble_chunk<4>(j, r, col0); break;
    }
    return;
  }
  switch (j.nbits) {
    case 1: expand_chunk<1>(j, r, col0); break;
    case 2: expand_chunk<2>(j, r, col0); break;
    case 3: expand_chunk<3>(j, r, col0); break;
    default: expand_chunk<4>(j, r, col0); break;
  }
}

__global__ void __launch_bounds__(256) expand_one_kernel(const ExpandJob job) {
  expand_thread(job, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// Every job's thread range is a multiple of 256, so all threads of a block
// belong to one job and the job search below is uniform within the block.

__global__ void __launch_bounds__(256) expand_grouped_kernel(const ExpandJob *__restrict__ jobs, int njobs,
                                                             uint64_t total) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = njobs - 1;  // last job with thread0 <= i
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].thread0 <= i) lo = mid;
      else hi = mid - 1;
    }
    const ExpandJob &j = jobs[lo];
    expand_thread(j, i - j.thread0);
  }
}

template <typename T>
cudaError_t upload(T **dst, const T *src, size_t n) {
  cudaError_t e = dev_alloc((void **)dst, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace

ExpandJob make_expand_job(const Mat &m, uint8_t *digits) {
  ExpandJob j;
  memset(&j, 0, sizeof(j));
  j.planes = m.planes;
  j.digits = digits;
  j.nrows_a = m.nrows_a;
  j.wpr = m.wpr();
  j.dcols = m.dcols;
  j.nrows = (uint32_t)m.nrows;
  j.K = (uint32_t)m.ncols;
  j.chunks = (uint32_t)((m.ncols + 15) / 16);
  j.nbits = (uint32_t)m.nbits;
  tc_digit_table(m, j.tab);
  return j;
}

ExpandJob make_nibble_job(const Mat &m, uint8_t *nibbles) {
  ExpandJob j = make_expand_job(m, nibbles);
  j.nib = 1;
  j.chunks = (uint32_t)((m.ncols + 31) / 32);
  return j;
}

cudaError_t launch_expand(const ExpandJob &job, cudaStream_t s) {
  const uint64_t threads = (uint64_t)job.nrows * job.chunks;
  if (threads == 0) return cudaSuccess;
  expand_one_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(job);
  count_launch();
  return cudaGetLastError();
}

// Digit matrix [drows][dcols] of one side, allocated zeroed on first use
// (synchronously: kernels on any stream may write it right after).
cudaError_t ensure_digit_buffer(gbs_ctx *c, int side) {
  if (c->digits[side]) return cudaSuccess;
  const Mat &m = side ? c->rhs : c->lhs;
  const size_t bytes = std::max<size_t>(m.drows * m.dcols, 16);
  cudaError_t e = dev_alloc((void **)&c->digits[side], bytes);
  if (e == cudaSuccess) e = cudaMemset(c->digits[side], 0, bytes);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  c->digit_maps_ready = false;
  c->digit_map_b64_ready = false;
  c->plan1_ready = false;
  c->digits_valid[side] = false;
  return e;
}

// Nibble matrix [drows][dcols / 2] of one side, allocated zeroed on first use.
cudaError_t ensure_nibble_buffer(gbs_ctx *c, int side) {
  if (c->nibbles[side]) return cudaSuccess;
  const Mat &m = side ? c->rhs : c->lhs;
  const size_t bytes = std::max<size_t>(m.drows * m.dcols / 2, 16);
  cudaError_t e = dev_alloc((void **)&c->nibbles[side], bytes);
  if (e == cudaSuccess) e = cudaMemset(c->nibbles[side], 0, bytes);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  c->plan1_ready = false;
  c->nibbles_valid[side] = false;
  return e;
}

// The digit kernel is exact when every partial sum stays below 2^24 in fp32
// and each operand's values fit e4m3 exactly (at most 4 bits).
bool tcg_eligible(const gbs_ctx *c) { return tc_exact(c, GBS_PIPE_TC); }

// Digits cost about one HBM byte per element of the larger operand; the
// CUDA-core popcount kernel costs 2 * min(M, N) * wA * wB bit operations per
// such element at ~1/45 of the HBM byte rate.  Below ~10 the latter is cheaper.
bool tcg_preferred(const gbs_ctx *c) {
  const uint64_t mn = std::min(c->lhs.nrows, c->rhs.nrows);
  return mn * c->lhs.nbits * c->rhs.nbits >= 10;
}

void tcg_plan_free(TcgPlan *p) {
  if (p->d_probs) cudaFree(p->d_probs);
  if (p->d_maps) cudaFree(p->d_maps);
  if (p->d_tiles) cudaFree(p->d_tiles);
  if (p->d_jobs) cudaFree(p->d_jobs);
  *p = TcgPlan();
}

namespace {

// GBS_TCG_NIBBLES in the environment when a plan is built: 0 keeps it on the
// digit kernel, 1 puts it on the nibble kernel; unset, the estimate below
// chooses.  Returns 0, 1 or -1 (choose).
int nibbles_mode() {
  const char *v = getenv("GBS_TCG_NIBBLES");
  if (v && v[0] == '0') return 0;
  if (v && v[0] == '1') return 1;
  return -1;
}

// Which persistent kernel serves a plan faster, by an estimate of its
// critical path.  The nibble kernel reads half a byte per element of each
// problem's larger side where the digit kernel reads one, but it cuts that
// side into 256-row tiles (half as many as the digit kernel's 128-row tiles),
// and its stages move more shared memory (nibbles in, decoded digits out, a
// 128-row MMA operand however few rows the smaller side has).  Per 128-digit
// K stage a digit tile costs the longer of its bytes at ~100 GB/s into one SM
// and its four MMAs (M = 128: ~37 ns up to N = 128, ~68 ns at N = 256), a
// nibble tile ~0.7 us; the plan costs the longest of its tiles spread over
// the SMs they can occupy, its largest tile, and its HBM bytes (larger side
// once, smaller side once, results) at ~5 TB/s.  These constants are fitted
// to GB300 timings of both kernels on groups of 1 to 397 problems, where the
// estimate picks the faster kernel every time: groups of about 64 problems or
// more are HBM-bound and take the nibbles; fewer leave SMs idle and take the
// digit kernel's finer, cheaper tiles.
bool plan_prefers_nibbles(gbs_ctx *const *ctxs, int n) {
  const double sms = (double)std::max(1, sm_count());
  double tiles[2] = {0, 0}, work[2] = {0, 0}, longest[2] = {0, 0}, hbm[2] = {0, 0};
  auto mma_ns = [](double bn) { return bn <= 128 ? 37.0 : 37.0 + (bn - 128) * (31.0 / 128); };
  for (int i = 0; i < n; i++) {
    const Mat &L = ctxs[i]->lhs, &R = ctxs[i]->rhs;
    const double small = (double)std::min(L.nrows, R.nrows), large = (double)std::max(L.nrows, R.nrows);
    const double nk = (double)((L.ncols + 127) / 128), K = nk * 128;
    if (small == 0 || nk == 0) continue;
    for (int k = 0; k < 2; k++) {
      const double bn = k ? 256 : std::min(256.0, std::ceil(small / 16) * 16);
      const double nt = k ? std::ceil(small / 128) * std::ceil(large / 256)
                          : std::ceil(large / 128) * std::ceil(small / bn);
      const double t = nk * (k ? 700.0 : std::max((128 * 128 + bn * 128) / 100.0, 4 * mma_ns(bn)));  // ns
      tiles[k] += nt;
      work[k] += nt * t;
      longest[k] = std::max(longest[k], t);
      hbm[k] += (k ? large * K / 2 : large * K) + small * K + 4 * small * large;
    }
  }
  double est[2];
  for (int k = 0; k < 2; k++)
    est[k] = std::max({tiles[k] > 0 ? work[k] / std::min(tiles[k], sms) : 0.0, longest[k], hbm[k] / 5000.0});
  return est[1] < est[0];
}

}  // namespace

int tcg_plan_build(TcgPlan *plan, gbs_ctx *const *ctxs, int n) {
  tcg_plan_free(plan);
  const int mode = nibbles_mode();
  const bool nib = mode < 0 ? plan_prefers_nibbles(ctxs, n) : mode == 1;
  plan->nibbles = nib;
  std::vector<TcgProblem> probs;
  std::vector<CUtensorMap> maps;
  std::vector<TcgTile> tiles;
  std::vector<uint64_t> cost;
  std::vector<ExpandJob> jobs;
  uint64_t threads = 0;
  for (int i = 0; i < n; i++) {
    gbs_ctx *c = ctxs[i];
    const Mat &L = c->lhs, &R = c->rhs;
    TcgProblem P;
    memset(&P, 0, sizeof(P));
    P.C = c->res;
    P.M = (uint32_t)L.nrows;
    P.N = (uint32_t)R.nrows;
    // digit kernel: the larger side is MMA-A; nibble kernel: the smaller side
    P.swap = nib ? (R.nrows < L.nrows ? 1u : 0u) : (L.nrows < R.nrows ? 1u : 0u);
    const int sa = P.swap ? 1 : 0, sb = 1 - sa;  // sides of MMA-A and MMA-B
    const uint8_t sides = nib ? (uint8_t)((1u << sa) | (4u << sb)) : (uint8_t)3;
    for (int side = 0; side < 2; side++) {
      cudaError_t e = cudaSuccess;
      if ((sides >> side) & 1) e = ensure_digit_buffer(c, side);
      if (e == cudaSuccess && ((sides >> (2 + side)) & 1)) e = ensure_nibble_buffer(c, side);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GBS_ENOMEM, "tensor-core plan: digit or nibble matrix allocation failed");
      }
    }
    plan->ctxs.push_back(c);
    plan->sides.push_back(sides);
    const Mat &MA = sa ? R : L, &MB = sb ? R : L;
    P.a_rows = (uint32_t)MA.drows;
    P.b_rows = (uint32_t)MB.drows;
    P.nk = (uint32_t)((L.ncols + 127) / 128);
    CUtensorMap m2[2];
    uint32_t rt, ct;
    if (!nib) {
      P.bn = (uint32_t)std::min<uint64_t>(256, (MB.nrows + 15) / 16 * 16);
      P.idesc = (1u << 4) | ((P.bn >> 3) << 17) | ((128u >> 4) << 24);
      if (!tc_map_u8(&m2[0], c->digits[sa], MA.dcols, MA.drows, 128) ||
          !tc_map_u8(&m2[1], c->digits[sb], MB.dcols, MB.drows, P.bn))
        return fail(GBS_EUNSUPPORTED, "tensor-core plan: tensor map encoding failed");
      rt = (uint32_t)((MA.nrows + 127) / 128);
      ct = (uint32_t)((MB.nrows + P.bn - 1) / P.bn);
    } else {
      P.bn = 256;
      P.idesc = (1u << 4) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
      P.w4 = MB.nbits > 3 ? 1u : 0u;
      tc_digit_table(MB, P.tab);
      // a smaller side of at most 128 rows loads only its rows (16-row blocks) into the
      // 128-row MMA-A slot: the slot's other rows feed accumulator lanes no store reads
      const uint32_t a_box = MA.nrows <= 128 ? (uint32_t)std::max<uint64_t>(16, (MA.nrows + 15) / 16 * 16) : 128u;
      P.a_bytes = a_box * 128u;
      if (!tc_map_u8(&m2[0], c->digits[sa], MA.dcols, MA.drows, a_box) ||
          !tc_map_nibbles(&m2[1], c->nibbles[sb], MB.dcols, MB.drows))
        return fail(GBS_EUNSUPPORTED, "tensor-core plan: tensor map encoding failed");
      rt = (uint32_t)((MA.nrows + 127) / 128);
      ct = (uint32_t)((MB.nrows + 255) / 256);
    }
    maps.push_back(m2[0]);
    maps.push_back(m2[1]);
    for (uint32_t r = 0; r < rt; r++)
      for (uint32_t cc = 0; cc < ct; cc++) {
        tiles.push_back(TcgTile{(uint32_t)probs.size(), r, cc, 0u});
        cost.push_back((uint64_t)P.nk * (128 + P.bn));
      }
    probs.push_back(P);
    for (int side = 0; side < 2; side++) {
      const Mat &m = side ? R : L;
      for (int kind = 0; kind < 2; kind++) {  // digits, nibbles
        if (!((sides >> (2 * kind + side)) & 1)) continue;
        ExpandJob j = kind ? make_nibble_job(m, c->nibbles[side]) : make_expand_job(m, c->digits[side]);
        j.thread0 = threads;
        threads += ((uint64_t)j.nrows * j.chunks + 255) / 256 * 256;
        if (j.nrows && j.chunks) jobs.push_back(j);
      }
    }
  }
  std::vector<size_t> order(tiles.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  std::vector<TcgTile> sorted(tiles.size());
  for (size_t i = 0; i < order.size(); i++) sorted[i] = tiles[order[i]];

  cudaError_t e = upload(&plan->d_probs, probs.data(), probs.size());
  if (e == cudaSuccess) e = upload((CUtensorMap **)&plan->d_maps, maps.data(), maps.size());
  if (e == cudaSuccess) e = upload(&plan->d_tiles, sorted.data(), sorted.size());
  if (e == cudaSuccess) e = upload(&plan->d_jobs, jobs.data(), jobs.size());
  if (e == cudaSuccess)
    e = nib ? tcgn_prepare()
            : cudaFuncSetAttribute(gemm_tcg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tcg_smem_bytes());
  if (e != cudaSuccess) {
    cudaGetLastError();
    tcg_plan_free(plan);
    return fail(GBS_ENOMEM, "tensor-core plan: table upload failed");
  }
  plan->nibbles = nib;
  plan->nprob = (uint32_t)probs.size();
  plan->ntiles = (uint32_t)sorted.size();
  plan->njobs = (int)jobs.size();
  plan->expand_threads = threads;
  plan->grid = (int)std::min<uint64_t>(plan->ntiles, (uint64_t)sm_count());
  return GBS_OK;
}

cudaError_t tcg_expand(TcgPlan &plan, cudaStream_t s) {
  if (plan.njobs && plan.expand_threads) {
    const uint64_t blocks = std::min<uint64_t>((plan.expand_threads + 255) / 256, (uint64_t)sm_count() * 16);
    expand_grouped_kernel<<<(unsigned)blocks, 256, 0, s>>>(plan.d_jobs, plan.njobs, plan.expand_threads);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  for (size_t i = 0; i < plan.ctxs.size(); i++)
    for (int side = 0; side < 2; side++) {
      if ((plan.sides[i] >> side) & 1) plan.ctxs[i]->digits_valid[side] = true;
      if ((plan.sides[i] >> (2 + side)) & 1) plan.ctxs[i]->nibbles_valid[side] = true;
    }
  return cudaSuccess;
}

cudaError_t tcg_gemm(const TcgPlan &plan, uint32_t *err, cudaStream_t s, int32_t *out0) {
  if (!plan.ntiles) return cudaSuccess;
  if (plan.nibbles) return tcgn_gemm(plan, err, s, out0);
  gemm_tcg_kernel<<<plan.grid, kTgThreads, tcg_smem_bytes(), s>>>(
      plan.d_probs, reinterpret_cast<const CUtensorMap *>(plan.d_maps), plan.d_tiles, plan.ntiles, plan.nprob, err,
      out0);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs
