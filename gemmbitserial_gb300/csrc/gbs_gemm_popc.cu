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
// Kernels:
//  * gemm_popc_tiled<BM, BN>: one BM x BN output tile per 256-thread CTA (64x64,
//    32x128 or 16x256, chosen by the lhs row count), 4 x 4 outputs per
//    thread, planes staged through shared memory by cp.async in K chunks
//    (double buffered).  Thread (tx, ty) owns lhs rows tx + (BM/4)i and rhs
//    rows ty + (BN/4)j, so consecutive lanes store consecutive results of the
//    transposed output row.
//  * gemm_popc_rows: for at most 16 lhs rows, every lhs row x 64-256 rhs rows
//    per CTA, 1, 2 or 4 threads per rhs row (popcounts on at most 1-4 lhs rows
//    per thread past M).
//  * gemm_popc_grouped: persistent; CTAs pull tiles of many independent
//    problems from a device queue (atomic counter) and run the same tile code
//    (the three BM x BN classes, the rows tile, or the skinny class).
//  * gemm_popc_skinny: one warp per output element, lanes stride over the K
//    words; for matrix-vector and other small-output shapes.
#include "gbs_internal.h"

namespace gbs {
namespace {

constexpr int NT = 256;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool pred) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = pred ? 16 : 0;  // src-size 0 zero-fills the destination
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
// 8-byte piece: rows of an odd word count start only 8-byte aligned
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem, bool pred) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = pred ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <bool XOR>
__device__ __forceinline__ uint32_t pc2(ulonglong2 a, ulonglong2 b) {
  if (XOR) return __popcll(a.x ^ b.x) + __popcll(a.y ^ b.y);
  return __popcll(a.x & b.x) + __popcll(a.y & b.y);
}

// Everything one output tile needs.
struct TileArgs {
  const uint64_t *A, *B;
  int32_t *C;
  const int32_t *ra, *rb;
  uint64_t M, N, wpr, a_plane, b_plane, a_rows, b_rows;
  int wa, wb, neg_i, neg_j, shift;
  uint32_t c0;
};

// One BM x BN output tile over the full K range.  smem must hold
// 2 * (wa*BM + wb*BN) * (KC+2) words.  Ends with a __syncthreads(), so the
// caller may reuse smem right away.
template <int BM, int BN, int KC, bool XOR>
__device__ __forceinline__ void popc_tile(const TileArgs &g, uint64_t m0, uint64_t n0, uint64_t *smem) {
  constexpr int LDW = KC + 2;  // padded row stride (words): conflict-free 16-byte reads
  constexpr int TX = BM / 4, TY = BN / 4;
  static_assert(TX * TY == NT, "4x4 outputs per thread");
  const int wa = g.wa, wb = g.wb;
  const int stage_words = (wa * BM + wb * BN) * LDW;
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  const uint64_t wpr = g.wpr;
  const int nchunks = (int)((wpr + KC - 1) / KC);

  auto load_stage = [&](int st, uint64_t k0) {
    uint64_t *s = smem + st * stage_words;
    if (wpr & 1) {  // the reference's 64-bit column padding can leave an odd word count: 8-byte pieces
      const int a_pieces = wa * BM * KC, all = a_pieces + wb * BN * KC;
      for (int idx = tid; idx < all; idx += NT) {
        const bool isA = idx < a_pieces;
        const int li = isA ? idx : idx - a_pieces;
        const int rows = isA ? BM : BN;
        const int plane = li / (rows * KC), rem = li % (rows * KC);
        const int row = rem / KC, p = rem % KC;
        const uint64_t k = k0 + p;
        const uint64_t grow = (isA ? m0 : n0) + row;
        const uint64_t *base = isA ? g.A + plane * g.a_plane : g.B + plane * g.b_plane;
        uint64_t *dst = s + (isA ? plane * BM : wa * BM + plane * BN) * LDW + row * LDW + p;
        const bool ok = k < wpr && grow < (isA ? g.a_rows : g.b_rows);
        cp_async8(dst, ok ? base + grow * wpr + k : base, ok);
      }
      return;
    }
    constexpr int per_row = KC / 2;  // 16-byte pieces per row
    const int a_pieces = wa * BM * per_row, all = a_pieces + wb * BN * per_row;
    for (int idx = tid; idx < all; idx += NT) {
      const bool isA = idx < a_pieces;
      const int li = isA ? idx : idx - a_pieces;
      const int rows = isA ? BM : BN;
      const int plane = li / (rows * per_row), rem = li % (rows * per_row);
      const int row = rem / per_row, p = rem % per_row;
      const uint64_t k = k0 + 2 * p;
      const uint64_t grow = (isA ? m0 : n0) + row;
      const uint64_t *base = isA ? g.A + plane * g.a_plane : g.B + plane * g.b_plane;
      uint64_t *dst = s + (isA ? plane * BM : wa * BM + plane * BN) * LDW + row * LDW + 2 * p;
      const bool ok = k < wpr && grow < (isA ? g.a_rows : g.b_rows);
      cp_async16(dst, ok ? base + grow * wpr + k : base, ok);
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
          for (int m = 0; m < 4; m++) a[m] = *reinterpret_cast<const ulonglong2 *>(pa + m * TX * LDW + 2 * kp);
#pragma unroll
          for (int n = 0; n < 4; n++) b[n] = *reinterpret_cast<const ulonglong2 *>(pb + n * TY * LDW + 2 * kp);
#pragma unroll
          for (int m = 0; m < 4; m++)
#pragma unroll
            for (int n = 0; n < 4; n++) t[m][n] += pc2<XOR>(a[m], b[n]);
        }
        const uint32_t al = alpha_of(i, j, g.neg_i, g.neg_j, g.shift, XOR);
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
    const uint64_t gn = n0 + ty + TY * n;
    if (gn >= g.N) continue;
    const uint32_t bn = g.c0 - (g.rb ? (uint32_t)g.rb[gn] : 0u);
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const uint64_t gm = m0 + tx + TX * m;
      if (gm >= g.M) continue;
      const uint32_t v = acc[m][n] + bn - (g.ra ? (uint32_t)g.ra[gm] : 0u);
      g.C[gn * g.M + gm] = (int32_t)v;
    }
  }
}

// The rows tile: every lhs row of a problem with at most 16 of them x
// rows_tile_n(M) rhs rows.  TPR threads share one rhs row, each taking MT of
// the lhs rows (MT * TPR >= M, MT of 1 to 4), so popcounts are spent on at
// most that many lhs rows instead of a 16- or 32-row tile's
// padding (for M = 1 the BM x BN classes do 16x the work), and no thread
// counts more than 4 lhs rows per word (past that a tile's popcounts, not its
// loads, set its time).  The pipeline steps over (rhs plane j, K chunk) pairs:
// a stage holds one K chunk of rhs plane j for the tile's rhs rows and of
// every lhs plane for the 16 staged lhs rows, so its shared memory does not
// grow with wb.  The lhs words are read as broadcasts, an rhs word by its TPR
// threads at once.  Ends with a __syncthreads().
constexpr int kRowsStagedRows = kRowsMaxM;
__host__ __device__ constexpr size_t rows_stage_words(int wa, int kc) {
  return (size_t)(wa * kRowsStagedRows + NT) * (kc + 2);
}

template <int MT, int TPR, int KC, bool XOR>
__device__ __forceinline__ void popc_rows_tile(const TileArgs &g, uint64_t n0, uint64_t *smem) {
  constexpr int LDW = KC + 2;
  constexpr int BNR = NT / TPR;  // rhs rows of the tile
  const int wa = g.wa, wb = g.wb, tid = threadIdx.x;
  const int r = tid / TPR, q = tid % TPR;  // the thread's rhs row and lhs rows q*MT .. q*MT + MT-1
  const int stage_words = (int)rows_stage_words(wa, KC);
  const uint64_t wpr = g.wpr;
  const int nchunks = (int)((wpr + KC - 1) / KC);
  const int nsteps = nchunks * wb;

  auto load_stage = [&](int st, int step) {
    const int j = step / nchunks;
    const uint64_t k0 = (uint64_t)(step % nchunks) * KC;
    uint64_t *s = smem + st * stage_words;
    const int a_rows = wa * kRowsStagedRows;
    const int piece = (wpr & 1) ? 1 : 2;  // odd word counts (64-bit column padding): 8-byte pieces
    const int per_row = KC / piece, all = (a_rows + BNR) * per_row;
    for (int idx = tid; idx < all; idx += NT) {
      const int row = idx / per_row, p = idx % per_row;
      const bool isA = row < a_rows;
      const uint64_t k = k0 + (uint64_t)(p * piece);
      const uint64_t *base;
      uint64_t grow;
      bool ok;
      if (isA) {
        const int plane = row / kRowsStagedRows, rr = row % kRowsStagedRows;
        base = g.A + plane * g.a_plane;
        grow = (uint64_t)rr;
        ok = k < wpr && grow < g.a_rows;
      } else {
        base = g.B + j * g.b_plane;
        grow = n0 + (uint64_t)(row - a_rows);
        ok = k < wpr && grow < g.b_rows;
      }
      uint64_t *dst = s + row * LDW + p * piece;
      if (piece == 2) cp_async16(dst, ok ? base + grow * wpr + k : base, ok);
      else cp_async8(dst, ok ? base + grow * wpr + k : base, ok);
    }
  };

  uint32_t acc[MT];
#pragma unroll
  for (int m = 0; m < MT; m++) acc[m] = 0u;

  if (nsteps > 0) {
    load_stage(0, 0);
    cp_commit();
  }
  for (int st = 0; st < nsteps; st++) {
    if (st + 1 < nsteps) {
      load_stage((st + 1) & 1, st + 1);
      cp_commit();
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const int j = st / nchunks;
    const uint64_t *sa = smem + (st & 1) * stage_words;
    const uint64_t *pb = sa + (wa * kRowsStagedRows + r) * LDW;
#pragma unroll 1
    for (int i = 0; i < wa; i++) {
      const uint64_t *pa = sa + (i * kRowsStagedRows + q * MT) * LDW;
      const uint32_t al = alpha_of(i, j, g.neg_i, g.neg_j, g.shift, XOR);  // weights fold in per count (mod 2^32)
      constexpr int kUnroll = 8 / MT;  // about 8 independent counts per unrolled step
#pragma unroll kUnroll
      for (int kp = 0; kp < KC / 2; kp++) {
        const ulonglong2 b = *reinterpret_cast<const ulonglong2 *>(pb + 2 * kp);
#pragma unroll
        for (int m = 0; m < MT; m++)
          acc[m] += pc2<XOR>(*reinterpret_cast<const ulonglong2 *>(pa + m * LDW + 2 * kp), b) * al;
      }
    }
    __syncthreads();
  }

  const uint64_t gn = n0 + (uint64_t)r;
  if (gn < g.N) {
    const uint32_t bn = g.c0 - (g.rb ? (uint32_t)g.rb[gn] : 0u);
#pragma unroll
    for (int mm = 0; mm < MT; mm++) {
      const int m = q * MT + mm;
      if (m < (int)g.M) g.C[gn * g.M + m] = (int32_t)(acc[mm] + bn - (g.ra ? (uint32_t)g.ra[m] : 0u));
    }
  }
}

// lhs rows per thread x threads per rhs row: the smallest product >= M (3-row
// buckets for M = 3, 5-6, 9-12), with the threads per row rows_tile_n's
template <int KC, bool XOR>
__device__ __forceinline__ void popc_rows_dispatch(const TileArgs &g, uint64_t n0, uint64_t *smem) {
  if (g.M <= 1) popc_rows_tile<1, 1, KC, XOR>(g, n0, smem);
  else if (g.M <= 2) popc_rows_tile<2, 1, KC, XOR>(g, n0, smem);
  else if (g.M <= 3) popc_rows_tile<3, 1, KC, XOR>(g, n0, smem);
  else if (g.M <= 4) popc_rows_tile<4, 1, KC, XOR>(g, n0, smem);
  else if (g.M <= 6) popc_rows_tile<3, 2, KC, XOR>(g, n0, smem);
  else if (g.M <= 8) popc_rows_tile<4, 2, KC, XOR>(g, n0, smem);
  else if (g.M <= 12) popc_rows_tile<3, 4, KC, XOR>(g, n0, smem);
  else popc_rows_tile<4, 4, KC, XOR>(g, n0, smem);
}

template <bool XOR>
__global__ void __launch_bounds__(NT, 2) gemm_popc_rows(TileArgs g) {
  extern __shared__ __align__(16) uint64_t smem[];
  popc_rows_dispatch<kRowsKC, XOR>(g, (uint64_t)blockIdx.x * rows_tile_n(g.M), smem);
}

template <int BM, int BN, int KC, bool XOR>
__global__ void __launch_bounds__(NT, 2) gemm_popc_tiled(TileArgs g) {
  extern __shared__ __align__(16) uint64_t smem[];
  popc_tile<BM, BN, KC, XOR>(g, (uint64_t)blockIdx.x * BM, (uint64_t)blockIdx.y * BN, smem);
}

// One output's weighted popcounts over every plane pair, this lane's share:
// words lane, lane + 32, ... of lhs row a0 and rhs row b0 (planes a_plane /
// b_plane words apart).  Each step loads U x 32 words of every plane first --
// independent loads, one memory latency per step rather than one per plane
// pair and 32 words -- then counts.  WM >= max(wa, wb) sizes the register
// arrays.  Words past wpr count as zero (AND and XOR alike).
template <int WM, int U, typename Alpha>
__device__ __forceinline__ uint32_t skinny_lane_sum_t(const uint64_t *__restrict__ a0, uint64_t a_plane,
                                                      const uint64_t *__restrict__ b0, uint64_t b_plane, uint64_t wpr,
                                                      int wa, int wb, bool use_xor, int lane, Alpha alpha) {
  uint32_t acc = 0;
  for (uint64_t w0 = 0; w0 < wpr; w0 += 32 * U) {
    uint64_t av[WM][U], bv[WM][U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint64_t w = w0 + (uint64_t)(32 * u + lane);
      const bool in = w < wpr;
#pragma unroll
      for (int i = 0; i < WM; i++) av[i][u] = (in && i < wa) ? __ldg(a0 + i * a_plane + w) : 0ull;
#pragma unroll
      for (int j = 0; j < WM; j++) bv[j][u] = (in && j < wb) ? __ldg(b0 + j * b_plane + w) : 0ull;
    }
#pragma unroll
    for (int i = 0; i < WM; i++) {
      if (i >= wa) break;
#pragma unroll
      for (int j = 0; j < WM; j++) {
        if (j >= wb) break;
        uint32_t c = 0;
#pragma unroll
        for (int u = 0; u < U; u++) c += (uint32_t)(use_xor ? __popcll(av[i][u] ^ bv[j][u]) : __popcll(av[i][u] & bv[j][u]));
        acc += c * alpha(i, j);
      }
    }
  }
  return acc;
}

template <typename Alpha>
__device__ __forceinline__ uint32_t skinny_lane_sum(const uint64_t *__restrict__ a0, uint64_t a_plane,
                                                    const uint64_t *__restrict__ b0, uint64_t b_plane, uint64_t wpr,
                                                    int wa, int wb, bool use_xor, int lane, Alpha alpha) {
  const int wm = wa > wb ? wa : wb;
  if (wm <= 1) return skinny_lane_sum_t<1, 4>(a0, a_plane, b0, b_plane, wpr, wa, wb, use_xor, lane, alpha);
  if (wm <= 2) return skinny_lane_sum_t<2, 4>(a0, a_plane, b0, b_plane, wpr, wa, wb, use_xor, lane, alpha);
  if (wm <= 4) return skinny_lane_sum_t<4, 2>(a0, a_plane, b0, b_plane, wpr, wa, wb, use_xor, lane, alpha);
  return skinny_lane_sum_t<kMaxBits, 1>(a0, a_plane, b0, b_plane, wpr, wa, wb, use_xor, lane, alpha);
}

// One output (m, n) of a grouped problem by one warp, lanes over the K words
// (the skinny tile class: matrix-vector and other small-output problems).
__device__ __forceinline__ void grouped_skinny_output(const GroupProblem &P, uint64_t o, int lane) {
  const uint64_t n = o / P.M, m = o % P.M;
  uint32_t acc = skinny_lane_sum(P.A + m * P.wpr, P.a_plane, P.B + n * P.wpr, P.b_plane, P.wpr, P.wa, P.wb,
                                 P.use_xor != 0, lane,
                                 [&](int i, int j) { return alpha_of(i, j, P.neg_i, P.neg_j, P.shift, P.use_xor); });
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if (lane == 0) {
    const uint32_t v = acc + P.c0 - (P.ra ? (uint32_t)P.ra[m] : 0u) - (P.rb ? (uint32_t)P.rb[n] : 0u);
    P.C[n * P.M + m] = (int32_t)v;
  }
}

// Persistent grouped GEMM: each CTA takes the next tile from the queue until
// the queue is drained.  Tile classes 0-2 are BM x BN output tiles; class 3
// is kSkinnyTile outputs, one per warp.  A descriptor that fails validation
// sets a bit in *err and is skipped (no device fault, no wait).
__global__ void __launch_bounds__(NT, 2) gemm_popc_grouped(const GroupProblem *__restrict__ probs, int nprob,
                                                           const GroupTile *__restrict__ tiles, uint32_t ntiles,
                                                           uint32_t *counter, uint32_t *err) {
  extern __shared__ __align__(16) uint64_t smem[];
  __shared__ uint32_t s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t t = s_tile;
    __syncthreads();
    if (t >= ntiles) break;
    const GroupTile tl = tiles[t];
    if (tl.p >= (uint32_t)nprob || tl.cls > kRowsCls) {
      if (threadIdx.x == 0) atomicOr(err, 1u);
      continue;
    }
    const GroupProblem &P = probs[tl.p];
    if (tl.cls == kSkinnyCls) {
      const uint64_t o0 = (uint64_t)tl.mt * kSkinnyTile;
      if (o0 >= P.M * P.N || P.wa < 1 || P.wa > kMaxBits || P.wb < 1 || P.wb > kMaxBits) {
        if (threadIdx.x == 0) atomicOr(err, 2u);
        continue;
      }
      const uint64_t o = o0 + (threadIdx.x >> 5);
      if (o < P.M * P.N) grouped_skinny_output(P, o, threadIdx.x & 31);
      continue;
    }
    const bool rows = tl.cls == kRowsCls;
    const int bm = rows ? kRowsMaxM : tile_bm((int)tl.cls), bn = rows ? rows_tile_n(P.M) : tile_bn((int)tl.cls);
    const uint64_t m0 = (uint64_t)tl.mt * bm, n0 = (uint64_t)tl.nt * bn;
    if (m0 >= P.M || n0 >= P.N || P.wa < 1 || P.wa > kMaxBits || P.wb < 1 || P.wb > kMaxBits ||
        (rows && P.M > (uint64_t)kRowsMaxM)) {
      if (threadIdx.x == 0) atomicOr(err, 2u);
      continue;
    }
    TileArgs g;
    g.A = P.A; g.B = P.B; g.C = P.C; g.ra = P.ra; g.rb = P.rb;
    g.M = P.M; g.N = P.N; g.wpr = P.wpr; g.a_plane = P.a_plane; g.b_plane = P.b_plane;
    g.a_rows = P.a_rows; g.b_rows = P.b_rows;
    g.wa = P.wa; g.wb = P.wb; g.neg_i = P.neg_i; g.neg_j = P.neg_j; g.shift = P.shift; g.c0 = P.c0;
    if (rows) {
      if (P.use_xor) popc_rows_dispatch<kRowsKC, true>(g, n0, smem);
      else popc_rows_dispatch<kRowsKC, false>(g, n0, smem);
    } else if (P.use_xor) {
      if (tl.cls == 0) popc_tile<64, 64, kGroupKC, true>(g, m0, n0, smem);
      else if (tl.cls == 1) popc_tile<32, 128, kGroupKC, true>(g, m0, n0, smem);
      else popc_tile<16, 256, kGroupKC, true>(g, m0, n0, smem);
    } else {
      if (tl.cls == 0) popc_tile<64, 64, kGroupKC, false>(g, m0, n0, smem);
      else if (tl.cls == 1) popc_tile<32, 128, kGroupKC, false>(g, m0, n0, smem);
      else popc_tile<16, 256, kGroupKC, false>(g, m0, n0, smem);
    }
  }
}

// One warp per output (m, n); lanes stride over the K words.
__global__ void __launch_bounds__(256) gemm_popc_skinny(GemmShape g, Epilogue e) {
  const uint64_t o = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (o >= g.M * g.N) return;  // warp-uniform
  const uint64_t n = o / g.M, m = o % g.M;
  uint32_t acc = skinny_lane_sum(g.A + m * g.wpr, g.a_plane, g.B + n * g.wpr, g.b_plane, g.wpr, g.wa, g.wb,
                                 e.use_xor != 0, lane, [&](int i, int j) { return (uint32_t)e.alpha[i][j]; });
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if (lane == 0) {
    uint32_t v = acc + e.c0 - (e.ra ? (uint32_t)e.ra[m] : 0u) - (e.rb ? (uint32_t)e.rb[n] : 0u);
    g.C[n * g.M + m] = (int32_t)v;
  }
}

template <int BM, int BN, int KC, bool XOR>
cudaError_t run_tiled(const TileArgs &t, cudaStream_t s) {
  const size_t smem = 2ull * (t.wa * BM + t.wb * BN) * (KC + 2) * sizeof(uint64_t);
  auto kern = gemm_popc_tiled<BM, BN, KC, XOR>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  dim3 grid((unsigned)((t.M + BM - 1) / BM), (unsigned)((t.N + BN - 1) / BN));
  kern<<<grid, NT, smem, s>>>(t);
  count_launch();
  return cudaGetLastError();
}

template <int BM, int BN, bool XOR>
cudaError_t run_tiled_kc(const TileArgs &t, cudaStream_t s) {
  const int rows = t.wa * BM + t.wb * BN;
  if (rows <= 384) return run_tiled<BM, BN, 16, XOR>(t, s);  // <= 110 KB: 2 CTAs/SM
  if (rows <= 768) return run_tiled<BM, BN, 8, XOR>(t, s);   // <= 123 KB
  return run_tiled<BM, BN, 4, XOR>(t, s);                    // <= 2304 rows: <= 221 KB
}

template <bool XOR>
cudaError_t run_tiled_cls(int cls, const TileArgs &t, cudaStream_t s) {
  if (cls == 2) return run_tiled_kc<16, 256, XOR>(t, s);
  if (cls == 1) return run_tiled_kc<32, 128, XOR>(t, s);
  return run_tiled_kc<64, 64, XOR>(t, s);
}

template <bool XOR>
cudaError_t run_rows(const TileArgs &t, cudaStream_t s) {
  const size_t smem = popc_rows_smem(t.wa, kRowsKC);
  auto kern = gemm_popc_rows<XOR>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  const uint64_t bnr = rows_tile_n(t.M);
  kern<<<(unsigned)((t.N + bnr - 1) / bnr), NT, smem, s>>>(t);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

size_t popc_rows_smem(int wa, int kc) { return 2 * rows_stage_words(wa, kc) * sizeof(uint64_t); }

size_t popc_stage_smem(int cls, int wa, int wb, int kc) {
  return 2ull * (wa * tile_bm(cls) + wb * tile_bn(cls)) * (kc + 2) * sizeof(uint64_t);
}

// Tile class for a problem: the narrowest lhs tile that covers M without
// exceeding the shared-memory cap at the grouped chunk size.
bool popc_skinny(uint64_t M, uint64_t N) { return M * N <= 32768 || N < 16 || M < 4; }

int popc_tile_class(uint64_t M, int wa, int wb, size_t smem_cap) {
  int cls = M <= 16 ? 2 : (M <= 32 ? 1 : 0);
  while (cls > 0 && popc_stage_smem(cls, wa, wb, kGroupKC) > smem_cap) cls--;
  return cls;
}

cudaError_t launch_gemm_popc(const GemmShape &g, const Epilogue &e, cudaStream_t s) {
  if (g.M == 0 || g.N == 0) return cudaSuccess;
  const bool skinny = g.tile_cls < 0 && popc_skinny(g.M, g.N);
  if (skinny) {
    const uint64_t threads = g.M * g.N * 32;
    gemm_popc_skinny<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(g, e);
    count_launch();
    return cudaGetLastError();
  }
  TileArgs t;
  t.A = g.A; t.B = g.B; t.C = g.C; t.ra = e.ra; t.rb = e.rb;
  t.M = g.M; t.N = g.N; t.wpr = g.wpr; t.a_plane = g.a_plane; t.b_plane = g.b_plane;
  t.a_rows = g.a_rows; t.b_rows = g.b_rows;
  t.wa = g.wa; t.wb = g.wb; t.neg_i = e.neg_i; t.neg_j = e.neg_j; t.shift = e.shift; t.c0 = e.c0;
  // at most 16 lhs rows: the rows tile (no popcounts on padding rows), unless a class is forced
  if (g.tile_cls == kRowsCls || (g.tile_cls < 0 && g.M <= (uint64_t)kRowsMaxM))
    return e.use_xor ? run_rows<true>(t, s) : run_rows<false>(t, s);
  const int cls = (g.tile_cls >= 0 && g.tile_cls <= 2) ? g.tile_cls : popc_tile_class(g.M, g.wa, g.wb, 220 * 1024);
  if (e.use_xor) return run_tiled_cls<true>(cls, t, s);
  return run_tiled_cls<false>(cls, t, s);
}

cudaError_t prepare_gemm_popc_grouped(size_t smem) {
  return cudaFuncSetAttribute(gemm_popc_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int grouped_blocks_per_sm(size_t smem) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gemm_popc_grouped, NT, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_gemm_popc_grouped(const GroupProblem *probs, int nprob, const GroupTile *tiles, uint32_t ntiles,
                                     uint32_t *counter, uint32_t *err, size_t smem, int grid, cudaStream_t s) {
  gemm_popc_grouped<<<grid, NT, smem, s>>>(probs, nprob, tiles, ntiles, counter, err);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs
