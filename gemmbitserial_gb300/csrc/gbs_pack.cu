// gbs_pack.cu -- packing of regular integer matrices into bit planes, and the
// plane-reading helpers (row sums, export).
//
// Semantics follow BitSerialMatrix::importRegular<T> (gemmbitserial.hpp:213-245),
// its quantize step (:170-186) and the uint8_t overload (:249-275): element
// (r, c) of plane b is bit b of the element's code, where the code is
//   * the raw byte for uint8 input (no quantisation),
//   * 1 if x > 0 else 0 for bipolar matrices (1-bit signed),
//   * the low byte of x otherwise (two's complement for signed matrices; the
//     reference's "add 2^(w-1) twice" leaves the low w bits of x unchanged).
// Rows >= nrows and columns >= ncols are zero in every plane.
#include "gbs_internal.h"

namespace gbs {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int64_t load_elem(const void *src, int dtype, uint64_t idx) {
  switch (dtype) {
    case GBS_I8: return ((const int8_t *)src)[idx];
    case GBS_U8: return ((const uint8_t *)src)[idx];
    case GBS_I16: return ((const int16_t *)src)[idx];
    default: return ((const int32_t *)src)[idx];
  }
}

__device__ __forceinline__ uint32_t code_of(int64_t x, int dtype, int bipolar) {
  if (dtype == GBS_U8) return (uint32_t)(x & 0xff);
  if (bipolar) return x > 0 ? 1u : 0u;
  return (uint32_t)(x & 0xff);
}

// quantize<float> (gemmbitserial.hpp:170-186): bipolar maps x > 0 to 1; a
// negative x of a signed matrix becomes 2^(w-1) + (uint8_t)(x + 2^(w-1)), the
// sum taken in float; otherwise (uint8_t)x.  Float -> integer casts truncate
// toward zero, then keep the low byte.
__device__ __forceinline__ uint32_t code_of_f32(float x, int bipolar, int issigned, int nbits) {
  if (bipolar) return x > 0.f ? 1u : 0u;
  if (issigned && x < 0.f) {
    const int64_t h = (int64_t)1 << (nbits - 1);
    return (uint32_t)(h + (int64_t)(x + (float)h)) & 0xffu;
  }
  return (uint32_t)(int64_t)x & 0xffu;
}

__device__ __forceinline__ uint32_t elem_code(const void *src, int dtype, uint64_t idx, int bipolar, int issigned,
                                              int nbits) {
  if (dtype == GBS_F32) return code_of_f32(((const float *)src)[idx], bipolar, issigned, nbits);
  return code_of(load_elem(src, dtype, idx), dtype, bipolar);
}

// Row-major packing: a warp takes a 1024-column segment of one padded row;
// lane l owns the 32 columns [seg*1024 + 32l, +32).  Its 32 codes (byte j%4
// of q[j/4]) give, per plane, one whole 32-bit half of a plane word, so the
// 32 lanes store 128 contiguous bytes per plane with no shuffles.
constexpr int kSegCols = 1024;

__host__ __device__ inline uint64_t segs_per_row(uint64_t wpr) { return (wpr * 64 + kSegCols - 1) / kSegCols; }

__device__ __forceinline__ void load_codes32(const void *__restrict__ src, int dtype, int bipolar, int issigned,
                                             int nbits, uint64_t nrows, uint64_t ncols, int vec, uint64_t r,
                                             uint64_t col0, uint32_t (&q)[8]) {
#pragma unroll
  for (int i = 0; i < 8; i++) q[i] = 0u;
  if (r >= nrows || col0 >= ncols) return;
  const uint64_t base = r * ncols + col0;
  if (vec) {  // 1-byte elements, 16-byte aligned rows, ncols % 16 == 0
    const uint4 *p = reinterpret_cast<const uint4 *>((const uint8_t *)src + base);
    const uint4 v0 = p[0];
    q[0] = v0.x; q[1] = v0.y; q[2] = v0.z; q[3] = v0.w;
    if (col0 + 32 <= ncols) {
      const uint4 v1 = p[1];
      q[4] = v1.x; q[5] = v1.y; q[6] = v1.z; q[7] = v1.w;
    }
    if (bipolar && dtype == GBS_I8) {
#pragma unroll
      for (int i = 0; i < 8; i++) q[i] = __vcmpgts4(q[i], 0u) & 0x01010101u;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; j++)
      if (col0 + j < ncols) q[j >> 2] |= elem_code(src, dtype, base + j, bipolar, issigned, nbits) << (8 * (j & 3));
  }
}

// Bits b of the eight bytes of (hi:lo), gathered into a byte (byte i -> bit i):
// masking leaves one bit per byte at 8i; the multiply by sum_i 2^(56-7i)
// moves it to 56+i.  All partial products land on distinct bit positions
// (8i - 7j is unique for i, j in 0..7), so nothing carries.
__device__ __forceinline__ uint32_t gather8(uint32_t lo, uint32_t hi, int b) {
  const uint64_t x = ((((uint64_t)hi << 32) | lo) >> b) & 0x0101010101010101ull;
  return (uint32_t)((x * 0x0102040810204080ull) >> 56);
}

__device__ __forceinline__ void emit_planes32(int nbits, uint64_t nrows_a, uint64_t wpr, uint64_t *__restrict__ planes,
                                              uint64_t r, uint64_t col0, const uint32_t (&q)[8]) {
  uint32_t *p32 = reinterpret_cast<uint32_t *>(planes);  // little-endian halves of the u64 plane words
  const uint64_t row32 = 2 * wpr, idx = r * row32 + (col0 >> 5), plane32 = nrows_a * row32;
  for (int b = 0; b < nbits; b++) {
    const uint32_t w = gather8(q[0], q[1], b) | (gather8(q[2], q[3], b) << 8) | (gather8(q[4], q[5], b) << 16) |
                       (gather8(q[6], q[7], b) << 24);
    p32[b * plane32 + idx] = w;
  }
}

// e4m3 digits of 4 codes (one per byte): the code's low nbits bits index the
// 16-entry byte table tab (byte-permute lookup; PRMT reads only 3 index bits,
// so 4-bit codes take the high half of the table when bit 3 is set).
__device__ __forceinline__ uint32_t digits4(uint32_t x, int nbits, uint4 tab) {
  const uint32_t xm = x & (0x01010101u * ((1u << nbits) - 1u));
  const uint32_t t = xm | (xm >> 4);                  // byte 0 = c0 | c1 << 4, byte 2 = c2 | c3 << 4
  const uint32_t sel = __byte_perm(t, 0u, 0x0020u);   // nibbles c0 c1 c2 c3
  if (nbits <= 3) return __byte_perm(tab.x, tab.y, sel);
  const uint32_t lo = __byte_perm(tab.x, tab.y, sel & 0x7777u);
  const uint32_t hi = __byte_perm(tab.z, tab.w, sel & 0x7777u);
  const uint32_t m = ((xm >> 3) & 0x01010101u) * 0xFFu;
  return (lo & ~m) | (hi & m);
}

// The lane's 32 digits of row r < nrows (0 past ncols) into the digit matrix
// (dcols columns, 16-row blocks: digit_offset).  Digit rows past nrows and
// columns past the planes' padded width stay as allocated: zero.
__device__ __forceinline__ void write_digits32(uint8_t *__restrict__ digits, int nbits, uint64_t nrows,
                                               uint64_t ncols, uint64_t dcols, uint4 tab, uint64_t r, uint64_t col0,
                                               const uint32_t (&q)[8]) {
  uint32_t d[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    d[i] = 0u;
    if (r < nrows) {
      d[i] = digits4(q[i], nbits, tab);
      const uint64_t c = col0 + 4 * i;
      if (c + 4 > ncols) d[i] &= c >= ncols ? 0u : (0xFFFFFFFFu >> (8 * (4 - (ncols - c))));
    }
  }
  uint4 *dst = reinterpret_cast<uint4 *>(digits + digit_offset(r, col0, dcols));
  dst[0] = make_uint4(d[0], d[1], d[2], d[3]);
  dst[1] = make_uint4(d[4], d[5], d[6], d[7]);
}

// The lane's 32 codes of row r < nrows into the nibble matrix (dcols columns,
// blocks of nibble_offset): the low nbits bits of each code byte, two codes a
// byte (even column low).  Codes past ncols are whatever the source gave:
// the tensor-core kernel multiplies them by digits that are zero there.
__device__ __forceinline__ void write_nibbles32(uint8_t *__restrict__ nib, int nbits, uint64_t dcols, uint64_t r,
                                                uint64_t col0, const uint32_t (&q)[8]) {
  const uint32_t msk = 0x01010101u * ((1u << nbits) - 1u);
  uint32_t o[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    uint32_t t0 = q[2 * i] & msk, t1 = q[2 * i + 1] & msk;
    t0 |= t0 >> 4;  // bytes 0 and 2: code pairs
    t1 |= t1 >> 4;
    o[i] = __byte_perm(t0, t1, 0x6420u);
  }
  *reinterpret_cast<uint4 *>(nib + nibble_offset(r, col0, dcols)) = make_uint4(o[0], o[1], o[2], o[3]);
}

// One 1024-column unit: codes, planes and (optionally) digits of the lane's 32 columns.
__device__ __forceinline__ void pack_unit(const void *__restrict__ src, int dtype, int bipolar, int issigned,
                                          int nbits,
                                          uint64_t nrows, uint64_t ncols, uint64_t nrows_a, uint64_t wpr, int vec,
                                          uint64_t *__restrict__ planes, uint8_t *__restrict__ digits,
                                          uint64_t dcols, uint4 dtab, uint64_t r, uint64_t seg, int lane) {
  const uint64_t col0 = seg * kSegCols + (uint64_t)lane * 32;
  if (col0 >= wpr * 64) return;  // past the padded row
  uint32_t q[8];
  load_codes32(src, dtype, bipolar, issigned, nbits, nrows, ncols, vec, r, col0, q);
  emit_planes32(nbits, nrows_a, wpr, planes, r, col0, q);
  if (digits && r < nrows) write_digits32(digits, nbits, nrows, ncols, dcols, dtab, r, col0, q);
}

// Row-major pack of padded rows [row0, row0 + nrows_launch).  With digits
// set, the lanes also write the rows' e4m3 digits (the tensor-core pipe's
// operand), from the same loads.
__global__ void __launch_bounds__(256) pack_rowmajor(const void *__restrict__ src, int dtype, int bipolar,
                                                     int issigned, int nbits, uint64_t nrows, uint64_t ncols,
                                                     uint64_t nrows_a, uint64_t wpr, int vec,
                                                     uint64_t *__restrict__ planes, uint64_t row0,
                                                     uint64_t nrows_launch, uint8_t *__restrict__ digits,
                                                     uint64_t dcols, uint4 dtab) {
  const uint64_t segs = segs_per_row(wpr);
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= nrows_launch * segs) return;  // warp-uniform
  pack_unit(src, dtype, bipolar, issigned, nbits, nrows, ncols, nrows_a, wpr, vec, planes, digits, dcols, dtab,
            row0 + warp / segs,
            warp % segs, threadIdx.x & 31);
}

// ---------------------------------------------------------------- threshold quantisation
// importRegularAndQuantize<T> (gemmbitserial.hpp:282-305): element x of row r
// becomes the index of the first threshold thr[t * nrows + r] with x <= thr
// (compared in T), or nthres when x exceeds them all; with no thresholds the
// element keeps its own value.  The low byte of that code is the code the
// planes store (the (uint8_t) cast of :298).  For float input without
// thresholds the float is truncated toward zero to an integer first.
template <typename T>
__device__ __forceinline__ uint32_t own_code(T x) {
  return (uint32_t)(int64_t)x & 0xFFu;
}

template <typename T>
__device__ __forceinline__ uint32_t threshold_code(T x, const T *__restrict__ thr, int nthres, uint64_t r,
                                                   uint64_t nrows) {
  if (nthres == 0) return own_code(x);
  int t = 0;
  for (; t < nthres; t++)
    if (x <= thr[(uint64_t)t * nrows + r]) break;
  return (uint32_t)t & 0xFFu;
}

// Row-major: a warp per 1024-column segment of a padded row, lane = 32
// columns.  Column-major (matrix[c * nrows + r]): a warp per 32 x 32 block,
// lane = row, so the lanes' loads of one column are contiguous.  Either way a
// lane ends up with 32 consecutive columns of one row and stores them like
// the regular import (planes, and digits when requested).
template <typename T>
__global__ void __launch_bounds__(256) pack_quantize_kernel(const T *__restrict__ src, const T *__restrict__ thr,
                                                            int nthres, int nbits, uint64_t nrows, uint64_t ncols,
                                                            uint64_t nrows_a, uint64_t wpr, int col_major,
                                                            uint64_t *__restrict__ planes,
                                                            uint8_t *__restrict__ digits, uint64_t dcols, uint4 dtab) {
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  uint64_t r, col0;
  if (!col_major) {
    const uint64_t segs = segs_per_row(wpr);
    if (warp >= nrows_a * segs) return;
    r = warp / segs;
    col0 = (warp % segs) * kSegCols + (uint64_t)lane * 32;
  } else {
    const uint64_t cblocks = wpr * 2;
    if (warp >= ((nrows_a + 31) / 32) * cblocks) return;
    r = (warp / cblocks) * 32 + lane;
    col0 = (warp % cblocks) * 32;
    if (r >= nrows_a) return;  // lanes past the padded rows (no warp-wide step follows)
  }
  if (col0 >= wpr * 64) return;
  uint32_t q[8];
#pragma unroll
  for (int i = 0; i < 8; i++) q[i] = 0u;
  if (r < nrows) {
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const uint64_t c = col0 + j;
      if (c < ncols) {
        const T x = src[col_major ? c * nrows + r : r * ncols + c];
        q[j >> 2] |= threshold_code(x, thr, nthres, r, nrows) << (8 * (j & 3));
      }
    }
  }
  emit_planes32(nbits, nrows_a, wpr, planes, r, col0, q);
  if (digits && r < nrows) write_digits32(digits, nbits, nrows, ncols, dcols, dtab, r, col0, q);
}

// Index of the job owning global warp w: the last job with warp0 <= w.
__device__ __forceinline__ int find_job(const PackJob *jobs, int njobs, uint64_t w) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].warp0 <= w) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Grouped import: one launch packs every operand of a grouped GEMM
// (row-major sources); units (1024-column segments of a row) are numbered
// across the jobs.  A warp takes kRun consecutive units: one job lookup,
// then the units in order.
constexpr int kRun = 8;

__global__ void __launch_bounds__(256) pack_grouped(const PackJob *__restrict__ jobs, int njobs, uint64_t total) {
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (uint64_t base = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kRun; base < total;
       base += nw * kRun) {
    int j = find_job(jobs, njobs, base);
    // unit w -> (job, row, segment), advancing the job index monotonically
    auto locate = [&](uint64_t w, int &jj, uint64_t &r, uint64_t &sg) {
      while (jj + 1 < njobs && jobs[jj + 1].warp0 <= w) jj++;
      const PackJob &J = jobs[jj];
      const uint64_t local = w - J.warp0;
      if (local < 0xFFFFFFFFull) {  // 32-bit division in the common case
        const uint32_t l32 = (uint32_t)local, r32 = l32 / J.segs;
        r = r32;
        sg = l32 - r32 * J.segs;
      } else {
        r = local / J.segs;
        sg = local % J.segs;
      }
    };
    auto load = [&](int jj, uint64_t r, uint64_t sg, uint32_t (&q)[8]) {
      const PackJob &J = jobs[jj];
      const uint64_t col0 = sg * kSegCols + (uint64_t)lane * 32;
      if (col0 < J.wpr * 64)
        load_codes32(J.src, J.dtype, J.nbits == 1 && J.issigned, J.issigned, J.nbits, J.nrows, J.ncols, J.vec, r,
                     col0, q);
    };
    // the next unit's loads are in flight while the current unit is packed
    const uint64_t last = min(base + (uint64_t)kRun, total);
    int jc = j;
    uint64_t rc, sc;
    locate(base, jc, rc, sc);
    uint32_t q[8];
    load(jc, rc, sc, q);
#pragma unroll 1
    for (uint64_t w = base; w < last; w++) {
      int jn = jc;
      uint64_t rn = 0, sn = 0;
      uint32_t qn[8];
      if (w + 1 < last) {
        locate(w + 1, jn, rn, sn);
        load(jn, rn, sn, qn);
      }
      const PackJob &J = jobs[jc];
      const uint64_t col0 = sc * kSegCols + (uint64_t)lane * 32;
      if (col0 < J.wpr * 64) {
        emit_planes32(J.nbits, J.nrows_a, J.wpr, J.planes, rc, col0, q);
        if (J.digits && rc < J.nrows) {
          const uint4 tab = make_uint4(J.dtab[0], J.dtab[1], J.dtab[2], J.dtab[3]);
          write_digits32(J.digits, J.nbits, J.nrows, J.ncols, J.dcols, tab, rc, col0, q);
        }
        if (J.nibbles && rc < J.nrows) write_nibbles32(J.nibbles, J.nbits, J.dcols, rc, col0, q);
      }
      if (w + 1 < last) {
        jc = jn;
        rc = rn;
        sc = sn;
#pragma unroll
        for (int i = 0; i < 8; i++) q[i] = qn[i];
      }
    }
  }
}

// Column-major pack (the reference's readColMajor: element (r, c) at c*nrows + r).
// One warp covers 32 padded rows x 64 columns (one word per row and plane):
// lane l reads column c0+l (then c0+32+l) down the 32 rows, and one ballot per
// (row, plane) gathers 32 columns of that row.  Lane j keeps row j's word.
__global__ void __launch_bounds__(256) pack_colmajor(const void *__restrict__ src, int dtype, int bipolar,
                                                     int issigned, int nbits, uint64_t nrows, uint64_t ncols,
                                                     uint64_t nrows_a, uint64_t wpr,
                                                     uint64_t *__restrict__ planes) {
  const uint64_t rgroups = (nrows_a + 31) / 32;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= rgroups * wpr) return;  // warp-uniform
  const uint64_t w = warp / rgroups, r0 = (warp % rgroups) * 32;
  uint32_t lo[kMaxBits], hi[kMaxBits];
#pragma unroll
  for (int b = 0; b < kMaxBits; b++) lo[b] = hi[b] = 0u;
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const uint64_t c = w * 64 + half * 32 + lane;
    uint32_t q[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};  // codes of rows r0..r0+31 of column c
    if (c < ncols) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        uint64_t r = r0 + j;
        if (r < nrows) q[j >> 2] |= elem_code(src, dtype, c * nrows + r, bipolar, issigned, nbits) << (8 * (j & 3));
      }
    }
#pragma unroll
    for (int j = 0; j < 32; j++) {
      uint32_t code = (q[j >> 2] >> (8 * (j & 3))) & 0xffu;
#pragma unroll
      for (int b = 0; b < kMaxBits; b++) {
        if (b < nbits) {
          uint32_t m = __ballot_sync(kFull, (code >> b) & 1u);
          if (lane == j) { if (half) hi[b] = m; else lo[b] = m; }
        }
      }
    }
  }
  const uint64_t plane_words = nrows_a * wpr;
  const uint64_t r = r0 + lane;
  if (r >= nrows_a) return;  // the last group's lanes past the padded rows
#pragma unroll
  for (int b = 0; b < kMaxBits; b++)
    if (b < nbits) planes[b * plane_words + r * wpr + w] = (uint64_t)lo[b] | ((uint64_t)hi[b] << 32);
}

// sumRows (arch-generic.hpp:6-37) of row r by one warp.  uint32 arithmetic
// reproduces the reference's int32 wrap-around.
__device__ __forceinline__ int32_t row_sum(const uint64_t *__restrict__ planes, int nbits, int issigned,
                                           uint64_t ncols, uint64_t nrows_a, uint64_t wpr, uint64_t r, int lane) {
  const bool bip = nbits == 1 && issigned;
  uint32_t acc = 0;
  for (int b = 0; b < nbits; b++) {
    const uint64_t *row = planes + (uint64_t)b * nrows_a * wpr + r * wpr;
    uint32_t cnt = 0;
    for (uint64_t w = lane; w < wpr; w += 32) cnt += __popcll(row[w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
    cnt <<= b;
    if (issigned && !bip && b == nbits - 1) cnt = 0u - cnt;
    acc += cnt;
  }
  if (bip) acc = 2u * acc - (uint32_t)ncols;
  return (int32_t)acc;
}

__global__ void __launch_bounds__(256) rowsum_kernel(const uint64_t *__restrict__ planes, int nbits, int issigned,
                                                     uint64_t nrows, uint64_t ncols, uint64_t nrows_a,
                                                     uint64_t wpr, int32_t *__restrict__ dst) {
  const uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  const int32_t v = row_sum(planes, nbits, issigned, ncols, nrows_a, wpr, r, lane);
  if (lane == 0) dst[r] = v;
}

// Grouped row sums: one warp per row over every job (warp0 counts rows).
__global__ void __launch_bounds__(256) rowsum_grouped(const PackJob *__restrict__ jobs, int njobs, uint64_t total) {
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < total; w += nw) {
    const PackJob &J = jobs[find_job(jobs, njobs, w)];
    const uint64_t r = w - J.warp0;
    const int32_t v = row_sum(J.planes, J.nbits, J.issigned, J.ncols, J.nrows_a, J.wpr, r, lane);
    if (lane == 0) J.rowsum[r] = v;
  }
}

// exportRegular (gemmbitserial.hpp:313-333): one thread per element.
__global__ void __launch_bounds__(256) export_kernel(const uint64_t *__restrict__ planes, int nbits, int issigned,
                                                     uint64_t nrows, uint64_t ncols, uint64_t nrows_a,
                                                     uint64_t wpr, int32_t *__restrict__ dst) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows * ncols) return;
  const uint64_t r = i / ncols, c = i % ncols;
  const bool bip = nbits == 1 && issigned;
  int32_t v = 0;
  for (int b = 0; b < nbits; b++) {
    uint64_t bit = (planes[(uint64_t)b * nrows_a * wpr + r * wpr + (c >> 6)] >> (c & 63)) & 1u;
    if (bip) v = bit ? 1 : -1;
    else if (bit) v += (issigned && b == nbits - 1) ? -(1 << b) : (1 << b);
  }
  dst[i] = v;
}

inline unsigned blocks_for(uint64_t threads, unsigned per_block) {
  return (unsigned)((threads + per_block - 1) / per_block);
}

}  // namespace

cudaError_t launch_pack_rows(const Mat &m, const void *src, int dtype, uint64_t r0, uint64_t r1, uint8_t *digits,
                             const uint32_t *dtab, cudaStream_t s) {
  if (m.nrows_a == 0 || m.wpr() == 0 || r1 <= r0) return cudaSuccess;
  const int bip = m.bipolar() ? 1 : 0;
  const size_t esz = dtype == GBS_I16 ? 2 : (dtype == GBS_I32 || dtype == GBS_F32) ? 4 : 1;
  const int vec = (esz == 1 && m.ncols % 16 == 0 && ((uintptr_t)src % 16) == 0) ? 1 : 0;
  const uint64_t warps = (r1 - r0) * segs_per_row(m.wpr());
  const uint4 tab = dtab ? make_uint4(dtab[0], dtab[1], dtab[2], dtab[3]) : make_uint4(0u, 0u, 0u, 0u);
  pack_rowmajor<<<blocks_for(warps * 32, 256), 256, 0, s>>>(src, dtype, bip, m.issigned, (int)m.nbits, m.nrows, m.ncols,
                                                          m.nrows_a, m.wpr(), vec, m.planes, r0, r1 - r0,
                                                          digits, m.dcols, tab);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pack_quantize(const Mat &m, const void *src, const void *thr, int nthres, int dtype,
                                 int col_major, uint8_t *digits, const uint32_t *dtab, cudaStream_t s) {
  if (m.nrows_a == 0 || m.wpr() == 0) return cudaSuccess;
  const uint64_t warps = col_major ? ((m.nrows_a + 31) / 32) * m.wpr() * 2 : m.nrows_a * segs_per_row(m.wpr());
  const unsigned blocks = blocks_for(warps * 32, 256);
  const uint4 tab = dtab ? make_uint4(dtab[0], dtab[1], dtab[2], dtab[3]) : make_uint4(0u, 0u, 0u, 0u);
#define GBS_QLAUNCH(T)                                                                                              \
  pack_quantize_kernel<T><<<blocks, 256, 0, s>>>((const T *)src, (const T *)thr, nthres, (int)m.nbits, m.nrows,      \
                                                 m.ncols, m.nrows_a, m.wpr(), col_major, m.planes, digits, m.dcols, \
                                                 tab)
  switch (dtype) {
    case GBS_I8: GBS_QLAUNCH(int8_t); break;
    case GBS_U8: GBS_QLAUNCH(uint8_t); break;
    case GBS_I16: GBS_QLAUNCH(int16_t); break;
    case GBS_I32: GBS_QLAUNCH(int32_t); break;
    default: GBS_QLAUNCH(float); break;
  }
#undef GBS_QLAUNCH
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pack(const Mat &m, const void *src, int dtype, int col_major, cudaStream_t s) {
  if (m.nrows_a == 0 || m.wpr() == 0) return cudaSuccess;
  const int bip = m.bipolar() ? 1 : 0;
  if (!col_major) {
    return launch_pack_rows(m, src, dtype, 0, m.nrows_a, nullptr, nullptr, s);
  } else {
    const uint64_t warps = ((m.nrows_a + 31) / 32) * m.wpr();
    pack_colmajor<<<blocks_for(warps * 32, 256), 256, 0, s>>>(src, dtype, bip, m.issigned, (int)m.nbits, m.nrows, m.ncols,
                                                            m.nrows_a, m.wpr(), m.planes);
  }
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pack_grouped(const PackJob *jobs, int njobs, uint64_t total_warps, cudaStream_t s) {
  if (total_warps == 0 || njobs == 0) return cudaSuccess;
  const uint64_t blocks = (total_warps + 8 * kRun - 1) / (8 * kRun);
  pack_grouped<<<(unsigned)(blocks < 152 * 64 ? blocks : 152 * 64), 256, 0, s>>>(jobs, njobs, total_warps);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rowsum_grouped(const PackJob *jobs, int njobs, uint64_t total_warps, cudaStream_t s) {
  if (total_warps == 0 || njobs == 0) return cudaSuccess;
  const uint64_t blocks = (total_warps + 7) / 8;
  rowsum_grouped<<<(unsigned)(blocks < 152 * 64 ? blocks : 152 * 64), 256, 0, s>>>(jobs, njobs, total_warps);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rowsum(const Mat &m, int32_t *dst, cudaStream_t s) {
  if (m.nrows == 0) return cudaSuccess;
  rowsum_kernel<<<blocks_for(m.nrows * 32, 256), 256, 0, s>>>(m.planes, (int)m.nbits, m.issigned, m.nrows,
                                                              m.ncols, m.nrows_a, m.wpr(), dst);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_export(const Mat &m, int32_t *dst, cudaStream_t s) {
  if (m.nrows * m.ncols == 0) return cudaSuccess;
  export_kernel<<<blocks_for(m.nrows * m.ncols, 256), 256, 0, s>>>(m.planes, (int)m.nbits, m.issigned, m.nrows,
                                                                   m.ncols, m.nrows_a, m.wpr(), dst);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs
