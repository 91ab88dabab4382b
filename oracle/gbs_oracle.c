/*
 * gbs_oracle.c -- CPU oracle for the bit-serial GEMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the tests, the smoke
 * entry and the CPU-baseline leg of the benchmark call it to produce the
 * results the GPU path must reproduce bit for bit.  Nothing in the product
 * library links against it or falls back to it.
 *
 * It restates, in plain C, the algorithm of maltanar/gemmbitserial's generic
 * (non-NEON) code path.  Every function names the reference file:line it
 * follows.  The arithmetic is the reference's, including its int32 wrap-around
 * (all sums are formed modulo 2^32 through uint32_t, which is what the
 * reference's int32 accumulators do on two's-complement hardware).
 *
 * Pinned by: the reference's MNIST known-answer vector (test/mnistdata.h:46,
 * used at test/test.cpp:157-172), the reference's naive_int_gemm
 * (test/testhelpers.hpp:34-45), and golden vectors produced by the reference
 * compiled from its own headers (recipe in oracle/Makefile).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>

#define ORC_EXPORT __attribute__((visibility("default")))

/* Input element types accepted by the import routine. */
enum { ORC_I8 = 0, ORC_U8 = 1, ORC_I16 = 2, ORC_I32 = 3, ORC_F32 = 4 };

typedef struct {
  int issigned;
  uint64_t nbits, nrows, ncols, nrows_a, ncols_a;
  uint64_t *data; /* [nbits][nrows_a][ncols_a/64] */
} orc_matrix;

typedef struct {
  orc_matrix lhs, rhs;
  uint64_t lhsBlock, rhsBlock;
  int32_t *res; /* [rhs.nrows][lhs.nrows] : transposed result */
} orc_ctx;

/* gemmbitserial.hpp:11-17 alignTo */
static uint64_t round_up(uint64_t x, uint64_t a) {
  if (a == 0) return x; /* only reachable for empty matrices, where the reference divides by zero */
  uint64_t r = x % a;
  return r ? x + (a - r) : x;
}

static int mat_bipolar(const orc_matrix *m) { return m->nbits == 1 && m->issigned; } /* :74-76 */
static uint64_t mat_wpr(const orc_matrix *m) { return m->ncols_a / 64; }            /* :79-82 */
static uint64_t mat_wpp(const orc_matrix *m) { return m->nrows_a * mat_wpr(m); }    /* :85-87 */
static uint64_t *mat_row(const orc_matrix *m, uint64_t b, uint64_t r) {             /* :117-119 */
  return m->data + b * mat_wpp(m) + r * mat_wpr(m);
}

/* gemmbitserial.hpp:24-35 BitSerialMatrix::alloc */
static orc_matrix mat_alloc(uint64_t nbits, uint64_t nrows, uint64_t ncols, int issigned,
                            uint64_t rowalign, uint64_t colalign) {
  orc_matrix m;
  m.issigned = issigned;
  m.nbits = nbits;
  m.nrows = nrows;
  m.ncols = ncols;
  m.nrows_a = round_up(nrows, rowalign);
  m.ncols_a = round_up(ncols, colalign);
  m.data = (uint64_t *)calloc(nbits * mat_wpp(&m) + 1, sizeof(uint64_t));
  return m;
}

/* gemmbitserial.hpp:343-360 computeBlockSize: positive root of
 * 4*l*r*x^2 + d*(l+r)*x - cacheBits = 0, in single precision like the reference. */
static void block_size(float lm, float rm, float cache_bits, float dbits, uint64_t *lb, uint64_t *rb) {
  float qa = (float)sizeof(int32_t) * lm * rm;
  float qb = dbits * (lm + rm);
  float qc = -cache_bits;
  float disc = sqrtf(qb * qb - 4.0f * qa * qc);
  int64_t r0 = (int64_t)floorf((-qb + disc) / (2.0f * qa));
  int64_t r1 = (int64_t)floorf((-qb - disc) / (2.0f * qa));
  int64_t x = r0 > r1 ? r0 : r1;
  if (x > 0) {
    *lb = (uint64_t)(lm * (float)x);
    *rb = (uint64_t)(rm * (float)x);
  } else {
    *lb = (uint64_t)lm;
    *rb = (uint64_t)rm;
  }
}

/* gemmbitserial.hpp:364-377 finetuneBlockSize: smallest padding waste over
 * candidates bs_max, bs_max-div, ... (> div). */
static uint64_t tune_block(uint64_t rows, uint64_t bs_max, uint64_t div) {
  uint64_t best = bs_max, waste = round_up(rows, bs_max) - rows;
  for (uint64_t c = bs_max; c > div; c -= div) {
    if (c % div) continue;
    uint64_t w = round_up(rows, c) - rows;
    if (w < waste) { best = c; waste = w; }
  }
  return best;
}

/* gemmbitserial.hpp:415-452 allocGEMMContext_base, called with the
 * register blocking chosen in arch-generic.hpp:78-100. */
ORC_EXPORT orc_ctx *orc_ctx_alloc(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB,
                                  int sA, int sB) {
  const uint64_t cache_bits = 32 * 1024 * 8;
  uint64_t rl = 2, rd = 1, rr = 2;
  if (N == 1) { rl = 1; rd = 4; rr = 1; } /* matrix-vector: depth aligned to 256 */
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  uint64_t kal = round_up(K, rd * 64);
  block_size((float)rl, (float)rr, (float)cache_bits, (float)kal, &c->lhsBlock, &c->rhsBlock);
  if (c->lhsBlock > M || c->rhsBlock > N) {
    c->lhsBlock = round_up(M, rl);
    c->rhsBlock = round_up(N, rr);
  } else {
    if ((double)(round_up(M, c->lhsBlock) - M) > 0.1 * (double)M)
      c->lhsBlock = tune_block(M, c->lhsBlock, rl);
    if ((double)(round_up(N, c->rhsBlock) - N) > 0.1 * (double)N)
      c->rhsBlock = tune_block(N, c->rhsBlock, rr);
  }
  c->lhs = mat_alloc(wA, M, K, sA, c->lhsBlock, rd * 64);
  c->rhs = mat_alloc(wB, N, K, sB, c->rhsBlock, rd * 64);
  c->res = (int32_t *)calloc(M * N + 1, sizeof(int32_t));
  return c;
}

/* gemmbitserial.hpp:454-458 */
ORC_EXPORT void orc_ctx_free(orc_ctx *c) {
  if (!c) return;
  free(c->lhs.data);
  free(c->rhs.data);
  free(c->res);
  free(c);
}

/* dims: [lhs.nrows_a, rhs.nrows_a, lhs.ncols_a, rhs.ncols_a, lhsBlock, rhsBlock] */
ORC_EXPORT void orc_ctx_dims(const orc_ctx *c, uint64_t *out) {
  out[0] = c->lhs.nrows_a;
  out[1] = c->rhs.nrows_a;
  out[2] = c->lhs.ncols_a;
  out[3] = c->rhs.ncols_a;
  out[4] = c->lhsBlock;
  out[5] = c->rhsBlock;
}

ORC_EXPORT uint64_t *orc_planes(orc_ctx *c, int side) { return side ? c->rhs.data : c->lhs.data; }
ORC_EXPORT int32_t *orc_res(orc_ctx *c) { return c->res; }

static int64_t load_elem(const void *src, int dtype, uint64_t idx) {
  switch (dtype) {
    case ORC_I8: return ((const int8_t *)src)[idx];
    case ORC_U8: return ((const uint8_t *)src)[idx];
    case ORC_I16: return ((const int16_t *)src)[idx];
    default: return ((const int32_t *)src)[idx];
  }
}

/* gemmbitserial.hpp:170-186 quantize<T>, and :249-275 for the uint8_t overload
 * (raw bits, no quantisation).  For non-bipolar matrices both reduce to the
 * low bits of (uint8_t)x: the signed branch adds 2^(w-1) twice, i.e. 2^w,
 * which leaves the low w bits unchanged.  The bipolar branch maps x>0 to 1. */
/* quantize<float> (gemmbitserial.hpp:170-186) for float input: bipolar maps
 * x > 0 to 1; a negative x of a signed matrix becomes 2^(w-1) + (uint8_t)(x +
 * 2^(w-1)) with the sum taken in float and truncated; otherwise (uint8_t)x.
 * The float -> uint8_t casts are taken as truncation toward zero to an
 * integer, then its low byte (C defines them only for values in [0, 256)). */
static uint8_t to_code_f32(const orc_matrix *m, float x) {
  if (mat_bipolar(m)) return x > 0 ? 1 : 0;
  if (m->issigned && x < 0) {
    const int64_t h = (int64_t)1 << (m->nbits - 1);
    return (uint8_t)(h + (int64_t)(x + (float)h));
  }
  return (uint8_t)(int64_t)x;
}

static uint8_t to_code(const orc_matrix *m, int dtype, int64_t x) {
  if (dtype == ORC_U8) return (uint8_t)x;
  if (mat_bipolar(m)) return x > 0 ? 1 : 0;
  if (m->issigned && x < 0) {
    uint8_t hi = (uint8_t)(1u << (m->nbits - 1));
    return (uint8_t)(hi + (uint8_t)(x + (int64_t)hi));
  }
  return (uint8_t)x;
}

/* gemmbitserial.hpp:213-245 importRegular: clear, then set bit b of the code
 * of element (r,c) into plane b, word c>>6, bit c&63.  readColMajor reads
 * matrix[c*nrows + r]. */
static void mat_import(orc_matrix *m, const void *src, int dtype, int colmajor) {
  memset(m->data, 0, m->nbits * mat_wpp(m) * sizeof(uint64_t));
  for (uint64_t r = 0; r < m->nrows; r++) {
    for (uint64_t col = 0; col < m->ncols; col++) {
      uint64_t idx = colmajor ? col * m->nrows + r : r * m->ncols + col;
      uint8_t q = dtype == ORC_F32 ? to_code_f32(m, ((const float *)src)[idx]) : to_code(m, dtype, load_elem(src, dtype, idx));
      for (uint64_t b = 0; b < m->nbits; b++)
        if ((q >> b) & 1u) mat_row(m, b, r)[col >> 6] |= (uint64_t)1 << (col & 63);
    }
  }
}

ORC_EXPORT void orc_import(orc_ctx *c, int side, const void *src, int dtype, int colmajor) {
  mat_import(side ? &c->rhs : &c->lhs, src, dtype, colmajor);
}

/* gemmbitserial.hpp:282-305 importRegularAndQuantize<T>: element x of row r
 * becomes the index t of the first threshold thresholds[t*nrows + r] with
 * x <= threshold (compared in T), or nThres when x exceeds every threshold;
 * with nThres == 0 the loop never runs and x keeps its own value.  The
 * (uint8_t) cast of :298 then keeps the low byte, of which the low nbits bits
 * are stored.  For float input with nThres == 0 the cast is taken as
 * truncation toward zero to an integer, then the low byte (C leaves float to
 * uint8_t undefined outside [0, 256)). */
static uint8_t quantize_code(const void *src, const void *thr, int nthres, int dtype, uint64_t idx, uint64_t r,
                             uint64_t nrows) {
  if (dtype == ORC_F32) {
    const float x = ((const float *)src)[idx];
    if (nthres == 0) return (uint8_t)(int64_t)x;
    for (int t = 0; t < nthres; t++)
      if (x <= ((const float *)thr)[(uint64_t)t * nrows + r]) return (uint8_t)t;
    return (uint8_t)nthres;
  }
  const int64_t x = load_elem(src, dtype, idx);
  if (nthres == 0) return (uint8_t)x;
  for (int t = 0; t < nthres; t++)
    if (x <= load_elem(thr, dtype, (uint64_t)t * nrows + r)) return (uint8_t)t;
  return (uint8_t)nthres;
}

static void mat_import_quantize(orc_matrix *m, const void *src, const void *thr, int nthres, int dtype,
                                int colmajor) {
  memset(m->data, 0, m->nbits * mat_wpp(m) * sizeof(uint64_t));
  for (uint64_t r = 0; r < m->nrows; r++)
    for (uint64_t col = 0; col < m->ncols; col++) {
      uint64_t idx = colmajor ? col * m->nrows + r : r * m->ncols + col;
      uint8_t q = quantize_code(src, thr, nthres, dtype, idx, r, m->nrows);
      for (uint64_t b = 0; b < m->nbits; b++)
        if ((q >> b) & 1u) mat_row(m, b, r)[col >> 6] |= (uint64_t)1 << (col & 63);
    }
}

/* Returns -1 for a signed matrix: the reference asserts !issigned (:283). */
ORC_EXPORT int orc_import_quantize(orc_ctx *c, int side, const void *src, const void *thr, int nthres, int dtype,
                                   int colmajor) {
  orc_matrix *m = side ? &c->rhs : &c->lhs;
  if (m->issigned) return -1;
  mat_import_quantize(m, src, thr, nthres, dtype, colmajor);
  return 0;
}

/* gemmbitserial.hpp:313-333 exportRegular */
ORC_EXPORT void orc_export(orc_ctx *c, int side, int32_t *dst) {
  orc_matrix *m = side ? &c->rhs : &c->lhs;
  for (uint64_t r = 0; r < m->nrows; r++)
    for (uint64_t col = 0; col < m->ncols; col++) {
      int bitv[8];
      for (uint64_t b = 0; b < m->nbits; b++) bitv[b] = (mat_row(m, b, r)[col >> 6] >> (col & 63)) & 1;
      int32_t v = 0;
      if (mat_bipolar(m)) {
        v = bitv[0] ? 1 : -1;
      } else {
        for (uint64_t b = 0; b < m->nbits; b++)
          if (bitv[b]) v += (m->issigned && b == m->nbits - 1) ? -(1 << b) : (1 << b);
      }
      dst[r * m->ncols + col] = v;
    }
}

/* arch-generic.hpp:6-37 sumRows_generic */
static void mat_rowsums(const orc_matrix *m, int32_t *out) {
  uint64_t nw = mat_wpr(m);
  for (uint64_t r = 0; r < m->nrows; r++) {
    uint32_t acc = 0;
    if (mat_bipolar(m)) {
      const uint64_t *p = mat_row(m, 0, r);
      for (uint64_t w = 0; w < nw; w++) acc += (uint32_t)__builtin_popcountll(p[w]);
      out[r] = (int32_t)(2u * acc - (uint32_t)m->ncols);
    } else {
      for (uint64_t b = 0; b < m->nbits; b++) {
        const uint64_t *p = mat_row(m, b, r);
        uint32_t cnt = 0;
        for (uint64_t w = 0; w < nw; w++) cnt += (uint32_t)__builtin_popcountll(p[w]);
        cnt <<= b;
        if (m->issigned && b == m->nbits - 1) cnt = 0u - cnt;
        acc += cnt;
      }
      out[r] = (int32_t)acc;
    }
  }
}

ORC_EXPORT void orc_sum_rows(orc_ctx *c, int side, int32_t *out) { mat_rowsums(side ? &c->rhs : &c->lhs, out); }

/* arch-generic.hpp:39-76 prepareAccumulators_generic, restricted to result
 * rows [n0, n1) of the transposed result. */
static void init_acc(orc_ctx *c, uint64_t n0, uint64_t n1) {
  int lb = mat_bipolar(&c->lhs), rb = mat_bipolar(&c->rhs);
  uint64_t M = c->lhs.nrows;
  if (n1 <= n0) return;
  if (lb != rb) {
    const orc_matrix *reg = lb ? &c->rhs : &c->lhs;
    int32_t *rs = (int32_t *)malloc((reg->nrows + 1) * sizeof(int32_t));
    mat_rowsums(reg, rs);
    for (uint64_t n = n0; n < n1; n++)
      for (uint64_t m = 0; m < M; m++) c->res[n * M + m] = (int32_t)(0u - (uint32_t)(lb ? rs[n] : rs[m]));
    free(rs);
  } else {
    memset(c->res + n0 * M, 0, (n1 - n0) * M * sizeof(int32_t));
  }
}

/* arch-generic.hpp:106-163: binary GEMM over one plane pair with cache blocks
 * lhsBlock x rhsBlock and a 2x2 register tile, result rows [bn0, bn1). */
static void plane_pair_gemm(const uint64_t *A, const uint64_t *BT, int32_t *CT, uint32_t alpha,
                            uint64_t rowsA, uint64_t nw, uint64_t bn0, uint64_t bn1,
                            uint64_t M, uint64_t N, uint64_t lblk, uint64_t rblk) {
  for (uint64_t bn = bn0; bn < bn1; bn += rblk) {
    for (uint64_t bm = 0; bm < rowsA; bm += lblk) {
      for (uint64_t n = bn; n < bn + rblk; n += 2) {
        const uint64_t *b0 = BT + n * nw, *b1 = b0 + nw;
        for (uint64_t m = bm; m < bm + lblk; m += 2) {
          const uint64_t *a0 = A + m * nw, *a1 = a0 + nw;
          uint32_t s00 = 0, s01 = 0, s10 = 0, s11 = 0;
          for (uint64_t w = 0; w < nw; w++) {
            uint64_t x0 = a0[w], x1 = a1[w], y0 = b0[w], y1 = b1[w];
            s00 += (uint32_t)__builtin_popcountll(x0 & y0);
            s01 += (uint32_t)__builtin_popcountll(x0 & y1);
            s10 += (uint32_t)__builtin_popcountll(x1 & y0);
            s11 += (uint32_t)__builtin_popcountll(x1 & y1);
          }
          uint32_t s[2][2] = {{s00, s01}, {s10, s11}};
          for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
              if (m + i < M && n + j < N) {
                uint32_t *dst = (uint32_t *)&CT[(n + j) * M + (m + i)];
                *dst += s[i][j] * alpha;
              }
        }
      }
    }
  }
}

/* arch-generic.hpp:169-193 gemmBitSerial_generic_usingBinary over result rows
 * handled by rhs blocks [bn0, bn1). */
static void gemm_planes(orc_ctx *c, uint64_t bn0, uint64_t bn1) {
  uint64_t wA = c->lhs.nbits, wB = c->rhs.nbits;
  int mixed = mat_bipolar(&c->lhs) != mat_bipolar(&c->rhs);
  uint64_t n_hi = bn1 < c->rhs.nrows ? bn1 : c->rhs.nrows;
  init_acc(c, bn0, n_hi);
  for (uint64_t i = 0; i < wA; i++) {
    int ni = c->lhs.issigned && !mat_bipolar(&c->lhs) && i == wA - 1;
    for (uint64_t j = 0; j < wB; j++) {
      int nj = c->rhs.issigned && !mat_bipolar(&c->rhs) && j == wB - 1;
      uint32_t alpha = 1u << (i + j);
      if (ni != nj) alpha = 0u - alpha;
      if (mixed) alpha *= 2u;
      plane_pair_gemm(mat_row(&c->lhs, i, 0), mat_row(&c->rhs, j, 0), c->res, alpha,
                      c->lhs.nrows_a, mat_wpr(&c->lhs), bn0, bn1,
                      c->lhs.nrows, c->rhs.nrows, c->lhsBlock, c->rhsBlock);
    }
  }
}

/* arch-generic.hpp:239-262 gemmBipolar_generic_naive: res += ncols - 2*popc(a^b). */
static void gemm_bipolar(orc_ctx *c, uint64_t n0, uint64_t n1) {
  uint64_t M = c->lhs.nrows, nw = mat_wpr(&c->lhs);
  init_acc(c, n0, n1);
  for (uint64_t n = n0; n < n1; n++) {
    const uint64_t *y = mat_row(&c->rhs, 0, n);
    for (uint64_t m = 0; m < M; m++) {
      const uint64_t *x = mat_row(&c->lhs, 0, m);
      uint32_t cnt = 0;
      for (uint64_t w = 0; w < nw; w++) cnt += (uint32_t)__builtin_popcountll(x[w] ^ y[w]);
      uint32_t *dst = (uint32_t *)&c->res[n * M + m];
      *dst += (uint32_t)c->lhs.ncols - 2u * cnt;
    }
  }
}

/* arch-generic.hpp:267-300 gemvBitSerial_generic */
static void gemv_planes(orc_ctx *c) {
  uint64_t M = c->lhs.nrows, nw = mat_wpr(&c->lhs), wA = c->lhs.nbits, wB = c->rhs.nbits;
  unsigned sh0 = mat_bipolar(&c->lhs) != mat_bipolar(&c->rhs) ? 1 : 0;
  init_acc(c, 0, 1);
  for (uint64_t m = 0; m < M; m++) {
    uint32_t tot = 0;
    for (uint64_t i = 0; i < wA; i++) {
      int ni = c->lhs.issigned && !mat_bipolar(&c->lhs) && i == wA - 1;
      for (uint64_t j = 0; j < wB; j++) {
        int nj = c->rhs.issigned && !mat_bipolar(&c->rhs) && j == wB - 1;
        const uint64_t *x = mat_row(&c->lhs, i, m), *y = mat_row(&c->rhs, j, 0);
        uint64_t cnt = 0;
        for (uint64_t w = 0; w < nw; w++) cnt += (uint64_t)__builtin_popcountll(x[w] & y[w]);
        cnt <<= (i + j + sh0);
        tot += (ni != nj) ? (uint32_t)(0u - (uint32_t)cnt) : (uint32_t)cnt;
      }
    }
    uint32_t *dst = (uint32_t *)&c->res[m];
    *dst += tot;
  }
}

/* arch-generic.hpp:306-329 gemvBipolar_generic */
static void gemv_bipolar(orc_ctx *c) { gemm_bipolar(c, 0, 1); }

/* arch-generic.hpp:331-345 gemmBitSerial_generic dispatch */
ORC_EXPORT void orc_gemm(orc_ctx *c) {
  int bb = mat_bipolar(&c->lhs) && mat_bipolar(&c->rhs);
  if (c->rhs.nrows == 1) {
    if (bb) gemv_bipolar(c);
    else gemv_planes(c);
  } else {
    if (bb) gemm_bipolar(c, 0, c->rhs.nrows);
    else gemm_planes(c, 0, c->rhs.nrows_a);
  }
}

/* Multi-threaded CPU baseline: the rhs-row (N) range is split into contiguous
 * slices of whole rhs cache blocks, one per thread.  The transposed result is
 * N-major, so slices write disjoint ranges and the result is bit-identical to
 * orc_gemm. */
typedef struct { orc_ctx *c; uint64_t n0, n1; } orc_slice;

static void *slice_main(void *p) {
  orc_slice *s = (orc_slice *)p;
  int bb = mat_bipolar(&s->c->lhs) && mat_bipolar(&s->c->rhs);
  if (bb) gemm_bipolar(s->c, s->n0, s->n1 < s->c->rhs.nrows ? s->n1 : s->c->rhs.nrows);
  else gemm_planes(s->c, s->n0, s->n1);
  return NULL;
}

ORC_EXPORT void orc_gemm_threads(orc_ctx *c, int nthreads) {
  if (nthreads <= 1 || c->rhs.nrows == 1) { orc_gemm(c); return; }
  int bb = mat_bipolar(&c->lhs) && mat_bipolar(&c->rhs);
  uint64_t unit = bb ? 1 : c->rhsBlock;
  uint64_t total = bb ? c->rhs.nrows : c->rhs.nrows_a;
  uint64_t nunits = total / unit;
  if ((uint64_t)nthreads > nunits) nthreads = (int)nunits;
  pthread_t th[256];
  orc_slice sl[256];
  if (nthreads > 256) nthreads = 256;
  uint64_t u0 = 0;
  for (int t = 0; t < nthreads; t++) {
    uint64_t cnt = nunits / nthreads + ((uint64_t)t < nunits % nthreads ? 1 : 0);
    sl[t].c = c;
    sl[t].n0 = u0 * unit;
    sl[t].n1 = (u0 + cnt) * unit;
    u0 += cnt;
    pthread_create(&th[t], NULL, slice_main, &sl[t]);
  }
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* test/testhelpers.hpp:34-45 naive_int_gemm on int32 inputs:
 * res[n*M + m] = sum_k lhs[m*K + k] * rhs[n*K + k]  (mod 2^32). */
ORC_EXPORT void orc_naive_gemm(const int32_t *lhs, const int32_t *rhs, int32_t *res,
                               uint64_t M, uint64_t K, uint64_t N) {
  for (uint64_t n = 0; n < N; n++)
    for (uint64_t m = 0; m < M; m++) {
      uint32_t acc = 0;
      for (uint64_t k = 0; k < K; k++) acc += (uint32_t)lhs[m * K + k] * (uint32_t)rhs[n * K + k];
      res[n * M + m] = (int32_t)acc;
    }
}
