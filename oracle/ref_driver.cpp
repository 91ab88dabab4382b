// ref_driver.cpp -- C entry points over the UNMODIFIED reference library.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit is compiled against the
// reference's own header (gemmbitserial.hpp, included by path, never copied)
// into oracle/_ref/libgbsref.so by oracle/Makefile.  It exists where the
// reference sources exist and is used to pin the C restatement in
// gbs_oracle.c and to generate golden vectors.  It calls only the reference's
// public API: allocGEMMContext, importRegular, importRegularAndQuantize,
// gemmBitSerial, sumRows, exportRegular and deallocGEMMContext.
#include <stdint.h>
#include <string.h>
#include <chrono>
#include <thread>
#include <vector>
#include "gemmbitserial.hpp"

using namespace gemmbitserial;

namespace {
enum { I8 = 0, U8 = 1, I16 = 2, I32 = 3, F32 = 4 };

void do_import(BitSerialMatrix &m, const void *src, int dtype, bool colmajor) {
  switch (dtype) {
    case I8: m.importRegular((int8_t *)src, colmajor); break;
    case U8: m.importRegular((uint8_t *)src, colmajor); break;  // non-template overload
    case I16: m.importRegular((int16_t *)src, colmajor); break;
    case F32: m.importRegular((float *)src, colmajor); break;
    default: m.importRegular((int32_t *)src, colmajor); break;
  }
}
}  // namespace

extern "C" {

// One full reference pass: alloc -> import lhs/rhs -> gemmBitSerial -> copy res.
// dims_out (optional, 6 entries): lhs.nrows_a, rhs.nrows_a, lhs.ncols_a, rhs.ncols_a, lhsBlock, rhsBlock.
// planes_out (optional): lhs planes followed by rhs planes, in the reference layout.
int ref_run(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB, int sA, int sB,
            const void *A, int dtA, int cmA, const void *B, int dtB, int cmB,
            int32_t *res_out, uint64_t *dims_out, uint64_t *planes_out) {
  GEMMContext ctx = allocGEMMContext(M, K, N, wA, wB, sA != 0, sB != 0);
  do_import(ctx.lhs, A, dtA, cmA != 0);
  do_import(ctx.rhs, B, dtB, cmB != 0);
  gemmBitSerial(ctx);
  memcpy(res_out, ctx.res, M * N * sizeof(int32_t));
  if (dims_out) {
    dims_out[0] = ctx.lhs.nrows_a; dims_out[1] = ctx.rhs.nrows_a;
    dims_out[2] = ctx.lhs.ncols_a; dims_out[3] = ctx.rhs.ncols_a;
    dims_out[4] = ctx.lhsBlock; dims_out[5] = ctx.rhsBlock;
  }
  if (planes_out) {
    uint64_t na = ctx.lhs.nbits * ctx.lhs.wordsPerBitplane();
    uint64_t nb = ctx.rhs.nbits * ctx.rhs.wordsPerBitplane();
    memcpy(planes_out, ctx.lhs.data, na * 8);
    memcpy(planes_out + na, ctx.rhs.data, nb * 8);
  }
  deallocGEMMContext(ctx);
  return 0;
}

// sumRows over an imported matrix (the lhs of a GEMV context, as test.cpp:44-49 does).
int ref_sum_rows(uint64_t rows, uint64_t cols, uint64_t bits, int sgn, const void *src, int dt,
                 int32_t *out) {
  GEMMContext ctx = allocGEMMContext(rows, cols, 1, bits, 1, sgn != 0, false);
  do_import(ctx.lhs, src, dt, false);
  sumRows(ctx.lhs, out);
  deallocGEMMContext(ctx);
  return 0;
}

// import -> exportRegular round trip (test.cpp:87-89).
int ref_roundtrip(uint64_t rows, uint64_t cols, uint64_t bits, int sgn, const void *src, int dt,
                  int32_t *out) {
  BitSerialMatrix bsm = BitSerialMatrix::alloc(bits, rows, cols, sgn != 0);
  do_import(bsm, src, dt, false);
  bsm.exportRegular(out);
  BitSerialMatrix::dealloc(bsm);
  return 0;
}

// importRegularAndQuantize into an unsigned matrix, then exportRegular.
int ref_quantize_export(uint64_t rows, uint64_t cols, uint64_t bits, const void *src, const void *thr, int nthres,
                        int dt, int colmajor, int32_t *out) {
  BitSerialMatrix bsm = BitSerialMatrix::alloc(bits, rows, cols, false);
  const bool cm = colmajor != 0;
  switch (dt) {
    case I8: bsm.importRegularAndQuantize((int8_t *)src, (int8_t *)thr, nthres, cm); break;
    case U8: bsm.importRegularAndQuantize((uint8_t *)src, (uint8_t *)thr, nthres, cm); break;
    case I16: bsm.importRegularAndQuantize((int16_t *)src, (int16_t *)thr, nthres, cm); break;
    case I32: bsm.importRegularAndQuantize((int32_t *)src, (int32_t *)thr, nthres, cm); break;
    default: bsm.importRegularAndQuantize((float *)src, (float *)thr, nthres, cm); break;
  }
  bsm.exportRegular(out);
  BitSerialMatrix::dealloc(bsm);
  return 0;
}

// CPU baseline timing of gemmBitSerial only (imports untimed, benchmark.cpp:95-105).
// nthreads > 1 splits the rhs rows into contiguous slices, one context per
// thread, through the public API; each slice's transposed result is a
// contiguous range of the full result.  Returns mean seconds per call over
// `reps` timed calls after one warm-up call; res_out receives the result.
double ref_time_gemm(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB, int sA, int sB,
                     const void *A, int dtA, const void *B, int dtB, int reps, int nthreads,
                     int32_t *res_out) {
  if (nthreads < 1) nthreads = 1;
  if ((uint64_t)nthreads > N) nthreads = (int)N;
  size_t esz = dtB == I16 ? 2 : dtB == I32 ? 4 : 1;
  std::vector<GEMMContext> ctxs;
  std::vector<uint64_t> n0s;
  uint64_t n0 = 0;
  for (int t = 0; t < nthreads; t++) {
    uint64_t cnt = N / nthreads + ((uint64_t)t < N % nthreads ? 1 : 0);
    GEMMContext c = allocGEMMContext(M, K, cnt, wA, wB, sA != 0, sB != 0);
    do_import(c.lhs, A, dtA, false);
    do_import(c.rhs, (const char *)B + n0 * K * esz, dtB, false);
    ctxs.push_back(c);
    n0s.push_back(n0);
    n0 += cnt;
  }
  auto run_all = [&]() {
    if (nthreads == 1) { gemmBitSerial(ctxs[0]); return; }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back([&, t]() { gemmBitSerial(ctxs[t]); });
    for (auto &x : th) x.join();
  };
  run_all();
  auto t0 = std::chrono::steady_clock::now();
  for (int r = 0; r < reps; r++) run_all();
  auto t1 = std::chrono::steady_clock::now();
  for (int t = 0; t < nthreads; t++) {
    uint64_t cnt = ctxs[t].rhs.nrows;
    if (res_out) memcpy(res_out + n0s[t] * M, ctxs[t].res, cnt * M * sizeof(int32_t));
    deallocGEMMContext(ctxs[t]);
  }
  return std::chrono::duration<double>(t1 - t0).count() / (reps > 0 ? reps : 1);
}

}  // extern "C"
