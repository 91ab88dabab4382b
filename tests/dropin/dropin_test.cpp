// Drop-in check: code written against the reference's C++ API, compiled
// against include/gemmbitserial.hpp and linked with libgbs.so.  Groups follow
// the reference's test/test.cpp (conversions, row sums, matrix-matrix and
// matrix-vector, bipolar x regular both ways, bipolar x bipolar), compared in
// full against a naive integer GEMM (test/testhelpers.hpp:34-45).  Inputs come
// from a fixed-seed generator, so runs are reproducible.  Exit status is the
// number of failed groups.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "gemmbitserial.hpp"

using namespace gemmbitserial;

static uint64_t rng_state = 0x6762730000ull;
static uint64_t next_u64() {
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
template <typename T>
static void fill(std::vector<T> &v, int bits, bool sgn) {
  for (auto &x : v) {
    if (bits == 1 && sgn) x = (next_u64() & 1) ? 1 : -1;
    else if (sgn) x = (T)((int)(next_u64() % (1u << bits)) - (1 << (bits - 1)));
    else x = (T)(next_u64() % (1u << bits));
  }
}
template <typename L, typename R>
static void naive(const std::vector<L> &a, const std::vector<R> &b, std::vector<int32_t> &c, int M, int K, int N) {
  for (int n = 0; n < N; n++)
    for (int m = 0; m < M; m++) {
      int32_t acc = 0;
      for (int k = 0; k < K; k++) acc += (int32_t)a[m * K + k] * (int32_t)b[n * K + k];
      c[n * M + m] = acc;
    }
}

static int report(const char *name, int ok, int total) {
  printf("%s: %d/%d OK\n", name, ok, total);
  return ok == total ? 0 : 1;
}

int main() {
  const int dims[] = {3, 5, 7, 16, 17, 18, 30, 31, 32, 100, 177, 256};
  int failed = 0;
  {  // import -> export round trip, all d*d elements
    int ok = 0, total = 0;
    for (int b : {1, 2, 3, 7})
      for (int d : {4, 16, 17, 32, 77, 100, 1023})
        for (int s : {1, 0}) {
          std::vector<int8_t> x(d * d), y(d * d);
          fill(x, b, s);
          BitSerialMatrix m = BitSerialMatrix::alloc(b, d, d, s);
          m.importRegular(x.data());
          m.exportRegular(y.data());
          BitSerialMatrix::dealloc(m);
          ok += memcmp(x.data(), y.data(), d * d) == 0;
          total++;
        }
    failed += report("conversions", ok, total);
  }
  {  // BitSerialMatrix::alloc pads as the reference does: rows to rowalign, columns to colalign
    int ok = 0, total = 0;
    for (uint64_t ra : {1, 2, 7, 64})
      for (uint64_t ca : {64, 128, 256}) {
        BitSerialMatrix m = BitSerialMatrix::alloc(3, 37, 300, false, ra, ca);
        ok += m.nrows_a == (37 + ra - 1) / ra * ra && m.ncols_a == (300 + ca - 1) / ca * ca &&
              m.wordsPerRow() == m.ncols_a / 64;
        total++;
        BitSerialMatrix::dealloc(m);
      }
    GEMMContext g = allocGEMMContext(2048, 4096, 2048, 3, 2, false, true);  // the reference: 2070 / 4096 / 30
    ok += g.lhs.nrows_a == 2070 && g.rhs.nrows_a == 2070 && g.lhs.ncols_a == 4096 && g.lhsBlock == 30 &&
          g.rhsBlock == 30;
    total++;
    deallocGEMMContext(g);
    failed += report("padding", ok, total);
  }
  {  // word(): read, write and or-assign through the device proxy; padding bits stay zero
    int ok = 0, total = 0;
    BitSerialMatrix m = BitSerialMatrix::alloc(2, 5, 100, false, 8);  // rows 5..7 are padding
    m.word(1, 3, 70) = 0xF0F0F0F0F0F0F0F0ull;  // columns 64..99 of row 3: bits past column 99 are dropped
    ok += (uint64_t)m.word(1, 3, 70) == (0xF0F0F0F0F0F0F0F0ull & ((1ull << 36) - 1));
    total++;
    m.word(0, 2, 5) |= 0x21ull;
    ok += m.get(0, 2, 0) && m.get(0, 2, 5) && !m.get(0, 2, 1);
    total++;
    m.unset(0, 2, 0);
    ok += (uint64_t)m.word(0, 2, 0) == 0x20ull;
    total++;
    m.word(0, 4, 0) = ~0ull;
    m.word(0, 5, 0) = ~0ull;  // a padding row: stays zero
    ok += (uint64_t)m.word(0, 4, 0) == ~0ull && (uint64_t)m.word(0, 5, 0) == 0;  // columns 0..63 all exist
    total++;
    BitSerialMatrix::dealloc(m);
    failed += report("word", ok, total);
  }
  {  // sumRows on a copy of ctx.lhs, all d sums
    int ok = 0, total = 0;
    for (int b : {1, 2, 3, 4})
      for (int d : {4, 16, 17, 32, 77, 100, 1023})
        for (int s : {1, 0}) {
          std::vector<int8_t> x(d * d);
          fill(x, b, s);
          std::vector<int32_t> got(d), want(d, 0);
          GEMMContext ctx = allocGEMMContext(d, d, 1, b, 1, s, false);
          BitSerialMatrix bsm = ctx.lhs;
          bsm.importRegular(x.data());
          sumRows(bsm, got.data());
          deallocGEMMContext(ctx);
          for (int r = 0; r < d; r++)
            for (int c = 0; c < d; c++) want[r] += x[r * d + c];
          ok += got == want;
          total++;
        }
    failed += report("row sums", ok, total);
  }
  {  // unsigned matrix x matrix (d x 2d x 3d) and matrix x vector, uint8 overload
    int ok = 0, total = 0;
    for (int b : {2, 3, 4})
      for (int d : dims)
        for (int mv : {0, 1}) {
          int M = d, K = 2 * d, N = mv ? 1 : 3 * d;
          std::vector<uint8_t> a(M * K), bt(N * K);
          fill(a, b, false);
          fill(bt, b, false);
          std::vector<int32_t> want(M * N);
          naive(a, bt, want, M, K, N);
          GEMMContext ctx = allocGEMMContext(M, K, N, b, b, false, false);
          ctx.lhs.importRegular(a.data());
          ctx.rhs.importRegular(bt.data());
          gemmBitSerial(ctx);
          ok += memcmp(ctx.res, want.data(), M * N * 4) == 0;
          total++;
          deallocGEMMContext(ctx);
        }
    failed += report("matrix-matrix / matrix-vector", ok, total);
  }
  {  // bipolar x regular, lhs/rhs swapped and not, signed and unsigned
    int ok = 0, total = 0;
    for (int sw : {0, 1})
      for (int b : {2, 3, 4})
        for (int d : dims)
          for (int s : {1, 0}) {
            std::vector<int8_t> bip(d * d), reg(d * d);
            fill(bip, 1, true);
            fill(reg, b, s);
            std::vector<int32_t> want(d * d);
            GEMMContext ctx;
            if (sw) {
              ctx = allocGEMMContext(d, d, d, b, 1, s, true);
              ctx.lhs.importRegular(reg.data());
              ctx.rhs.importRegular(bip.data());
              naive(reg, bip, want, d, d, d);
            } else {
              ctx = allocGEMMContext(d, d, d, 1, b, true, s);
              ctx.lhs.importRegular(bip.data());
              ctx.rhs.importRegular(reg.data());
              naive(bip, reg, want, d, d, d);
            }
            gemmBitSerial(ctx);
            ok += memcmp(ctx.res, want.data(), d * d * 4) == 0;
            total++;
            deallocGEMMContext(ctx);
          }
    failed += report("bipolar x regular", ok, total);
  }
  {  // bipolar x bipolar, GEMM and GEMV
    int ok = 0, total = 0;
    for (int d : dims)
      for (int mv : {0, 1}) {
        int N = mv ? 1 : d;
        std::vector<int8_t> a(d * d), bt(N * d);
        fill(a, 1, true);
        fill(bt, 1, true);
        std::vector<int32_t> want(d * N);
        naive(a, bt, want, d, d, N);
        GEMMContext ctx = allocGEMMContext(d, d, N, 1, 1, true, true);
        ctx.lhs.importRegular(a.data());
        ctx.rhs.importRegular(bt.data());
        gemmBitSerial(ctx);
        ok += memcmp(ctx.res, want.data(), d * N * 4) == 0;
        total++;
        deallocGEMMContext(ctx);
      }
    failed += report("bipolar x bipolar", ok, total);
  }
  {  // by-value copies alias one context (as the reference's benchmark.cpp:205 relies on)
    std::vector<int8_t> a(40 * 70), bt(30 * 70);
    fill(a, 3, true);
    fill(bt, 2, false);
    std::vector<int32_t> want(40 * 30);
    naive(a, bt, want, 40, 70, 30);
    std::vector<GEMMContext> v;
    v.push_back(allocGEMMContext(40, 70, 30, 3, 2, true, false));
    GEMMContext copy = v[0];
    copy.lhs.importRegular(a.data());
    v[0].rhs.importRegular(bt.data());
    gemmBitSerial(v[0]);
    failed += report("aliasing copies", memcmp(v[0].res, want.data(), want.size() * 4) == 0, 1);
    deallocGEMMContext(copy);
  }
  {  // threshold-quantised import (importRegularAndQuantize) feeding a GEMM, float and int16 input
    int ok = 0, total = 0;
    for (int d : {7, 32, 100})
      for (int nthres : {0, 1, 3}) {
        const int M = d, K = 2 * d + 5, N = d + 3, wA = 2;
        std::vector<float> af(M * K);
        std::vector<int16_t> ai(M * K);
        for (int i = 0; i < M * K; i++) {
          af[i] = (float)(next_u64() % 1000) / 100.f;  // [0, 10)
          ai[i] = (int16_t)(next_u64() % 2000) - 1000;
        }
        std::vector<float> tf(nthres * M);
        std::vector<int16_t> ti(nthres * M);
        for (int r = 0; r < M; r++)
          for (int t = 0; t < nthres; t++) {  // ascending per row
            tf[t * M + r] = 2.5f * (t + 1) + (float)(r % 3);
            ti[t * M + r] = (int16_t)(300 * t - 400 + r);
          }
        std::vector<int8_t> bt(N * K);
        fill(bt, 2, false);
        for (int v = 0; v < 2; v++) {
          std::vector<uint8_t> q(M * K);  // the reference's loop: first threshold crossed, else nThres
          for (int r = 0; r < M; r++)
            for (int c = 0; c < K; c++) {
              int idx = r * K + c, t = 0;
              if (nthres == 0) {
                q[idx] = v ? (uint8_t)ai[idx] : (uint8_t)af[idx];
                continue;
              }
              for (; t < nthres; t++)
                if (v ? ai[idx] <= ti[t * M + r] : af[idx] <= tf[t * M + r]) break;
              q[idx] = (uint8_t)t;
            }
          for (auto &x : q) x &= (1 << wA) - 1;
          std::vector<int32_t> want(M * N);
          naive(q, bt, want, M, K, N);
          GEMMContext ctx = allocGEMMContext(M, K, N, wA, 2, false, false);
          if (v) ctx.lhs.importRegularAndQuantize(ai.data(), ti.data(), nthres);
          else ctx.lhs.importRegularAndQuantize(af.data(), tf.data(), nthres);
          ctx.rhs.importRegular(bt.data());
          gemmBitSerial(ctx);
          ok += memcmp(ctx.res, want.data(), M * N * 4) == 0;
          total++;
          deallocGEMMContext(ctx);
        }
      }
    failed += report("threshold-quantised import", ok, total);
  }
  {  // float importRegular, quantize<T>, and matrices built bit by bit with set / get / unset / clearAll
    int ok = 0, total = 0;
    for (int d : {5, 64, 130}) {
      const int M = d, K = d + 17, N = d / 2 + 1;
      std::vector<float> af(M * K);
      for (auto &x : af) x = (float)((int)(next_u64() % 800) - 400) / 100.f;  // [-4, 4)
      GEMMContext ctx = allocGEMMContext(M, K, N, 3, 2, true, false);
      ctx.lhs.importRegular(af.data());
      std::vector<int8_t> qa(M * K);  // the codes the reference's quantize<float> produces, as values
      for (int i = 0; i < M * K; i++) {
        const uint8_t q = ctx.lhs.quantize(af[i]) & 7;
        qa[i] = (int8_t)(q >= 4 ? q - 8 : q);
      }
      ctx.rhs.clearAll();
      std::vector<int8_t> bt(N * K, 0);
      for (int n = 0; n < N; n++)
        for (int k = 0; k < K; k += 3) {
          const int v = (int)(next_u64() % 4);
          bt[n * K + k] = (int8_t)v;
          if (v & 1) ctx.rhs.set(0, n, k);
          if (v & 2) ctx.rhs.set(1, n, k);
        }
      ok += ctx.rhs.get(0, 0, 0) == ((bt[0] & 1) != 0);
      total++;
      ctx.rhs.set(1, N - 1, K - 1);
      ctx.rhs.unset(1, N - 1, K - 1);
      bt[(N - 1) * K + K - 1] &= 1;
      if (ctx.rhs.get(0, N - 1, K - 1)) bt[(N - 1) * K + K - 1] |= 1;
      std::vector<int32_t> want(M * N);
      naive(qa, bt, want, M, K, N);
      gemmBitSerial(ctx);
      ok += memcmp(ctx.res, want.data(), M * N * 4) == 0;
      total++;
      if (d == 5) ctx.printSummary();
      deallocGEMMContext(ctx);
    }
    failed += report("float import, quantize and single bits", ok, total);
  }
  printf(failed ? "Some tests failed\n" : "All tests completed successfully\n");
  return failed;
}
