// gemmbitserial.hpp -- drop-in C++ API of maltanar/gemmbitserial over libgbs.
//
// Source-compatible with the reference's hot path
//   GEMMContext ctx = allocGEMMContext(M, K, N, lhsBits, rhsBits, lhsSigned, rhsSigned);
//   ctx.lhs.importRegular(A);   ctx.rhs.importRegular(BT);
//   gemmBitSerial(ctx);         // ctx.res holds the N x M (transposed) int32 result
//   deallocGEMMContext(ctx);
// plus sumRows, BitSerialMatrix::alloc/dealloc and exportRegular.  Link with
// -lgbs.  All compute runs on the current CUDA device; the packed planes live
// in device memory (BitSerialMatrix::data is a DEVICE pointer), ctx.res is a
// host array filled when gemmBitSerial returns.
//
// Like the reference, GEMMContext and BitSerialMatrix are plain values:
// copies alias the same context (gemmbitserial.hpp:454-458 of the reference
// frees through any copy).  Errors throw std::runtime_error with the
// library's message, where the reference would assert.
#pragma once

#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "gbs.h"

namespace gemmbitserial {

namespace detail {
inline void check(int rc) {
  if (rc != GBS_OK) throw std::runtime_error(std::string("gemmbitserial: ") + gbs_last_error());
}
template <typename T> struct elem;
template <> struct elem<int8_t> { static const int code = GBS_I8; };
template <> struct elem<int16_t> { static const int code = GBS_I16; };
template <> struct elem<int32_t> { static const int code = GBS_I32; };
template <> struct elem<float> { static const int code = GBS_F32; };
// element types of importRegularAndQuantize<T>, which also takes uint8_t
template <typename T> struct qelem { static const int code = elem<T>::code; };
template <> struct qelem<uint8_t> { static const int code = GBS_U8; };
}  // namespace detail

class BitSerialMatrix {
 public:
  bool issigned = false;
  uint64_t nbits = 0, nrows = 0, ncols = 0, nrows_a = 0, ncols_a = 0;
  uint64_t *data = nullptr;  // device planes [nbits][nrows_a][ncols_a/64]

  gbs_ctx *ctx_ = nullptr;  // owning context (shared by copies)
  int side_ = GBS_LHS;

  // BitSerialMatrix::alloc (reference gemmbitserial.hpp:24-35): rows padded
  // to rowalign, columns to colalign bits (a multiple of 64), on the device.
  static BitSerialMatrix alloc(uint64_t nbits, uint64_t nrows, uint64_t ncols, bool issigned,
                               uint64_t rowalign = 1, uint64_t colalign = 64) {
    gbs_ctx *c = nullptr;
    detail::check(gbs_matrix_alloc(nbits, nrows, ncols, issigned ? 1 : 0, rowalign, colalign, &c));
    try {
      return from_ctx(c, GBS_LHS);
    } catch (...) {
      gbs_ctx_free(c);
      throw;
    }
  }

  // BitSerialMatrix::dealloc (reference gemmbitserial.hpp:38-40) for matrices made by alloc().
  static void dealloc(BitSerialMatrix bsm) { detail::check(gbs_ctx_free(bsm.ctx_)); }

  static BitSerialMatrix from_ctx(gbs_ctx *c, int side) {
    gbs_ctx_info info;
    detail::check(gbs_ctx_get_info(c, &info));
    const gbs_matrix_info &m = side ? info.rhs : info.lhs;
    BitSerialMatrix b;
    b.issigned = m.issigned != 0;
    b.nbits = m.nbits;
    b.nrows = m.nrows;
    b.ncols = m.ncols;
    b.nrows_a = m.nrows_a;
    b.ncols_a = m.ncols_a;
    b.data = m.data;
    b.ctx_ = c;
    b.side_ = side;
    return b;
  }

  bool isBipolar() const { return nbits == 1 && issigned; }
  uint64_t wordsPerRow() const { return ncols_a / 64; }
  uint64_t wordsPerBitplane() const { return nrows_a * wordsPerRow(); }

  // importRegular<T> (reference gemmbitserial.hpp:213): int8/int16/int32/float,
  // host or device memory, row-major or (readColMajor) column-major.
  template <typename T>
  void importRegular(T *matrix, bool readColMajor = false) {
    detail::check(gbs_import(ctx_, side_, matrix, detail::elem<T>::code, readColMajor ? 1 : 0, nullptr));
  }
  // The uint8_t overload (reference gemmbitserial.hpp:249): raw low bits.
  void importRegular(uint8_t *matrix, bool readColMajor = false) {
    detail::check(gbs_import(ctx_, side_, matrix, GBS_U8, readColMajor ? 1 : 0, nullptr));
  }

  // importRegularAndQuantize<T> (reference gemmbitserial.hpp:282-305):
  // thresholds[nThres][nrows], sorted per row; unsigned matrices only.
  template <typename T>
  void importRegularAndQuantize(T *matrix, T *thresholds, int nThres, bool readColMajor = false) {
    detail::check(gbs_import_quantize(ctx_, side_, matrix, thresholds, nThres, detail::qelem<T>::code,
                                      readColMajor ? 1 : 0, nullptr));
  }

  // Single bits (reference gemmbitserial.hpp:90-108, 126-129).  The planes
  // live on the device: each call synchronises it and moves one word.
  uint64_t bitpos(uint64_t col) const { return col & 63; }
  bool get(uint64_t bit, uint64_t row, uint64_t col) const {
    int v = 0;
    detail::check(gbs_get_bit(ctx_, side_, bit, row, col, &v));
    return v != 0;
  }
  void set(uint64_t bit, uint64_t row, uint64_t col) { detail::check(gbs_set_bit(ctx_, side_, bit, row, col, 1)); }
  void unset(uint64_t bit, uint64_t row, uint64_t col) { detail::check(gbs_set_bit(ctx_, side_, bit, row, col, 0)); }
  void clearAll() { detail::check(gbs_clear(ctx_, side_, nullptr)); }
  // word (reference :110-115) returns a uint64_t& into host planes; the planes
  // live on the device, so here it returns a proxy that reads or writes the
  // word through the library (padding bits stay zero)
  class WordRef {
   public:
    WordRef(gbs_ctx *c, int side, uint64_t bit, uint64_t row, uint64_t col)
        : c_(c), side_(side), bit_(bit), row_(row), col_(col) {}
    operator uint64_t() const {
      uint64_t v = 0;
      detail::check(gbs_get_word(c_, side_, bit_, row_, col_, &v));
      return v;
    }
    WordRef &operator=(uint64_t v) {
      detail::check(gbs_set_word(c_, side_, bit_, row_, col_, v));
      return *this;
    }
    WordRef &operator=(const WordRef &o) { return *this = (uint64_t)o; }
    WordRef &operator|=(uint64_t v) { return *this = (uint64_t)*this | v; }
    WordRef &operator&=(uint64_t v) { return *this = (uint64_t)*this & v; }
    WordRef &operator^=(uint64_t v) { return *this = (uint64_t)*this ^ v; }

   private:
    gbs_ctx *c_;
    int side_;
    uint64_t bit_, row_, col_;
  };
  WordRef word(uint64_t bit, uint64_t row, uint64_t col) { return WordRef(ctx_, side_, bit, row, col); }
  // DEVICE pointers into the planes (reference :117-124)
  uint64_t *rowptr(uint64_t bit, uint64_t row) { return data + bit * wordsPerBitplane() + row * wordsPerRow(); }
  uint64_t *bitplaneptr(uint64_t bit) { return data + bit * wordsPerBitplane(); }

  // quantize<T> (reference gemmbitserial.hpp:170-186): the code an element
  // is stored as (float: casts truncate toward zero, then the low byte).
  template <typename T>
  uint8_t quantize(T x) const {
    if (isBipolar()) return x > 0 ? 1 : 0;
    if (issigned && x < 0) {
      const int64_t h = (int64_t)1 << (nbits - 1);
      return (uint8_t)(h + (int64_t)(x + h));  // x + h in int64 (integer T) or float, as the reference
    }
    return (uint8_t)(int64_t)x;
  }
  // importRegular_naive (reference :136-166): the same result as importRegular
  template <typename T>
  void importRegular_naive(T *matrix, bool readColMajor = false) {
    importRegular(matrix, readColMajor);
  }

  void printSummary() const {
    std::printf("BitSerialMatrix\nBits of precision: %llu signed: %d\nActual size: %llu x %llu\n"
                "Allocated size: %llu x %llu\n",
                (unsigned long long)nbits, (int)issigned, (unsigned long long)nrows, (unsigned long long)ncols,
                (unsigned long long)nrows_a, (unsigned long long)ncols_a);
  }
  void printHex() const {
    const uint64_t n = nbits * wordsPerBitplane();
    uint64_t *w = new uint64_t[n ? n : 1];
    int rc = gbs_get_planes(ctx_, side_, w, nullptr);
    if (rc == GBS_OK)
      for (uint64_t i = 0; i < nbits; i++) {
        std::printf("Bit %llu:\n", (unsigned long long)i);
        for (uint64_t j = 0; j < nrows_a; j++) {
          for (uint64_t k = 0; k < wordsPerRow(); k++)
            std::printf("%llx ", (unsigned long long)w[(i * nrows_a + j) * wordsPerRow() + k]);
          std::printf("\n");
        }
        std::printf("\n");
      }
    delete[] w;
    detail::check(rc);
  }

  // exportRegular<T> (reference gemmbitserial.hpp:313-333) into host memory.
  template <typename T>
  void exportRegular(T *matrix) {
    const uint64_t n = nrows * ncols;
    if (n == 0) return;
    int32_t *tmp = new int32_t[n];
    int rc = gbs_export(ctx_, side_, tmp, nullptr);
    if (rc == GBS_OK)
      for (uint64_t i = 0; i < n; i++) matrix[i] = (T)tmp[i];
    delete[] tmp;
    detail::check(rc);
  }
};

class GEMMContext {
 public:
  BitSerialMatrix lhs, rhs;
  uint64_t lhsBlock = 0, rhsBlock = 0;
  int32_t *res = nullptr;  // host, rhs.nrows x lhs.nrows (transposed result)
  gbs_ctx *handle = nullptr;

  void printSummary() const {
    std::printf("GEMMContext\nLHS: ");
    lhs.printSummary();
    std::printf("RHS: ");
    rhs.printSummary();
    std::printf("Block size: %llu x %llu\n", (unsigned long long)lhsBlock, (unsigned long long)rhsBlock);
  }

  bool isBipolarTimesRegular() const { return lhs.isBipolar() != rhs.isBipolar(); }
  bool isBipolarTimesBipolar() const { return lhs.isBipolar() && rhs.isBipolar(); }
  bool isMatrixVector() const { return rhs.nrows == 1; }
};

// allocGEMMContext (reference arch-generic.hpp:78-100, gemmbitserial.hpp:415-452).
inline GEMMContext allocGEMMContext(uint64_t lhsRows, uint64_t depth, uint64_t rhsRows, uint64_t lhsBits,
                                    uint64_t rhsBits, bool lhsSigned, bool rhsSigned) {
  gbs_ctx *c = nullptr;
  detail::check(gbs_ctx_alloc(lhsRows, depth, rhsRows, lhsBits, rhsBits, lhsSigned ? 1 : 0, rhsSigned ? 1 : 0, &c));
  GEMMContext g;
  g.handle = c;
  try {  // the context is freed if anything below throws
    g.lhs = BitSerialMatrix::from_ctx(c, GBS_LHS);
    g.rhs = BitSerialMatrix::from_ctx(c, GBS_RHS);
    gbs_ctx_info info;
    detail::check(gbs_ctx_get_info(c, &info));
    g.lhsBlock = info.lhsBlock;
    g.rhsBlock = info.rhsBlock;
    g.res = new int32_t[lhsRows * rhsRows + 1]();  // zeroed: its pages exist before the device writes them
  } catch (...) {
    gbs_ctx_free(c);
    throw;
  }
  return g;
}

// The name the reference README uses (README.md:15).
inline GEMMContext allocateGEMMContext(uint64_t lhsRows, uint64_t depth, uint64_t rhsRows, uint64_t lhsBits,
                                       uint64_t rhsBits, bool lhsSigned, bool rhsSigned) {
  return allocGEMMContext(lhsRows, depth, rhsRows, lhsBits, rhsBits, lhsSigned, rhsSigned);
}

// gemmBitSerial (reference arch-generic.hpp:331-345): runs on the GPU and
// leaves the result in ctx.res when it returns.  The kernels write ctx.res
// over the host link themselves where the device can address it.
inline void gemmBitSerial(GEMMContext ctx) { detail::check(gbs_gemm_to(ctx.handle, ctx.res, nullptr)); }

// deallocGEMMContext (reference gemmbitserial.hpp:454-458).
inline void deallocGEMMContext(GEMMContext ctx) {
  delete[] ctx.res;
  detail::check(gbs_ctx_free(ctx.handle));
}

// sumRows (reference arch-generic.hpp:6-37, macro gemmbitserial.hpp:478).
inline void sumRows(BitSerialMatrix m, int32_t *row_sums) {
  detail::check(gbs_sum_rows(m.ctx_, m.side_, row_sums, nullptr));
}

}  // namespace gemmbitserial
