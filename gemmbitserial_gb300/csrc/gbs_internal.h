// gbs_internal.h -- shared declarations of libgbs (not part of the public ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbs.h"

namespace gbs {

constexpr uint64_t kRowAlign = 128;  // device row padding (rows of a plane)
constexpr uint64_t kColAlign = 256;  // device column padding (bits of a row)
constexpr int kMaxBits = 8;

// One bit-serial matrix on the device: planes [nbits][nrows_a][wpr] of u64.
struct Mat {
  uint64_t nbits = 0, nrows = 0, ncols = 0, nrows_a = 0, ncols_a = 0;
  int issigned = 0;
  uint64_t *planes = nullptr;
  bool imported = false;
  bool bipolar() const { return nbits == 1 && issigned; }
  uint64_t wpr() const { return ncols_a / 64; }
  uint64_t words() const { return nbits * nrows_a * wpr(); }
};

// Encoding-dependent epilogue of one forward GEMM:
//   res[n*M+m] = sum_ij alpha[i][j] * popc(A_i[m] OP B_j[n]) + c0 - ra[m] - rb[n]  (mod 2^32)
struct Epilogue {
  int32_t alpha[kMaxBits][kMaxBits];
  uint32_t c0;
  const int32_t *ra;  // per-lhs-row subtrahend or null
  const int32_t *rb;  // per-rhs-row subtrahend or null
  int use_xor;
};

struct GemmShape {
  const uint64_t *A;  // lhs planes
  const uint64_t *B;  // rhs planes
  int32_t *C;         // result [N][M]
  uint64_t M, N, wpr;
  uint64_t a_plane, b_plane;  // words per plane (nrows_a * wpr)
  int wa, wb;
};

}  // namespace gbs

struct gbs_ctx {
  gbs::Mat lhs, rhs;
  uint64_t lhsBlock = 0, rhsBlock = 0;
  int32_t *res = nullptr;     // [N][M]
  int32_t *rowsum = nullptr;  // scratch: row sums, lhs rows at [0, M), rhs rows at [M, M+N)
  void *stage = nullptr;      // device staging for host-side imports
  size_t stage_bytes = 0;
  int device = 0;
  int pipe = GBS_PIPE_AUTO;
};

namespace gbs {

// error and bookkeeping (gbs_api.cu)
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
void count_launch(uint64_t n = 1);
cudaError_t dev_alloc(void **p, size_t bytes);

// kernels (gbs_pack.cu)
cudaError_t launch_pack(const Mat &m, const void *src, int dtype, int col_major, cudaStream_t s);
cudaError_t launch_rowsum(const Mat &m, int32_t *dst, cudaStream_t s);
cudaError_t launch_export(const Mat &m, int32_t *dst, cudaStream_t s);

// forward kernels
cudaError_t launch_gemm_popc(const GemmShape &g, const Epilogue &e, cudaStream_t s);
cudaError_t launch_gemm_bmma(const GemmShape &g, const Epilogue &e, cudaStream_t s);
bool bmma_supported(int wa, int wb, int use_xor);

}  // namespace gbs
