// gbs_internal.h -- shared declarations of libgbs (not part of the public ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gbs.h"

namespace gbs {

struct AdjPlan;   // workspace of the tensor-core adjoint (gbs_adjoint_tc.cu)
struct WidePlan;  // part sub-contexts of a context with 5-8-bit operands (gbs_wide.cu)

// Padding of the e4m3 digit matrices (the tensor-core operands): rows to a
// multiple of every tile's row count, columns to whole 256-digit stages.  The
// bit planes themselves keep the reference's padding (gbs_ctx_alloc).
constexpr uint64_t kRowAlign = 256;
constexpr uint64_t kColAlign = 256;
constexpr int kMaxBits = 8;

// e4m3 digit matrices (the tensor-core pipe's operands) are stored in 16-row
// blocks: each 16-row x 128-digit tile is 2 KB contiguous, laid out
// [row/16][col/128][row%16][col%128], and read through 4-D tensor maps whose
// boxes are whole blocks.  The SM-pair kernel's leader loads both CTAs'
// halves; writing into the peer's shared memory, these boxes run ~20 %
// faster per stage than 2-D boxes of 128-byte rows.
__host__ __device__ inline uint64_t digit_offset(uint64_t r, uint64_t col, uint64_t ncols_a) {
  return ((r >> 4) * (ncols_a >> 7) + (col >> 7)) * 2048 + ((r & 15) << 7) + (col & 127);
}
// The nibble matrix (the tensor-core pipe's compact copy of an operand: each
// element's plane code in 4 bits, the even column in the low nibble) has the
// same blocks at half the bytes: [rows/16][cols/128][16][64].  Byte offset
// of the code pair holding column col (col even).
__host__ __device__ inline uint64_t nibble_offset(uint64_t r, uint64_t col, uint64_t ncols_a) {
  return ((r >> 4) * (ncols_a >> 7) + (col >> 7)) * 1024 + ((r & 15) << 6) + ((col & 127) >> 1);
}

// One bit-serial matrix on the device: planes [nbits][nrows_a][wpr] of u64,
// with the reference's nrows_a and ncols_a (BitSerialMatrix, gemmbitserial.hpp:
// 24-50): rows padded to the context's cache block, columns to 64 bits (256
// for matrix-vector contexts).  drows x dcols is the geometry of the
// matrix's e4m3 digit matrix (rows and columns padded to 256).
struct Mat {
  uint64_t nbits = 0, nrows = 0, ncols = 0, nrows_a = 0, ncols_a = 0;
  uint64_t drows = 0, dcols = 0;
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
  // compact form of alpha used by the tiled CUDA-core kernels (alpha_of)
  int neg_i, neg_j, shift;
};

// alpha[i][j] from its compact form: +-2^(i+j+shift), negative iff exactly one
// of i == neg_i, j == neg_j (the signed MSB planes; -1 for none); -2 for XOR.
__host__ __device__ inline uint32_t alpha_of(int i, int j, int neg_i, int neg_j, int shift, int use_xor) {
  if (use_xor) return 0u - 2u;
  const uint32_t a = 1u << (i + j + shift);
  return ((i == neg_i) != (j == neg_j)) ? 0u - a : a;
}

// Output tile classes of the CUDA-core kernels: (rows of lhs) x (rows of rhs).
// 256 threads, 4 x 4 outputs per thread in every class.
__host__ __device__ constexpr int tile_bm(int cls) { return cls == 0 ? 64 : (cls == 1 ? 32 : 16); }
__host__ __device__ constexpr int tile_bn(int cls) { return cls == 0 ? 64 : (cls == 1 ? 128 : 256); }

// One problem of a grouped launch (device resident).
struct GroupProblem {
  const uint64_t *A, *B;
  int32_t *C;
  const int32_t *ra, *rb;
  uint64_t M, N, wpr, a_plane, b_plane, a_rows, b_rows;  // a_rows/b_rows: padded rows (nrows_a)
  int wa, wb, use_xor, neg_i, neg_j, shift;
  uint32_t c0;
  int cls;
};

// One output tile of a grouped launch: problem, tile row/column, class.
struct GroupTile {
  uint32_t p, mt, nt, cls;
};

// One operand of a grouped import / row-sum pass; warp0 = first global warp.
// With digits set, the import also writes the operand's e4m3 digit matrix
// [nrows_a][64 * wpr] (table dtab), the operand of the tensor-core pipe.
struct PackJob {
  const void *src;
  uint64_t *planes;
  int32_t *rowsum;
  uint8_t *digits;
  uint8_t *nibbles;  // with nibbles set, the import also writes the nibble matrix (codes, 4 bits each)
  uint64_t nrows, ncols, nrows_a, wpr, warp0;
  uint64_t dcols;  // digit-matrix columns (a multiple of 256)
  int nbits, issigned, dtype, vec;
  uint32_t segs;  // 512-column segments per row
  uint32_t dtab[4];
};

// One problem of the persistent tensor-core kernels (device resident).  The
// MMA's row operand ("MMA-A", 128 rows per tile) is the lhs, or the rhs when
// swap is set; the other operand gives the MMA's N columns per tile.  The
// digit kernel (gbs_gemm_tcg.cu) takes the larger side as MMA-A and reads
// both operands' digit matrices, N = bn; the nibble kernel
// (gbs_gemm_tcgn.cu) takes the smaller side as MMA-A (digits) and decodes
// the larger from its nibble matrix, N = 256.
struct TcgProblem {
  int32_t *C;               // result [N][M]
  uint32_t M, N;
  uint32_t a_rows, b_rows;  // padded rows of the MMA-A digit matrix / the MMA-B digit (nibble) matrix
  uint32_t nk;              // K stages of 128 digits
  uint32_t bn;              // digit kernel: MMA N, a multiple of 16 in [16, 256]
  uint32_t idesc;           // tcgen05 instruction descriptor for M = 128 and the kernel's N
  uint32_t swap;            // 1: MMA-A = rhs (tile rows are n), MMA-B = lhs (columns are m)
  uint32_t w4;              // nibble kernel: MMA-B codes of 4 bits (the two-table lookup)
  uint32_t tab[4];          // nibble kernel: e4m3 byte of every MMA-B code
  uint32_t a_bytes;         // nibble kernel: MMA-A bytes loaded per stage (rows of the smaller side, 16-row
                            // multiples up to 128, x 128 digits; the tile's other rows only feed unstored lanes)
};

// One output tile: problem, 128-row block of MMA-A, bn-column block of MMA-B.
struct TcgTile {
  uint32_t p, r, c, pad;
};

// One operand of an expansion pass: planes -> e4m3 digit matrix, or planes
// -> nibble matrix (nib set: the plane codes, 4 bits each).
struct ExpandJob {
  const uint64_t *planes;
  uint8_t *digits;   // the digit or nibble matrix
  uint64_t nrows_a, wpr, dcols;  // plane rows and words per row; digit-matrix columns
  uint64_t thread0;  // first global thread of this job (16 digits or 32 codes per thread)
  uint32_t nrows, K, chunks, nbits;
  uint32_t tab[4];   // e4m3 byte of every plane code, 4 per word
  uint32_t nib;
};

// Host-side plan of the persistent tensor-core kernels over some contexts.
struct TcgPlan {
  std::vector<gbs_ctx *> ctxs;
  // derived matrices each context needs: bit 0 / 1 the lhs / rhs digit
  // matrix, bit 2 / 3 the lhs / rhs nibble matrix (both digit matrices for
  // the digit kernel; the smaller side's digits and the larger side's
  // nibbles for the nibble kernel)
  std::vector<uint8_t> sides;
  bool nibbles = false;  // the nibble kernel (gbs_gemm_tcgn.cu) runs the plan
  TcgProblem *d_probs = nullptr;
  void *d_maps = nullptr;  // CUtensorMap [2 * nprob]: MMA-A map, MMA-B map of each problem
  TcgTile *d_tiles = nullptr;
  ExpandJob *d_jobs = nullptr;
  uint32_t nprob = 0, ntiles = 0;
  int njobs = 0;
  uint64_t expand_threads = 0;
  int grid = 0;
};

struct GemmShape {
  const uint64_t *A;  // lhs planes
  const uint64_t *B;  // rhs planes
  int32_t *C;         // result [N][M]
  uint64_t M, N, wpr;
  uint64_t a_plane, b_plane;  // words per plane (nrows_a * wpr)
  uint64_t a_rows, b_rows;    // padded rows (nrows_a) of lhs and rhs
  int tile_cls;               // CUDA-core tile class override (0..2), -1 = built-in rule
  int wa, wb;
};

}  // namespace gbs

struct gbs_ctx {
  gbs::Mat lhs, rhs;
  uint64_t lhsBlock = 0, rhsBlock = 0;
  int32_t *res = nullptr;     // [N][M]
  // result target of the forward launch being issued: res, or a caller's
  // buffer the device can write (gbs_gemm_to); res is stale after the latter
  int32_t *out = nullptr;
  bool res_stale = false;
  int32_t *rowsum = nullptr;  // scratch: row sums, lhs rows at [0, M), rhs rows at [M, M+N)
  // host-source imports: per-side device staging, a copy stream and events
  // that let the packing of each copied chunk overlap the copy of the next
  void *stage[2] = {nullptr, nullptr};
  size_t stage_bytes[2] = {0, 0};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_chunk[8] = {};
  cudaEvent_t ev_packed[2] = {};
  bool ev_packed_set[2] = {false, false};
  void *thr_stage[2] = {nullptr, nullptr};  // device copies of host-side quantisation thresholds
  size_t thr_bytes[2] = {0, 0};
  int device = 0;
  int pipe = GBS_PIPE_AUTO;
  int variant = -1;  // pipe variant: CUDA-core tile class (0..2) or tensor-core N tile (128/256); -1 = built-in rule
  // TMA descriptors (CUtensorMap, 128 bytes, 64-byte aligned) over the planes, built on first use
  alignas(64) unsigned char tc_map_a[128];
  alignas(64) unsigned char tc_map_b[128];
  bool tc_maps_ready = false;
  // e4m3 digit matrices [drows][dcols] of both operands (the tensor-core
  // pipe's operands), built from the planes on first use after each import
  uint8_t *digits[2] = {nullptr, nullptr};
  bool digits_valid[2] = {false, false};
  // nibble matrices [drows][dcols / 2] (4-bit plane codes) of either side, the
  // larger operand's form for the nibble kernel, built like the digits
  uint8_t *nibbles[2] = {nullptr, nullptr};
  bool nibbles_valid[2] = {false, false};
  int host_import = 0;  // GBS_HOST_IMPORT_*: how gbs_import reads host-memory sources
  alignas(64) unsigned char tc_map_da[128];
  alignas(64) unsigned char tc_map_db[128];
  bool digit_maps_ready = false;
  alignas(64) unsigned char tc_map_db64[128];  // rhs digits in 64-row boxes (the pair kernel's 128-column tiles)
  bool digit_map_b64_ready = false;
  int last_pair_bn = 0, last_pair_splits = 0;  // configuration of the last SM-pair launch (test hook)
  bool last_pair_persistent = false;
  int last_pair_streamk = 0;
  uint32_t debug_wait_limit = 0;  // test hook of gbs_debug_tc_timeout (0: normal launches)  // SM pairs of the last stream-K launch, 0 if the last pair launch was another kernel
  // stream-K pair kernel: fp32 partial-tile slots and flags, one per SM pair, and the launch epoch
  float *sk_ws = nullptr;
  uint32_t *sk_flags = nullptr;
  uint32_t sk_pairs = 0, sk_epoch = 0;
  // one-problem plan of the persistent tensor-core kernel (shapes with a side under 256 rows)
  gbs::TcgPlan *plan1 = nullptr;
  bool plan1_ready = false;
  gbs::AdjPlan *adj = nullptr;  // tensor-core adjoint workspace, built on first use
  gbs::WidePlan *wide = nullptr;  // tensor-core parts of 5-8-bit operands, built on first use
  bool vt_valid[2] = {false, false};  // its transposed bf16 operand values match the planes
};

namespace gbs {

// where the forward kernels of this context write the result
inline int32_t *result_ptr(const gbs_ctx *c) { return c->out ? c->out : c->res; }

// epilogue of one context (gbs_api.cu)
void make_epilogue(const gbs_ctx *c, Epilogue &e, int32_t *rowsum);

// error and bookkeeping (gbs_api.cu)
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
void count_launch(uint64_t n = 1);
cudaError_t dev_alloc(void **p, size_t bytes);

// kernels (gbs_pack.cu)
cudaError_t launch_pack(const Mat &m, const void *src, int dtype, int col_major, cudaStream_t s);
// threshold-quantising import (importRegularAndQuantize); dtype GBS_I8..GBS_F32, thr [nthres][nrows]
cudaError_t launch_pack_quantize(const Mat &m, const void *src, const void *thr, int nthres, int dtype,
                                 int col_major, uint8_t *digits, const uint32_t *dtab, cudaStream_t s);
// units of the row-major pack kernels: 1024-column segments per row
inline uint64_t pack_segs_per_row(uint64_t wpr) { return (wpr * 64 + 1023) / 1024; }
// row-major pack of padded rows [r0, r1); with digits set also the e4m3 digit rows (table dtab[4])
cudaError_t launch_pack_rows(const Mat &m, const void *src, int dtype, uint64_t r0, uint64_t r1, uint8_t *digits,
                             const uint32_t *dtab, cudaStream_t s);
cudaError_t launch_rowsum(const Mat &m, int32_t *dst, cudaStream_t s);
cudaError_t launch_export(const Mat &m, int32_t *dst, cudaStream_t s);

// forward kernels
cudaError_t launch_gemm_popc(const GemmShape &g, const Epilogue &e, cudaStream_t s);
int popc_tile_class(uint64_t M, int wa, int wb, size_t smem_cap);
// small-output shapes (matrix-vector and the like): one warp per output
bool popc_skinny(uint64_t M, uint64_t N);
constexpr int kSkinnyCls = 3;    // grouped tile class of kSkinnyTile outputs, one per warp
constexpr int kSkinnyTile = 8;
constexpr int kRowsCls = 4;      // grouped tile class of all <= kRowsMaxM lhs rows x 256 rhs rows
constexpr int kRowsMaxM = 16;
constexpr int kRowsKC = 16;      // K words per pipeline step of the rows tile (128 bytes of each row)
// rhs rows of a rows tile for M lhs rows: 256 threads, 1, 2 or 4 of them per rhs row
__host__ __device__ inline int rows_tile_n(uint64_t M) { return M <= 4 ? 256 : (M <= 8 ? 128 : 64); }
size_t popc_rows_smem(int wa, int kc);
size_t popc_stage_smem(int cls, int wa, int wb, int kc);
constexpr int kGroupKC = 8;
cudaError_t prepare_gemm_popc_grouped(size_t smem);
cudaError_t launch_gemm_popc_grouped(const GroupProblem *probs, int nprob, const GroupTile *tiles, uint32_t ntiles,
                                     uint32_t *counter, uint32_t *err, size_t smem, int grid, cudaStream_t s);
int grouped_blocks_per_sm(size_t smem);
cudaError_t launch_pack_grouped(const PackJob *jobs, int njobs, uint64_t total_warps, cudaStream_t s);
cudaError_t launch_rowsum_grouped(const PackJob *jobs, int njobs, uint64_t total_warps, cudaStream_t s);
cudaError_t launch_gemm_bmma(const GemmShape &g, const Epilogue &e, cudaStream_t s);
bool bmma_supported(int wa, int wb, int use_xor);
bool tc_exact(const gbs_ctx *c, int pipe);
uint32_t *tc_error_ptr();
cudaError_t launch_gemm_tc(gbs_ctx *c, cudaStream_t s, bool digits, int bn);
cudaError_t launch_gemm_tc_hbm(gbs_ctx *c, cudaStream_t s, int bn);
constexpr int kPairVariant = 512;     // tensor-core variant: 256 x 256 tiles on SM pairs (tcgen05 cta_group::2)
constexpr int kPairVariant128 = 513;  // the same with 256 x 128 tiles
constexpr int kPairVariantPersistent = 514;  // persistent SM pairs looping over 256 x 256 tiles
constexpr int kPairVariantStreamK = 515;     // stream-K SM pairs: (tile, K stage) units split evenly over the pairs
// SM-pair tiles with width and K split both given: 10 * width + split, width 128 or 256, split 1, 2 or 4
inline bool pair_split_variant(int v) {
  return (v == 1281 || v == 1282 || v == 1284 || v == 2561 || v == 2562 || v == 2564);
}
bool pdl_enabled();                          // programmatic dependent launch of the tensor-core kernels (GBS_PDL)
uint32_t tc_error_word();
int tc_peaks(double *f8, double *bf16);

// tensor-map and digit helpers shared by the tensor-core files (gbs_gemm_tc.cu)
bool tc_map_u8(void *map, const uint8_t *base, uint64_t cols, uint64_t rows, uint32_t box_rows);
void tc_digit_table(const Mat &m, uint32_t tab[4]);
uint64_t tc_max_abs(const Mat &m);
bool tc_encoder_available();

// persistent tensor-core kernel over a table of problems (gbs_gemm_tcg.cu)
bool tcg_eligible(const gbs_ctx *c);
bool tcg_preferred(const gbs_ctx *c);
int tcg_plan_build(TcgPlan *plan, gbs_ctx *const *ctxs, int n);
void tcg_plan_free(TcgPlan *plan);
cudaError_t tcg_expand(TcgPlan &plan, cudaStream_t s);
cudaError_t tcg_gemm(const TcgPlan &plan, uint32_t *err, cudaStream_t s, int32_t *out0 = nullptr);
cudaError_t ensure_digit_buffer(gbs_ctx *c, int side);
cudaError_t ensure_nibble_buffer(gbs_ctx *c, int side);
// the nibble kernel over a plan built with nibbles set (gbs_gemm_tcgn.cu)
cudaError_t tcgn_gemm(const TcgPlan &plan, uint32_t *err, cudaStream_t s, int32_t *out0);
cudaError_t tcgn_prepare();  // kernel attributes, once per plan build
bool tc_map_nibbles(void *map, const uint8_t *base, uint64_t cols, uint64_t rows);
// tensor-core pipe for 5-8-bit operands (gbs_wide.cu): operands split into parts of <= 4 bits
bool tc_wide(const gbs_ctx *c);
cudaError_t launch_gemm_wide(gbs_ctx *c, cudaStream_t s, int variant);
void wide_plan_free(WidePlan *p);
// tensor-core adjoint (gbs_adjoint_tc.cu)
int adjoint_tc(gbs_ctx *c, const float *dC, float *dA, float *dB, cudaStream_t s);
bool adjoint_tc_available();
void adj_plan_free(AdjPlan *p);
ExpandJob make_expand_job(const Mat &m, uint8_t *digits);
ExpandJob make_nibble_job(const Mat &m, uint8_t *nibbles);
cudaError_t launch_expand(const ExpandJob &job, cudaStream_t s);
int effective_pipe(const gbs_ctx *c);
int tuned_variant(const gbs_ctx *c, int pipe);

}  // namespace gbs
