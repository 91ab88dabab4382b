/*
 * gbs.h -- C ABI of the GB300 bit-serial GEMM library (libgbs.so).
 *
 * This is the drop-in boundary for maltanar/gemmbitserial's hot path
 *   allocGEMMContext -> lhs/rhs.importRegular -> gemmBitSerial -> ctx.res
 *   -> deallocGEMMContext
 * Every entry point takes plain pointers and sizes and returns an int status
 * (GBS_OK on success).  On failure gbs_last_error() returns a message for the
 * calling thread.  Device work is ordered on the caller's CUDA stream, passed
 * as an opaque handle (a cudaStream_t; NULL selects the legacy default
 * stream).  The C++ header gemmbitserial.hpp in this directory rebuilds the
 * reference's class API on top of these calls.
 *
 * Matrix storage on the device keeps the reference's bit-serial layout
 * (gemmbitserial.hpp:50) and padding: 64-bit words, [nbits][nrows_a][ncols_a/64],
 * column c of row r in plane b at word c>>6, bit c&63, all padding zero; a
 * context pads columns to 64 bits (256 for matrix-vector contexts) and rows to
 * the reference's cache block (gbs_ctx_dims).  The tensor-core pipe keeps its
 * e4m3 digit copies of the operands in a separate, 256-padded layout.
 */
#ifndef GBS_H_
#define GBS_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GBS_API __attribute__((visibility("default")))
#else
#define GBS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  GBS_OK = 0,
  GBS_EINVAL = 1,      /* invalid argument (shape, width, null pointer, ...) */
  GBS_ENOMEM = 2,      /* device or pinned-host allocation failed */
  GBS_ECUDA = 3,       /* a CUDA runtime call failed */
  GBS_ESTATE = 4,      /* call out of order (e.g. gemm before both imports) */
  GBS_ETIMEOUT = 5,    /* a bounded device wait gave up */
  GBS_EUNSUPPORTED = 6 /* valid request the library or the device cannot serve */
};

/* Element types accepted by gbs_import.  GBS_I8/I16/I32 follow the
 * reference's importRegular<T> (gemmbitserial.hpp:213): bipolar matrices map
 * x>0 to +1 and everything else to -1, other matrices keep the low nbits bits
 * of x (two's complement).  GBS_U8 follows the reference's non-template
 * uint8_t overload (gemmbitserial.hpp:249): raw low bits for every encoding.
 * GBS_F32 follows importRegular<float> (quantize<float>, :170-186): bipolar
 * x>0 -> +1; a negative x of a signed matrix -> 2^(w-1) + (uint8_t)(x +
 * 2^(w-1)); otherwise (uint8_t)x, float-to-integer casts truncating toward
 * zero (the reference defines them only for values in [0, 256)). */
enum { GBS_I8 = 0, GBS_U8 = 1, GBS_I16 = 2, GBS_I32 = 3, GBS_F32 = 4 };

enum { GBS_LHS = 0, GBS_RHS = 1 };

/* Compute pipe of the forward GEMM. */
enum {
  GBS_PIPE_AUTO = 0, /* per-shape choice (tuner store, else built-in rule) */
  GBS_PIPE_POPC = 1, /* CUDA cores: LOP3 AND/XOR + POPC */
  GBS_PIPE_BMMA = 2, /* tensor pipe: mma.sync b1 AND/XOR + popc */
  GBS_PIPE_TC = 3,       /* 5th-gen tensor cores: each operand's planes expand once (per import) into an
                            e4m3 digit matrix in HBM; TMA feeds tcgen05.mma, one MMA sums every plane pair */
  GBS_PIPE_TC_PAIRS = 4, /* 5th-gen tensor cores: packed planes staged through shared memory by TMA and
                            decoded per tile to e4m3 {0, +-2^i}; one tcgen05.mma per plane pair */
  GBS_PIPE_TC_SMEM = 5   /* as GBS_PIPE_TC_PAIRS, but each tile's planes decode to one digit tile */
};

typedef struct gbs_ctx gbs_ctx; /* opaque; copies of the handle alias one context */

typedef struct {
  uint64_t nbits, nrows, ncols, nrows_a, ncols_a;
  int issigned;
  int isbipolar;
  uint64_t *data; /* DEVICE pointer to the planes */
} gbs_matrix_info;

typedef struct {
  gbs_matrix_info lhs, rhs;
  uint64_t lhsBlock, rhsBlock; /* the reference's cache blocks (rows of lhs, rhs) */
  int32_t *res;                /* DEVICE pointer, rhs.nrows x lhs.nrows, transposed layout: the
                                  last gbs_gemm's result (not written by gbs_gemm_to into a caller
                                  buffer) */
  int pipe;                    /* pipe the next gbs_gemm will use */
} gbs_ctx_info;

/* Replaces allocGEMMContext / allocGEMMContext_generic (arch-generic.hpp:78-100,
 * gemmbitserial.hpp:415-452, macro gemmbitserial.hpp:477).  lhsRows = M,
 * depth = K, rhsRows = N; bits in [1, 8]; a 1-bit signed operand is bipolar
 * {-1,+1} (gemmbitserial.hpp:74-76).  Allocates the planes and the result on
 * the current CUDA device.  M, N or K may be 0 (empty result). */
GBS_API int gbs_ctx_alloc(uint64_t lhsRows, uint64_t depth, uint64_t rhsRows, uint64_t lhsBits,
                  uint64_t rhsBits, int lhsSigned, int rhsSigned, gbs_ctx **out);

/* The padding allocGEMMContext gives a context, without allocating:
 * dims = {lhs.nrows_a, rhs.nrows_a, lhs.ncols_a, rhs.ncols_a, lhsBlock,
 * rhsBlock}, as the reference computes them (arch-generic.hpp:78-100,
 * gemmbitserial.hpp:343-377, 415-452): columns to 64 bits (256 when N == 1),
 * rows to the cache blocks.  gbs_ctx_alloc allocates exactly this geometry. */
GBS_API int gbs_ctx_dims(uint64_t lhsRows, uint64_t depth, uint64_t rhsRows, uint64_t *dims);

/* Replaces BitSerialMatrix::alloc (gemmbitserial.hpp:24-35): a context whose
 * lhs is one nbits x nrows x ncols matrix with rows padded to rowalign (>= 1)
 * and columns to colalign bits (a positive multiple of 64); its rhs is empty.
 * Import, export, get/set and row sums work on it as on a context's lhs. */
GBS_API int gbs_matrix_alloc(uint64_t nbits, uint64_t nrows, uint64_t ncols, int issigned, uint64_t rowalign,
                             uint64_t colalign, gbs_ctx **out);

/* Alias of gbs_ctx_alloc under the name the reference README uses
 * (README.md:15, "allocateGEMMContext"). */
GBS_API int gbs_ctx_allocate(uint64_t lhsRows, uint64_t depth, uint64_t rhsRows, uint64_t lhsBits,
                     uint64_t rhsBits, int lhsSigned, int rhsSigned, gbs_ctx **out);

/* Replaces deallocGEMMContext (gemmbitserial.hpp:454-458).  Synchronises the
 * device, then frees every buffer of the context.  NULL is a no-op. */
GBS_API int gbs_ctx_free(gbs_ctx *ctx);

/* Shapes, padding and device pointers of a context (the public fields of
 * GEMMContext / BitSerialMatrix, gemmbitserial.hpp:44-50, 379-383). */
GBS_API int gbs_ctx_get_info(const gbs_ctx *ctx, gbs_ctx_info *info);

/* Replaces BitSerialMatrix::importRegular<T> (gemmbitserial.hpp:213-245) and
 * its uint8_t overload (:249-275) for ctx.lhs (side 0, M x K) or ctx.rhs
 * (side 1, N x K, i.e. B transposed).  src is row-major [rows][K], or
 * [K][rows] when col_major (the reference's readColMajor).  src may be host
 * memory (pageable or pinned) or device memory.  Host data the device can
 * address (pinned, or pageable where the GPU walks the host page tables) is
 * packed in place over the host link; other host data is copied to the
 * device first, in chunks whose packing overlaps the next copy.
 * GBS_HOST_DIRECT=0 in the environment forces the copies.  The packing runs
 * on `stream`; with host src the call returns once src may be reused. */
GBS_API int gbs_import(gbs_ctx *ctx, int side, const void *src, int dtype, int col_major, void *stream);

/* Replaces BitSerialMatrix::importRegularAndQuantize<T> (gemmbitserial.hpp:
 * 282-305) for one side: element x of row r becomes the index t of the first
 * threshold thresholds[t * rows + r] with x <= threshold, or nthres when x
 * exceeds them all (no thresholds: the element's own low byte); the low nbits
 * bits of that index are stored.  Thresholds are [nthres][rows], of the same
 * element type as src (GBS_I8, GBS_U8, GBS_I16, GBS_I32 or GBS_F32), sorted
 * ascending per row as the reference assumes (unsorted ones give the
 * reference's first-crossing result).  Only unsigned matrices: GBS_EINVAL for
 * a signed one, where the reference asserts.  src and thresholds may be host
 * or device memory; with host memory the call returns once both may be
 * reused.  Float input without thresholds is truncated toward zero first. */
GBS_API int gbs_import_quantize(gbs_ctx *ctx, int side, const void *src, const void *thresholds, int nthres,
                                int dtype, int col_major, void *stream);

/* Replaces gemmBitSerial / gemmBitSerial_generic (arch-generic.hpp:331-345,
 * macro gemmbitserial.hpp:476): res = lhs * rhs^T in the transposed layout
 * res[n*M + m], bit-exact with the reference (int32 with wrap-around).
 * Asynchronous on `stream`. */
GBS_API int gbs_gemm(gbs_ctx *ctx, void *stream);

/* gemmBitSerial followed by the read of ctx.res (gemmbitserial.hpp:383), as
 * the reference's callers do it, fused: the forward kernels write the N x M
 * result straight into dst (M*N int32) when dst is device or pinned host
 * memory, 16-byte aligned, so the transfer over the host link overlaps the
 * GEMM instead of following it.  Otherwise (pageable or unaligned dst) it
 * runs gbs_gemm and copies.  With host dst the
 * call returns after the result has landed.  A direct write leaves the
 * context's own device result stale: gbs_get_result then fails with
 * GBS_ESTATE until the next gbs_gemm. */
GBS_API int gbs_gemm_to(gbs_ctx *ctx, int32_t *dst, void *stream);

/* Copies the result (ctx.res in the reference, gemmbitserial.hpp:383) to dst,
 * host or device memory of M*N int32.  With host dst the call returns after
 * the copy has completed. */
GBS_API int gbs_get_result(gbs_ctx *ctx, int32_t *dst, void *stream);

/* Replaces sumRows / sumRows_generic (arch-generic.hpp:6-37, macro
 * gemmbitserial.hpp:478) for one side of the context: dst[r] = sum of the
 * values of row r.  dst is host or device memory of nrows int32. */
GBS_API int gbs_sum_rows(gbs_ctx *ctx, int side, int32_t *dst, void *stream);

/* Replaces BitSerialMatrix::exportRegular<int32_t> (gemmbitserial.hpp:313-333)
 * for one side: dst[r*ncols + c] = value of element (r, c).  dst is host or
 * device memory of nrows*ncols int32. */
GBS_API int gbs_export(gbs_ctx *ctx, int side, int32_t *dst, void *stream);

/* Copies the packed planes of one side (BitSerialMatrix::data,
 * gemmbitserial.hpp:50) to dst, host or device memory of
 * nbits * nrows_a * ncols_a/64 uint64 words.  With host dst the call returns
 * after the copy has completed. */
GBS_API int gbs_get_planes(gbs_ctx *ctx, int side, uint64_t *dst, void *stream);

/* BitSerialMatrix::get / set / unset (gemmbitserial.hpp:90-108) on one bit
 * of one side's device planes: bit < nbits, row < nrows_a, col < ncols_a
 * for get, row < nrows and col < ncols for set (padding stays zero), else
 * GBS_EINVAL (the reference does not check).  Both synchronise the
 * device, then read or read-modify-write the one word; a set marks the side
 * imported, so matrices can be built bit by bit as with the reference. */
GBS_API int gbs_get_bit(gbs_ctx *ctx, int side, uint64_t bit, uint64_t row, uint64_t col, int *value);
GBS_API int gbs_set_bit(gbs_ctx *ctx, int side, uint64_t bit, uint64_t row, uint64_t col, int value);

/* BitSerialMatrix::word (gemmbitserial.hpp:110-115): the 64-bit plane word
 * holding (bit, row, col), read or written (the device is synchronised first;
 * one word moves).  A written word keeps the padding zero: bits of columns
 * past ncols, and whole words of rows past nrows, are stored as 0. */
GBS_API int gbs_get_word(gbs_ctx *ctx, int side, uint64_t bit, uint64_t row, uint64_t col, uint64_t *value);
GBS_API int gbs_set_word(gbs_ctx *ctx, int side, uint64_t bit, uint64_t row, uint64_t col, uint64_t value);

/* BitSerialMatrix::clearAll (gemmbitserial.hpp:95-98): zeroes every plane of
 * one side on `stream` (and marks the side imported). */
GBS_API int gbs_clear(gbs_ctx *ctx, int side, void *stream);

/* Forces the variant of a context's pipe: CUDA-core tile class (0: 64x64,
 * 1: 32x128, 2: 16x256 outputs per CTA, 4: every lhs row of a context with
 * at most 16 of them x 256 rhs rows, one rhs row per thread), tensor-core N
 * tile (128 or 256 rows
 * of rhs per 128-row lhs tile on one SM), or 512 / 513 for GBS_PIPE_TC:
 * 256 x 256 / 256 x 128 tiles computed by pairs of SMs (tcgen05
 * cta_group::2), K split over up to 4 pairs of one cluster when the tiles are
 * too few to fill the GPU, or 514: persistent SM pairs looping over
 * 256 x 256 tiles (about three per pair when forced; the built-in rule takes
 * them for grids of more tiles than one wave holds), or 515: stream-K SM
 * pairs, the (256 x 256 tile, K stage) units split evenly over every pair the
 * GPU holds at once, split tiles summed through a per-context workspace, or
 * 10 * width + split (1281, 1282, 1284, 2561, 2562, 2564): SM-pair tiles of
 * that width with K split over that many pairs of a cluster (a split that
 * cannot run -- fewer K stages than chunks, too many clusters -- runs as 1);
 * -1 restores the built-in rule.  No reference counterpart. */
GBS_API int gbs_set_variant(gbs_ctx *ctx, int variant);

/* Forces the pipe of a context's forward GEMM (GBS_PIPE_*). */
GBS_API int gbs_set_pipe(gbs_ctx *ctx, int pipe);

/* How gbs_import brings a host-memory source of this context to the GPU. */
enum {
  GBS_HOST_IMPORT_AUTO = 0,  /* the pack kernel reads the source in place where the device can
                                (pinned memory; pageable memory where the GPU walks the host page
                                tables), unless GBS_HOST_DIRECT=0; otherwise staged copies */
  GBS_HOST_IMPORT_STAGED = 1 /* copy-engine copies into a device buffer, in chunks whose packing
                                overlaps the next copy */
};
/* Sets a context's host import mode (GBS_HOST_IMPORT_*; default AUTO).  Reading
 * in place needs no copy and is the faster choice while the GPU runs one
 * context at a time; staged copies leave the transfer to the copy engines and
 * the SMs to other work, the faster choice when another context's GEMM holds
 * most SMs at the same time (two host threads driving two contexts).  Either
 * way gbs_import returns once the source has been read.  No reference
 * counterpart. */
GBS_API int gbs_set_host_import(gbs_ctx *ctx, int mode);

/* ---- one-shot GEMM without allocation ---------------------------------- *
 * No counterpart in the reference.  For callers that cannot let the library
 * call cudaMalloc -- code running while a stream is captured into a CUDA
 * graph in global capture mode, real-time loops that must not enter the
 * allocator, hosts with a fixed memory budget -- this computes
 * gemmBitSerial of device inputs straight into a device result:
 *   res[n*M + m] = sum_k A[m*K + k] * B[n*K + k]   (bit-exact, int32 wrap)
 * with lhs = A (M x K) and rhs = B (N x K) row-major DEVICE arrays of the
 * given GBS_* element types, encoded as in gbs_import.  Inputs and result
 * must be memory of the current device (or managed memory); another GPU's
 * memory or host memory is rejected with GBS_EINVAL.  It allocates nothing:
 * the packed planes and row sums live in one fixed file-scope device array of
 * gbs_noalloc_scratch_bytes() bytes (16 MiB), which every GPU that loads the
 * library holds until exit.  A GEMM whose packed operands do not fit is
 * rejected with GBS_EINVAL.  The first call on each device looks up the
 * array's device address; make that first call before any stream capture.
 * Every call shares the array: calls that overlap on the GPU (other streams
 * or host threads) race, so order them on one stream. */
GBS_API int gbs_gemm_noalloc(const void *lhs, int lhs_dtype, const void *rhs, int rhs_dtype, uint64_t M,
                             uint64_t K, uint64_t N, uint64_t lhsBits, uint64_t rhsBits, int lhsSigned,
                             int rhsSigned, int32_t *res, void *stream);

/* Size in bytes of the fixed device array gbs_gemm_noalloc works in. */
GBS_API uint64_t gbs_noalloc_scratch_bytes(void);

/* ---- adjoint (quantisation-aware training) ------------------------------ *
 * No reference counterpart: the reference has no backward pass.  For the
 * forward res[n*M + m] = sum_k A[m,k] * B[n,k] of an imported context and an
 * FP32 upstream gradient dC in the same transposed layout (N x M):
 *   dA[m*K + k] = sum_n dC[n*M + m] * B[n,k]     (M x K, row-major)
 *   dB[n*K + k] = sum_m dC[n*M + m] * A[m,k]     (N x K, the rhs layout)
 * with A, B the values the planes encode (bipolar: +-1; signed MSB negative).
 * FP32 accumulation.  dC, dA, dB are DEVICE pointers, 16-byte aligned (as
 * cudaMalloc returns them; GBS_EINVAL otherwise); dA or dB may be NULL to
 * skip that gradient.  Asynchronous on `stream`. */
GBS_API int gbs_adjoint(gbs_ctx *ctx, const float *dC, float *dA, float *dB, void *stream);

/* ---- grouped GEMM ------------------------------------------------------ *
 * No single reference counterpart: the reference runs a list of GEMMs as a
 * host loop of gemmBitSerial over a vector of contexts (benchmark.cpp:192-219).
 * A group runs the GEMMs of many contexts (any shapes, widths and encodings,
 * same device) as ONE persistent kernel that drains a device tile queue;
 * results land in each context's result buffer.  Contexts must outlive the
 * group and keep their shapes. */
typedef struct gbs_group gbs_group;

/* Builds the device problem table and the tile queue for ctxs[0..count). */
GBS_API int gbs_group_create(gbs_ctx *const *ctxs, int count, gbs_group **out);

/* importRegular for every operand in one launch: lhs_srcs[p] (M x K) and
 * rhs_srcs[p] (N x K) are row-major DEVICE pointers; dtypes holds 2*count
 * GBS_* codes (lhs, rhs per problem) or is NULL for all GBS_I8. */
GBS_API int gbs_group_import(gbs_group *g, const void *const *lhs_srcs, const void *const *rhs_srcs,
                             const int *dtypes, void *stream);

/* gemmBitSerial for every problem of the group: one persistent launch (plus
 * one row-sum launch when some problem is bipolar x regular). */
GBS_API int gbs_group_gemm(gbs_group *g, void *stream);

/* Captures [grouped import of the given sources] + grouped GEMM into a CUDA
 * graph held by the group (sources NULL: GEMM only, operands already
 * imported).  The captured sources are fixed; refill their contents and
 * replay.  `stream` must be a created stream (GBS_EINVAL for NULL: CUDA
 * cannot capture the legacy default stream). */
GBS_API int gbs_group_capture(gbs_group *g, const void *const *lhs_srcs, const void *const *rhs_srcs,
                              const int *dtypes, void *stream);

/* Launches the captured graph on `stream`. */
GBS_API int gbs_group_replay(gbs_group *g, void *stream);

/* Reads the device error word of the group (synchronises `stream`):
 * GBS_EINVAL if the grouped kernel rejected a tile descriptor. */
GBS_API int gbs_group_status(gbs_group *g, void *stream);

/* Tile count (both kernels), and dynamic shared memory per CTA and
 * persistent grid size of the CUDA-core popcount kernel. */
GBS_API int gbs_group_stats(const gbs_group *g, uint64_t *ntiles, uint64_t *smem_bytes, uint64_t *grid);

/* How the group's problems are split between the CUDA-core popcount kernel
 * and the tensor-core kernel over e4m3 digit matrices, and the tensor-core
 * kernel's tile count.  The tensor-core kernel takes a problem when its
 * result is exact in fp32 (K * max|a| * max|b| < 2^24, at most 4 bits per
 * operand) and it is the cheaper one; GBS_GROUP_PIPE=popc or =tc in the
 * environment at gbs_group_create forces one kernel. */
GBS_API int gbs_group_split(const gbs_group *g, uint64_t *popc_problems, uint64_t *tc_problems, uint64_t *tc_tiles);

/* Synchronises the device and frees the group (not its contexts). */
GBS_API int gbs_group_free(gbs_group *g);

/* Measures the sustained AND+popcount rate (bit operations per second: one
 * bit of one plane pair of one output) of the CUDA-core pipe and of the b1
 * tensor pipe on the current device (~50 ms).  Either pointer may be NULL.
 * No reference counterpart: the reference has a single CPU pipe. */
GBS_API int gbs_pipe_peaks(double *popc_bitops, double *bmma_bitops);

/* Measures the tcgen05.mma rate at full SM clock (FLOP/s, 2 per
 * multiply-add) of the current device for e4m3 (kind::f8f6f4) and bf16
 * (kind::f16) operands with an fp32 accumulator, M=128 N=256: short bursts,
 * too short for the power limit to lower the clock (~30 ms in all).  No
 * reference counterpart. */
GBS_API int gbs_tc_peaks(double *f8_flops, double *bf16_flops);

/* Measures the sustained FP32 FMA rate (FLOP/s, 2 per FMA) of the current
 * device, the roofline of gbs_adjoint (~20 ms).  No reference counterpart. */
GBS_API int gbs_fma_peak(double *flops);

/* ---- autotuner ----------------------------------------------------------- *
 * No reference counterpart (the reference picks cache blocks analytically,
 * gemmbitserial.hpp:343-377).  gbs_tune times every pipe and variant that
 * applies to an imported context on `stream` (reps timed calls each) and
 * records the fastest for the context's shape class (log4 buckets of M, N,
 * K), widths and encodings; GBS_PIPE_AUTO contexts of that class then use
 * it.  The store persists through gbs_tuner_save / gbs_tuner_load (a
 * versioned text file; a file from another version is rejected and its
 * entries ignored).  The library also loads the file named by the
 * environment variable GBS_TUNER_STORE on first use. */
GBS_API int gbs_tune(gbs_ctx *ctx, int reps, int *best_pipe, void *stream);
GBS_API int gbs_tuner_save(const char *path);
GBS_API int gbs_tuner_load(const char *path, int replace);
GBS_API int gbs_tuner_entries(void);
GBS_API int gbs_tuner_clear(void);
/* The store's entry for ctx's shape class: its pipe, variant and the time
 * gbs_tune measured (us); GBS_ESTATE when the store has none. */
GBS_API int gbs_tuner_lookup(const gbs_ctx *ctx, int *pipe, int *variant, double *us);

/* Message describing the last failure on the calling thread ("" if none). */
GBS_API const char *gbs_last_error(void);

/* Library version string. */
GBS_API const char *gbs_version(void);

/* ---- test hooks (host-side fault injection; no device faults) ---------- */

/* Makes the n-th next allocation made by the library fail (n >= 1); 0 disarms. */
GBS_API void gbs_debug_fail_alloc_after(int n);

/* Error bits raised by tensor-core kernels whose bounded waits gave up (0 = none). */
GBS_API uint32_t gbs_debug_tc_error(void);

/* Overwrites tile `tile` of a group's queue with an invalid descriptor, to
 * exercise the grouped kernel's descriptor validation (host-side injection). */
GBS_API int gbs_debug_group_poison_tile(gbs_group *g, uint32_t tile);

/* Which persistent tensor-core kernel runs a group's tensor-core problems:
 * 0 none, 1 the digit kernel (both operands as e4m3 digit matrices), 2 the
 * nibble kernel (the larger operand as 4-bit codes, decoded to digits in
 * shared memory).  By default an estimate of both kernels' critical paths
 * chooses (hundreds of problems: nibbles; one or a few: digits);
 * GBS_TCG_NIBBLES=0 or 1 in the environment at gbs_group_create forces the
 * digit or the nibble kernel.  Negative on a NULL group. */
GBS_API int gbs_debug_group_tc_kernel(const gbs_group *g);

/* Exercises the tensor-core kernels' bounded waits without a GPU fault: one
 * launch of the SM-pair kernel over ctx (an imported context of M, N >= 256
 * whose widths the tensor cores cover) that loads and multiplies nothing, so
 * its first mbarrier wait gives up after `rounds` try_wait rounds.  The kernel
 * then takes the abort path every such wait has -- error bit, bounded drains,
 * TMEM freed, return -- and this call returns GBS_ETIMEOUT once the stream is
 * idle, with the error word cleared again and the context usable.  The
 * result buffer is not written.  No reference counterpart. */
GBS_API int gbs_debug_tc_timeout(gbs_ctx *ctx, uint32_t rounds, void *stream);

/* Number of kernel launches the library has issued since load (all entry points). */
GBS_API uint64_t gbs_debug_launch_count(void);

/* Tile width (256 or 128), K split (1, 2 or 4; for the stream-K kernel the
 * number of SM pairs it ran on) and which SM-pair kernel ran for the last
 * SM-pair launch of ctx: 0 one tile per pair, 1 the persistent kernel, 2 the
 * stream-K kernel; all 0 if none was. */
GBS_API int gbs_debug_last_pair(const gbs_ctx *ctx, int *bn, int *splits, int *persistent);

#ifdef __cplusplus
}
#endif

#endif /* GBS_H_ */
