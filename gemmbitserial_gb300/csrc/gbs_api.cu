// gbs_api.cu -- the C ABI declared in include/gbs.h.
//
// Host-side control of the bit-serial GEMM path: context allocation and
// sizing (allocGEMMContext_base, gemmbitserial.hpp:415-452), imports
// (importRegular, :213-275), the forward dispatch (gemmBitSerial_generic,
// arch-generic.hpp:331-345) with its encoding-dependent epilogue
// (prepareAccumulators_generic, :39-76; usingBinary weights, :179-192;
// bipolar correction, :255-259), result read-back and deallocation.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "gbs_internal.h"

namespace gbs {

static thread_local std::string g_last_error;
static std::atomic<int> g_fail_alloc_countdown{0};
static std::atomic<uint64_t> g_launches{0};

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return GBS_ECUDA;
}

void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaError_t dev_alloc(void **p, size_t bytes) {
  int c = g_fail_alloc_countdown.load();
  if (c > 0) {
    if (g_fail_alloc_countdown.fetch_sub(1) == 1) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  if (bytes == 0) bytes = 256;
  return cudaMalloc(p, bytes);
}

namespace {

uint64_t round_up(uint64_t x, uint64_t a) { return a ? (x + a - 1) / a * a : x; }

// Makes the context's device current for the scope of one call.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) { ok = false; return; }
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
  }
  ~DeviceGuard() {
    int cur;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

bool is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown host pointer
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Address through which this device reads or writes caller memory `p`, or
// nullptr when it cannot: its own and managed memory as they are, pinned host
// memory through its mapped device address, and (with `pageable`) pageable
// host memory as it is where the GPU walks the host's page tables
// (NVLink-C2C systems such as GB300).  GBS_HOST_DIRECT=0 turns the host cases
// off (staged copies instead).
void *device_view(const void *p, int dev, bool pageable_ok) {
  const char *env = getenv("GBS_HOST_DIRECT");
  const bool host_direct = !(env && env[0] == '0');
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeManaged) return const_cast<void *>(p);
  if (a.type == cudaMemoryTypeDevice) return a.device == dev ? const_cast<void *>(p) : nullptr;  // other GPUs: copies
  if (!host_direct) return nullptr;
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  static std::atomic<int> pageable[64];  // 0 unknown, 1 yes, 2 no (racing first calls store the same value)
  if (!pageable_ok || dev < 0 || dev >= 64) return nullptr;
  int known = pageable[dev].load(std::memory_order_relaxed);
  if (!known) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    known = v ? 1 : 2;
    pageable[dev].store(known, std::memory_order_relaxed);
  }
  return known == 1 ? const_cast<void *>(p) : nullptr;
}

size_t elem_size(int dtype) { return dtype == GBS_I16 ? 2 : (dtype == GBS_I32 || dtype == GBS_F32) ? 4 : 1; }

void free_ctx_buffers(gbs_ctx *c) {
  if (c->lhs.planes) cudaFree(c->lhs.planes);
  if (c->rhs.planes) cudaFree(c->rhs.planes);
  if (c->res) cudaFree(c->res);
  if (c->rowsum) cudaFree(c->rowsum);
  for (int side = 0; side < 2; side++) {
    if (c->stage[side]) cudaFree(c->stage[side]);
    if (c->thr_stage[side]) cudaFree(c->thr_stage[side]);
    if (c->ev_packed[side]) cudaEventDestroy(c->ev_packed[side]);
  }
  for (cudaEvent_t ev : c->ev_chunk)
    if (ev) cudaEventDestroy(ev);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->plan1) {
    tcg_plan_free(c->plan1);
    delete c->plan1;
  }
  adj_plan_free(c->adj);
  wide_plan_free(c->wide);
  if (c->sk_ws) cudaFree(c->sk_ws);
  if (c->sk_flags) cudaFree(c->sk_flags);
  if (c->digits[0]) cudaFree(c->digits[0]);
  if (c->digits[1]) cudaFree(c->digits[1]);
  if (c->nibbles[0]) cudaFree(c->nibbles[0]);
  if (c->nibbles[1]) cudaFree(c->nibbles[1]);
}

// The reference's padding of a context's bit planes, restated:
// allocGEMMContext_generic (arch-generic.hpp:78-100) picks the register
// blocking (2 x 1 x 2 words, or 1 x 4 x 1 for matrix-vector contexts, whose
// depth aligns to 256 bits) and a 32 KiB cache budget; allocGEMMContext_base
// (gemmbitserial.hpp:415-452) turns them into cache blocks with
// computeBlockSize (:343-360, the positive root of a quadratic in single
// precision, as the reference computes it) and finetuneBlockSize (:364-377),
// and BitSerialMatrix::alloc (:24-35) pads rows to the block and columns to
// 64 bits times the depth blocking.  Empty sides (M or N = 0, where the
// reference divides by zero) pad to nothing.
struct Geometry {
  uint64_t lhs_rows = 0, rhs_rows = 0, cols = 0, lhs_block = 0, rhs_block = 0;
};

void block_size(float lm, float rm, float cache_bits, float dbits, uint64_t &lb, uint64_t &rb) {
  const float qa = (float)sizeof(int32_t) * lm * rm, qb = dbits * (lm + rm), qc = -cache_bits;
  const float disc = sqrtf(qb * qb - 4.0f * qa * qc);
  const int64_t x0 = (int64_t)floorf((-qb + disc) / (2.0f * qa)), x1 = (int64_t)floorf((-qb - disc) / (2.0f * qa));
  const int64_t x = x0 > x1 ? x0 : x1;
  if (x > 0) {
    lb = (uint64_t)(lm * (float)x);
    rb = (uint64_t)(rm * (float)x);
  } else {
    lb = (uint64_t)lm;
    rb = (uint64_t)rm;
  }
}

uint64_t finetune_block(uint64_t rows, uint64_t bs_max, uint64_t div) {
  uint64_t best = bs_max, waste = round_up(rows, bs_max) - rows;
  for (uint64_t cand = bs_max; cand > div; cand -= div) {
    if (cand % div) continue;
    const uint64_t wst = round_up(rows, cand) - rows;
    if (wst < waste) {
      best = cand;
      waste = wst;
    }
  }
  return best;
}

Geometry reference_geometry(uint64_t M, uint64_t K, uint64_t N) {
  const uint64_t rl = N == 1 ? 1 : 2, rd = N == 1 ? 4 : 1, rr = N == 1 ? 1 : 2;
  const float cache_bits = 32.0f * 1024.0f * 8.0f;
  Geometry g;
  const uint64_t kal = round_up(K, rd * 64);
  block_size((float)rl, (float)rr, cache_bits, (float)kal, g.lhs_block, g.rhs_block);
  if (g.lhs_block > M || g.rhs_block > N) {
    g.lhs_block = round_up(M, rl);
    g.rhs_block = round_up(N, rr);
  } else {
    if ((double)(round_up(M, g.lhs_block) - M) > 0.1 * (double)M) g.lhs_block = finetune_block(M, g.lhs_block, rl);
    if ((double)(round_up(N, g.rhs_block) - N) > 0.1 * (double)N) g.rhs_block = finetune_block(N, g.rhs_block, rr);
  }
  g.lhs_rows = round_up(M, g.lhs_block);
  g.rhs_rows = round_up(N, g.rhs_block);
  g.cols = round_up(K, rd * 64);
  return g;
}

int alloc_context(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB, int sA, int sB, const Geometry &geo,
                  gbs_ctx **out, const char *who);

// Epilogue and operand order for one context (see gbs_internal.h: Epilogue).
}  // namespace

void make_epilogue(const gbs_ctx *c, Epilogue &e, int32_t *rowsum) {
  memset(&e, 0, sizeof(e));
  const bool lb = c->lhs.bipolar(), rb = c->rhs.bipolar();
  e.neg_i = (c->lhs.issigned && !lb) ? (int)c->lhs.nbits - 1 : -1;
  e.neg_j = (c->rhs.issigned && !rb) ? (int)c->rhs.nbits - 1 : -1;
  if (lb && rb) {  // arch-generic.hpp:255-259: ncols - 2 * popc(a ^ b)
    e.use_xor = 1;
    e.alpha[0][0] = -2;
    e.c0 = (uint32_t)c->lhs.ncols;
    return;
  }
  const bool mixed = lb != rb;  // arch-generic.hpp:185: alpha doubled, res seeded with -rowsum(regular)
  e.shift = mixed ? 1 : 0;
  for (uint64_t i = 0; i < c->lhs.nbits; i++) {
    const bool ni = c->lhs.issigned && !lb && i == c->lhs.nbits - 1;
    for (uint64_t j = 0; j < c->rhs.nbits; j++) {
      const bool nj = c->rhs.issigned && !rb && j == c->rhs.nbits - 1;
      uint32_t a = 1u << (i + j);
      if (ni != nj) a = 0u - a;
      if (mixed) a *= 2u;
      e.alpha[i][j] = (int32_t)a;
    }
  }
  if (mixed) {
    if (lb) e.rb = rowsum;  // result row n is seeded with -rowsum(rhs row n)
    else e.ra = rowsum;     // result column m is seeded with -rowsum(lhs row m)
  }
}

int choose_pipe(const gbs_ctx *c);

// The pipe gbs_gemm will actually run: a forced tensor-core pipe falls back to
// the CUDA cores for shapes it does not cover.
int effective_pipe(const gbs_ctx *c) {
  const int p = c->pipe == GBS_PIPE_AUTO ? choose_pipe(c) : c->pipe;
  if (p == GBS_PIPE_TC && tc_wide(c)) return p;  // 5-8-bit operands in parts of <= 4 bits
  if ((p == GBS_PIPE_TC || p == GBS_PIPE_TC_PAIRS || p == GBS_PIPE_TC_SMEM) && !tc_exact(c, p)) return GBS_PIPE_POPC;
  return p;
}

}  // namespace gbs

using namespace gbs;

extern "C" {

const char *gbs_version(void) { return "gemmbitserial-gb300 0.1 (sm_103a)"; }

const char *gbs_last_error(void) { return g_last_error.c_str(); }

void gbs_debug_fail_alloc_after(int n) { g_fail_alloc_countdown.store(n > 0 ? n : 0); }

uint64_t gbs_debug_launch_count(void) { return g_launches.load(); }

uint32_t gbs_debug_tc_error(void) { return tc_error_word(); }

int gbs_debug_last_pair(const gbs_ctx *c, int *bn, int *splits, int *persistent) {
  if (!c || !bn || !splits || !persistent) return fail(GBS_EINVAL, "gbs_debug_last_pair: NULL argument");
  *bn = c->last_pair_bn;
  *splits = c->last_pair_streamk ? c->last_pair_streamk : c->last_pair_splits;
  *persistent = c->last_pair_streamk ? 2 : (c->last_pair_persistent ? 1 : 0);
  return GBS_OK;
}

int gbs_tc_peaks(double *f8_flops, double *bf16_flops) { return tc_peaks(f8_flops, bf16_flops); }

int gbs_ctx_dims(uint64_t M, uint64_t K, uint64_t N, uint64_t *dims) {
  if (!dims) return fail(GBS_EINVAL, "gbs_ctx_dims: dims is NULL");
  const Geometry g = reference_geometry(M, K, N);
  dims[0] = g.lhs_rows;
  dims[1] = g.rhs_rows;
  dims[2] = g.cols;
  dims[3] = g.cols;
  dims[4] = g.lhs_block;
  dims[5] = g.rhs_block;
  return GBS_OK;
}

int gbs_ctx_alloc(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB, int sA, int sB,
                  gbs_ctx **out) {
  return alloc_context(M, K, N, wA, wB, sA, sB, reference_geometry(M, K, N), out, "gbs_ctx_alloc");
}

int gbs_matrix_alloc(uint64_t nbits, uint64_t nrows, uint64_t ncols, int issigned, uint64_t rowalign,
                     uint64_t colalign, gbs_ctx **out) {
  if (rowalign < 1 || colalign < 64 || colalign % 64)
    return fail(GBS_EINVAL, "gbs_matrix_alloc: rowalign must be >= 1 and colalign a positive multiple of 64");
  Geometry g;
  g.lhs_rows = round_up(nrows, rowalign);
  g.rhs_rows = 0;
  g.cols = round_up(ncols, colalign);
  g.lhs_block = rowalign;
  g.rhs_block = 0;
  return alloc_context(nrows, ncols, 0, nbits, 1, issigned, 0, g, out, "gbs_matrix_alloc");
}

}  // extern "C"

namespace gbs {
namespace {

int alloc_context(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB, int sA, int sB, const Geometry &geo,
                  gbs_ctx **out, const char *who) {
  const std::string w(who);
  if (!out) return fail(GBS_EINVAL, w + ": out is NULL");
  *out = nullptr;
  if (wA < 1 || wA > (uint64_t)kMaxBits || wB < 1 || wB > (uint64_t)kMaxBits)
    return fail(GBS_EINVAL, w + ": bit widths must be in [1, 8], got " + std::to_string(wA) + " and " +
                                std::to_string(wB));
  if (M > (1ull << 31) || N > (1ull << 31) || K > (1ull << 31) || M * N > (1ull << 40) ||
      geo.lhs_rows > (1ull << 32) || geo.rhs_rows > (1ull << 32))
    return fail(GBS_EINVAL, w + ": shape too large");
  gbs_ctx *c = new gbs_ctx();
  if (cudaGetDevice(&c->device) != cudaSuccess) {
    delete c;
    return cuda_fail(cudaGetLastError(), (w + ": no CUDA device").c_str());
  }
  auto init = [&](Mat &m, uint64_t bits, uint64_t rows, uint64_t rows_a, int sgn) {
    m.nbits = bits;
    m.nrows = rows;
    m.ncols = K;
    m.issigned = sgn ? 1 : 0;
    m.nrows_a = rows_a;
    m.ncols_a = geo.cols;
    m.drows = round_up(rows, kRowAlign);
    m.dcols = round_up(K, kColAlign);
  };
  init(c->lhs, wA, M, geo.lhs_rows, sA);
  init(c->rhs, wB, N, geo.rhs_rows, sB);
  c->lhsBlock = geo.lhs_block;
  c->rhsBlock = geo.rhs_block;
  cudaError_t e = cudaSuccess;
  const char *what = "";
  if (e == cudaSuccess) { what = "lhs planes"; e = dev_alloc((void **)&c->lhs.planes, c->lhs.words() * 8); }
  if (e == cudaSuccess) { what = "rhs planes"; e = dev_alloc((void **)&c->rhs.planes, c->rhs.words() * 8); }
  if (e == cudaSuccess) { what = "result"; e = dev_alloc((void **)&c->res, M * N * 4); }
  if (e == cudaSuccess) { what = "row sums"; e = dev_alloc((void **)&c->rowsum, (M + N) * 4); }
  if (e != cudaSuccess) {
    cudaGetLastError();
    free_ctx_buffers(c);
    delete c;
    return fail(GBS_ENOMEM, w + ": device allocation failed (" + what + ")");
  }
  // Planes start zeroed so that a context is well defined even before import.
  cudaMemset(c->lhs.planes, 0, c->lhs.words() * 8);
  cudaMemset(c->rhs.planes, 0, c->rhs.words() * 8);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    free_ctx_buffers(c);
    delete c;
    return cuda_fail(e, who);
  }
  *out = c;
  return GBS_OK;
}

}  // namespace
}  // namespace gbs

extern "C" {

int gbs_ctx_allocate(uint64_t M, uint64_t K, uint64_t N, uint64_t wA, uint64_t wB, int sA, int sB,
                     gbs_ctx **out) {
  return gbs_ctx_alloc(M, K, N, wA, wB, sA, sB, out);
}

int gbs_ctx_free(gbs_ctx *c) {
  if (!c) return GBS_OK;
  DeviceGuard g(c->device);
  cudaDeviceSynchronize();
  free_ctx_buffers(c);
  delete c;
  return GBS_OK;
}

int gbs_ctx_get_info(const gbs_ctx *c, gbs_ctx_info *info) {
  if (!c || !info) return fail(GBS_EINVAL, "gbs_ctx_get_info: NULL argument");
  auto fill = [](const Mat &m, gbs_matrix_info &o) {
    o.nbits = m.nbits;
    o.nrows = m.nrows;
    o.ncols = m.ncols;
    o.nrows_a = m.nrows_a;
    o.ncols_a = m.ncols_a;
    o.issigned = m.issigned;
    o.isbipolar = m.bipolar() ? 1 : 0;
    o.data = m.planes;
  };
  fill(c->lhs, info->lhs);
  fill(c->rhs, info->rhs);
  info->lhsBlock = c->lhsBlock;
  info->rhsBlock = c->rhsBlock;
  info->res = c->res;
  info->pipe = effective_pipe(c);
  return GBS_OK;
}

namespace {

constexpr int kImportChunks = 8;            // at most this many copy/pack chunks per host import
constexpr size_t kImportChunkBytes = 4 << 20;

// Copy stream and events of host-source imports, created on first use.
cudaError_t ensure_import_streams(gbs_ctx *c) {
  if (c->copy_stream) return cudaSuccess;
  cudaError_t e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  for (int i = 0; i < kImportChunks && e == cudaSuccess; i++)
    e = cudaEventCreateWithFlags(&c->ev_chunk[i], cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&c->ev_packed[i], cudaEventDisableTiming);
  return e;
}

// Staging buffer of one side holding at least `bytes`.  A buffer that grows
// is freed only after the packing that reads it has finished.
int ensure_stage(gbs_ctx *c, int side, size_t bytes, cudaStream_t s) {
  if (c->stage_bytes[side] >= bytes) return GBS_OK;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && c->ev_packed_set[side]) e = cudaEventSynchronize(c->ev_packed[side]);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_import: stream sync");
  if (c->stage[side]) cudaFree(c->stage[side]);
  c->stage[side] = nullptr;
  c->stage_bytes[side] = 0;
  if (dev_alloc(&c->stage[side], bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(GBS_ENOMEM, "gbs_import: staging allocation failed");
  }
  c->stage_bytes[side] = bytes;
  return GBS_OK;
}

// The tensor-core digit pipe will run this context's GEMM: the import then
// writes the digit matrix too, so the GEMM needs no expansion pass.
bool import_writes_digits(const gbs_ctx *c) {
  return effective_pipe(c) == GBS_PIPE_TC && c->lhs.nbits <= 4 && c->rhs.nbits <= 4;  // wide operands: per part, later
}

}  // namespace

int gbs_import(gbs_ctx *c, int side, const void *src, int dtype, int col_major, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_import: ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, "gbs_import: side must be 0 (lhs) or 1 (rhs)");
  if (dtype < GBS_I8 || dtype > GBS_F32) return fail(GBS_EINVAL, "gbs_import: unknown dtype");
  Mat &m = side ? c->rhs : c->lhs;
  const uint64_t n = m.nrows * m.ncols;
  if (n && !src) return fail(GBS_EINVAL, "gbs_import: src is NULL");
  DeviceGuard g(c->device);
  if (!g.ok) return cuda_fail(cudaGetLastError(), "gbs_import: cudaSetDevice");
  cudaStream_t s = as_stream(stream);
  c->digits_valid[side] = c->nibbles_valid[side] = false;
  c->vt_valid[side] = false;
  uint8_t *digits = nullptr;
  uint32_t dtab[4] = {0, 0, 0, 0};
  if (!col_major && import_writes_digits(c)) {
    if (ensure_digit_buffer(c, side) == cudaSuccess) {
      digits = c->digits[side];
      tc_digit_table(m, dtab);
    } else {
      cudaGetLastError();  // the GEMM expands the digits itself
    }
  }
  cudaError_t e = cudaSuccess;
  const void *view = (n && !is_device_ptr(src) && c->host_import != GBS_HOST_IMPORT_STAGED)
                         ? device_view(src, c->device, true)
                         : nullptr;
  if (view) {  // host memory the device reads directly: the pack kernel is the copy
    if (!col_major) {
      e = launch_pack_rows(m, view, dtype, 0, m.nrows_a, digits, dtab, s);
      if (e == cudaSuccess && digits) c->digits_valid[side] = true;
    } else {
      e = launch_pack(m, view, dtype, 1, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: pack kernel");
    e = ensure_import_streams(c);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_packed[side], s);
    if (e == cudaSuccess) e = cudaEventSynchronize(c->ev_packed[side]);  // host memory may be reused once read
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: pack wait");
    c->ev_packed_set[side] = true;
  } else if (n && !is_device_ptr(src)) {
    const size_t esz = elem_size(dtype), bytes = n * esz;
    int rc = ensure_stage(c, side, bytes, s);
    if (rc != GBS_OK) return rc;
    e = ensure_import_streams(c);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: stream/event creation");
    // the copy overwrites the staging buffer only after the last packing that read it
    if (c->ev_packed_set[side]) e = cudaStreamWaitEvent(c->copy_stream, c->ev_packed[side], 0);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: stream wait");
    if (col_major) {  // one copy, then the column-major pack
      e = cudaMemcpyAsync(c->stage[side], src, bytes, cudaMemcpyHostToDevice, c->copy_stream);
      if (e == cudaSuccess) e = cudaEventRecord(c->ev_chunk[0], c->copy_stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_chunk[0], 0);
      if (e != cudaSuccess) return cuda_fail(e, "gbs_import: host-to-device copy");
      e = launch_pack(m, c->stage[side], dtype, 1, s);
      if (e != cudaSuccess) return cuda_fail(e, "gbs_import: pack kernel");
    } else {  // row chunks: the pack of chunk i overlaps the copy of chunk i+1
      const size_t row_bytes = m.ncols * esz;
      const uint64_t chunks = std::max<uint64_t>(1, std::min<uint64_t>(kImportChunks, bytes / kImportChunkBytes));
      const uint64_t rows_per = (m.nrows + chunks - 1) / chunks;
      int last = 0;
      for (uint64_t i = 0; i < chunks; i++) {
        const uint64_t r0 = i * rows_per, r1 = std::min(m.nrows, r0 + rows_per);
        if (r0 >= r1) break;
        const size_t off = r0 * row_bytes;
        e = cudaMemcpyAsync((char *)c->stage[side] + off, (const char *)src + off, (r1 - r0) * row_bytes,
                            cudaMemcpyHostToDevice, c->copy_stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_chunk[i], c->copy_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_chunk[i], 0);
        if (e != cudaSuccess) return cuda_fail(e, "gbs_import: host-to-device copy");
        // the last chunk also writes the zero padding rows [nrows, nrows_a)
        e = launch_pack_rows(m, c->stage[side], dtype, r0, r1 == m.nrows ? m.nrows_a : r1, digits, dtab, s);
        if (e != cudaSuccess) return cuda_fail(e, "gbs_import: pack kernel");
        last = (int)i;
      }
      if (digits) c->digits_valid[side] = true;
      e = cudaEventSynchronize(c->ev_chunk[last]);  // host memory may be reused once copied
      if (e != cudaSuccess) return cuda_fail(e, "gbs_import: copy wait");
    }
    e = cudaEventRecord(c->ev_packed[side], s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: event record");
    c->ev_packed_set[side] = true;
    if (col_major) {
      e = cudaEventSynchronize(c->ev_chunk[0]);
      if (e != cudaSuccess) return cuda_fail(e, "gbs_import: copy wait");
    }
  } else if (!col_major) {
    e = launch_pack_rows(m, src, dtype, 0, m.nrows_a, digits, dtab, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: pack kernel");
    if (digits) c->digits_valid[side] = true;
  } else {
    e = launch_pack(m, src, dtype, 1, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import: pack kernel");
  }
  m.imported = true;
  return GBS_OK;
}

int gbs_import_quantize(gbs_ctx *c, int side, const void *src, const void *thresholds, int nthres, int dtype,
                        int col_major, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_import_quantize: ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, "gbs_import_quantize: side must be 0 or 1");
  if (dtype < GBS_I8 || dtype > GBS_F32) return fail(GBS_EINVAL, "gbs_import_quantize: unknown dtype");
  Mat &m = side ? c->rhs : c->lhs;
  if (m.issigned)
    return fail(GBS_EINVAL, "gbs_import_quantize: threshold quantization needs an unsigned matrix");
  if (nthres < 0) return fail(GBS_EINVAL, "gbs_import_quantize: nthres must be >= 0");
  const uint64_t n = m.nrows * m.ncols;
  const size_t esz = dtype == GBS_I16 ? 2 : (dtype == GBS_I32 || dtype == GBS_F32) ? 4 : 1;
  const size_t tbytes = (size_t)nthres * m.nrows * esz;
  if ((n && !src) || (tbytes && !thresholds)) return fail(GBS_EINVAL, "gbs_import_quantize: NULL pointer");
  DeviceGuard g(c->device);
  if (!g.ok) return cuda_fail(cudaGetLastError(), "gbs_import_quantize: cudaSetDevice");
  cudaStream_t s = as_stream(stream);
  c->digits_valid[side] = c->nibbles_valid[side] = false;
  c->vt_valid[side] = false;
  uint8_t *digits = nullptr;
  uint32_t dtab[4] = {0, 0, 0, 0};
  if (import_writes_digits(c)) {
    if (ensure_digit_buffer(c, side) == cudaSuccess) {
      digits = c->digits[side];
      tc_digit_table(m, dtab);
    } else {
      cudaGetLastError();  // the GEMM expands the digits itself
    }
  }
  bool host = false;
  const void *dsrc = src, *dthr = thresholds;
  cudaError_t e = cudaSuccess;
  if (n && !is_device_ptr(src)) {
    int rc = ensure_stage(c, side, n * esz, s);
    if (rc != GBS_OK) return rc;
    if (c->ev_packed_set[side]) e = cudaStreamWaitEvent(s, c->ev_packed[side], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->stage[side], src, n * esz, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import_quantize: host-to-device copy");
    dsrc = c->stage[side];
    host = true;
  }
  if (tbytes && !is_device_ptr(thresholds)) {
    if (c->thr_bytes[side] < tbytes) {
      e = cudaStreamSynchronize(s);  // the old buffer may still be read
      if (e != cudaSuccess) return cuda_fail(e, "gbs_import_quantize: stream sync");
      if (c->thr_stage[side]) cudaFree(c->thr_stage[side]);
      c->thr_stage[side] = nullptr;
      c->thr_bytes[side] = 0;
      if (dev_alloc(&c->thr_stage[side], tbytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(GBS_ENOMEM, "gbs_import_quantize: threshold buffer allocation failed");
      }
      c->thr_bytes[side] = tbytes;
    }
    e = cudaMemcpyAsync(c->thr_stage[side], thresholds, tbytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import_quantize: threshold copy");
    dthr = c->thr_stage[side];
    host = true;
  }
  e = launch_pack_quantize(m, dsrc, dthr, nthres, dtype, col_major ? 1 : 0, digits, dtab, s);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_import_quantize: pack kernel");
  if (host && dsrc == c->stage[side]) {  // later host imports of this side wait before reusing the staging buffer
    e = ensure_import_streams(c);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_packed[side], s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import_quantize: event record");
    c->ev_packed_set[side] = true;
  }
  if (digits) c->digits_valid[side] = true;
  m.imported = true;
  if (host) {  // host memory may be reused on return
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_import_quantize: stream sync");
  }
  return GBS_OK;
}

namespace {

// The device word holding (bit, row, col) of one side, after bounds checks.
int bit_word(gbs_ctx *c, int side, uint64_t bit, uint64_t row, uint64_t col, uint64_t **word, const char *who) {
  if (!c) return fail(GBS_EINVAL, std::string(who) + ": ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, std::string(who) + ": bad side");
  const Mat &m = side ? c->rhs : c->lhs;
  if (bit >= m.nbits || row >= m.nrows_a || col >= m.ncols_a)
    return fail(GBS_EINVAL, std::string(who) + ": bit, row or column out of range");
  *word = m.planes + bit * m.nrows_a * m.wpr() + row * m.wpr() + (col >> 6);
  return GBS_OK;
}

}  // namespace

int gbs_get_bit(gbs_ctx *c, int side, uint64_t bit, uint64_t row, uint64_t col, int *value) {
  uint64_t *w = nullptr;
  int rc = bit_word(c, side, bit, row, col, &w, "gbs_get_bit");
  if (rc != GBS_OK) return rc;
  if (!value) return fail(GBS_EINVAL, "gbs_get_bit: value is NULL");
  DeviceGuard g(c->device);
  uint64_t v = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_get_bit");
  *value = (int)((v >> (col & 63)) & 1u);
  return GBS_OK;
}

int gbs_set_bit(gbs_ctx *c, int side, uint64_t bit, uint64_t row, uint64_t col, int value) {
  uint64_t *w = nullptr;
  int rc = bit_word(c, side, bit, row, col, &w, "gbs_set_bit");
  if (rc != GBS_OK) return rc;
  const Mat &mm = side ? c->rhs : c->lhs;
  if (row >= mm.nrows || col >= mm.ncols)  // padding stays zero: results never depend on it
    return fail(GBS_EINVAL, "gbs_set_bit: row or column in the padding");
  DeviceGuard g(c->device);
  uint64_t v = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) {
    const uint64_t mask = (uint64_t)1 << (col & 63);
    v = value ? (v | mask) : (v & ~mask);
    e = cudaMemcpy(w, &v, sizeof(v), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return cuda_fail(e, "gbs_set_bit");
  Mat &m = side ? c->rhs : c->lhs;
  m.imported = true;
  c->digits_valid[side] = c->nibbles_valid[side] = false;  // derived operands no longer match the planes
  c->vt_valid[side] = false;
  return GBS_OK;
}

int gbs_get_word(gbs_ctx *c, int side, uint64_t bit, uint64_t row, uint64_t col, uint64_t *value) {
  uint64_t *w = nullptr;
  int rc = bit_word(c, side, bit, row, col, &w, "gbs_get_word");
  if (rc != GBS_OK) return rc;
  if (!value) return fail(GBS_EINVAL, "gbs_get_word: value is NULL");
  DeviceGuard g(c->device);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(value, w, sizeof(uint64_t), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? GBS_OK : cuda_fail(e, "gbs_get_word");
}

int gbs_set_word(gbs_ctx *c, int side, uint64_t bit, uint64_t row, uint64_t col, uint64_t value) {
  uint64_t *w = nullptr;
  int rc = bit_word(c, side, bit, row, col, &w, "gbs_set_word");
  if (rc != GBS_OK) return rc;
  Mat &m = side ? c->rhs : c->lhs;
  // padding stays zero (results never depend on it): rows past nrows take no
  // bits, and a word's columns past ncols are cleared
  const uint64_t c0 = col & ~(uint64_t)63;
  if (row >= m.nrows || c0 >= m.ncols) value = 0;
  else if (m.ncols - c0 < 64) value &= ((uint64_t)1 << (m.ncols - c0)) - 1;
  DeviceGuard g(c->device);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(w, &value, sizeof(uint64_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_set_word");
  m.imported = true;
  c->digits_valid[side] = c->nibbles_valid[side] = false;  // derived operands no longer match the planes
  c->vt_valid[side] = false;
  return GBS_OK;
}

int gbs_clear(gbs_ctx *c, int side, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_clear: ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, "gbs_clear: bad side");
  Mat &m = side ? c->rhs : c->lhs;
  DeviceGuard g(c->device);
  if (m.words()) {
    cudaError_t e = cudaMemsetAsync(m.planes, 0, m.words() * 8, as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "gbs_clear");
  }
  m.imported = true;
  c->digits_valid[side] = c->nibbles_valid[side] = false;
  c->vt_valid[side] = false;
  return GBS_OK;
}

int gbs_set_variant(gbs_ctx *c, int variant) {
  if (!c) return fail(GBS_EINVAL, "gbs_set_variant: ctx is NULL");
  if (!(variant == -1 || (variant >= 0 && variant <= 2) || variant == kRowsCls || variant == 128 || variant == 256 ||
        variant == kPairVariant ||
        variant == kPairVariant128 || variant == kPairVariantPersistent || variant == kPairVariantStreamK ||
        pair_split_variant(variant)))
    return fail(GBS_EINVAL,
                "gbs_set_variant: variant must be -1, 0..2, 4, 128, 256, 512..515, 1281, 1282, 1284, 2561, 2562 or 2564");
  c->variant = variant;
  return GBS_OK;
}

int gbs_set_host_import(gbs_ctx *c, int mode) {
  if (!c) return fail(GBS_EINVAL, "gbs_set_host_import: ctx is NULL");
  if (mode != GBS_HOST_IMPORT_AUTO && mode != GBS_HOST_IMPORT_STAGED)
    return fail(GBS_EINVAL, "gbs_set_host_import: mode must be GBS_HOST_IMPORT_AUTO or GBS_HOST_IMPORT_STAGED");
  c->host_import = mode;
  return GBS_OK;
}

int gbs_set_pipe(gbs_ctx *c, int pipe) {
  if (!c) return fail(GBS_EINVAL, "gbs_set_pipe: ctx is NULL");
  if (pipe < GBS_PIPE_AUTO || pipe > GBS_PIPE_TC_SMEM) return fail(GBS_EINVAL, "gbs_set_pipe: unknown pipe");
  c->pipe = pipe;
  return GBS_OK;
}

int gbs_gemm(gbs_ctx *c, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_gemm: ctx is NULL");
  if (c->lhs.ncols != c->rhs.ncols) return fail(GBS_EINVAL, "gbs_gemm: lhs/rhs depth mismatch");
  if (!c->lhs.imported || !c->rhs.imported)
    return fail(GBS_ESTATE, "gbs_gemm: import both lhs and rhs before gemm");
  DeviceGuard g(c->device);
  if (!g.ok) return cuda_fail(cudaGetLastError(), "gbs_gemm: cudaSetDevice");
  cudaStream_t s = as_stream(stream);
  const uint64_t M = c->lhs.nrows, N = c->rhs.nrows;
  if (M == 0 || N == 0) return GBS_OK;
  const int pipe = effective_pipe(c);
  const bool tensor_core = pipe == GBS_PIPE_TC || pipe == GBS_PIPE_TC_PAIRS || pipe == GBS_PIPE_TC_SMEM;
  Epilogue e;
  make_epilogue(c, e, c->rowsum);
  if ((e.ra || e.rb) && !tensor_core) {  // the tensor-core pipes take bipolar values directly
    const Mat &reg = c->lhs.bipolar() ? c->rhs : c->lhs;
    cudaError_t re = launch_rowsum(reg, c->rowsum, s);
    if (re != cudaSuccess) return cuda_fail(re, "gbs_gemm: row-sum kernel");
  }
  GemmShape sh;
  sh.A = c->lhs.planes;
  sh.B = c->rhs.planes;
  sh.C = result_ptr(c);
  sh.M = M;
  sh.N = N;
  sh.wpr = c->lhs.wpr();
  sh.a_plane = c->lhs.nrows_a * sh.wpr;
  sh.b_plane = c->rhs.nrows_a * sh.wpr;
  sh.a_rows = c->lhs.nrows_a;
  sh.b_rows = c->rhs.nrows_a;
  sh.wa = (int)c->lhs.nbits;
  sh.wb = (int)c->rhs.nbits;
  const int variant = c->variant >= 0 ? c->variant : (c->pipe == GBS_PIPE_AUTO ? tuned_variant(c, pipe) : -1);
  sh.tile_cls = (pipe == GBS_PIPE_POPC && ((variant >= 0 && variant <= 2) || (variant == kRowsCls && M <= kRowsMaxM)))
                    ? variant
                    : -1;
  cudaError_t ke;
  if (pipe == GBS_PIPE_TC && tc_wide(c)) {
    ke = launch_gemm_wide(c, s, variant);
  } else if (pipe == GBS_PIPE_TC) {
    ke = launch_gemm_tc_hbm(c, s, variant);
  } else if (pipe == GBS_PIPE_TC_PAIRS || pipe == GBS_PIPE_TC_SMEM) {
    ke = launch_gemm_tc(c, s, pipe == GBS_PIPE_TC_SMEM, variant);
  } else if (pipe == GBS_PIPE_BMMA && bmma_supported(sh.wa, sh.wb, e.use_xor) && sh.wpr % 2 == 0) {
    // (b1 MMA tiles load 16-byte pieces of plane rows: an odd word count runs on the CUDA cores)
    if (e.use_xor) {
      // ncols - 2*popc(a^b) = 4*popc(a&b) - rsA - rsB - ncols, rs = bipolar row sums (2*popc - ncols)
      e.use_xor = 0;
      e.alpha[0][0] = 4;
      e.c0 = 0u - (uint32_t)c->lhs.ncols;
      e.ra = c->rowsum;
      e.rb = c->rowsum + M;
      cudaError_t re = launch_rowsum(c->lhs, c->rowsum, s);
      if (re == cudaSuccess) re = launch_rowsum(c->rhs, c->rowsum + M, s);
      if (re != cudaSuccess) return cuda_fail(re, "gbs_gemm: row-sum kernel");
    }
    ke = launch_gemm_bmma(sh, e, s);
  } else {
    ke = launch_gemm_popc(sh, e, s);
  }
  if (ke != cudaSuccess) return cuda_fail(ke, "gbs_gemm: forward kernel");
  if (!c->out) c->res_stale = false;
  return GBS_OK;
}

int gbs_gemm_to(gbs_ctx *c, int32_t *dst, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_gemm_to: ctx is NULL");
  const uint64_t n = c->lhs.nrows * c->rhs.nrows;
  if (n == 0) return gbs_gemm(c, stream);
  if (!dst) return fail(GBS_EINVAL, "gbs_gemm_to: dst is NULL");
  DeviceGuard g(c->device);
  if (!g.ok) return cuda_fail(cudaGetLastError(), "gbs_gemm_to: cudaSetDevice");
  cudaStream_t s = as_stream(stream);
  const bool host = !is_device_ptr(dst);
  // The epilogues store 16-byte vectors where rows allow: direct writes need an
  // aligned buffer.  Pageable destinations take the copy: the copy engine
  // writes them faster than the kernels' stores through the host page tables.
  int32_t *view =
      ((uintptr_t)dst % 16 == 0) ? static_cast<int32_t *>(device_view(dst, c->device, false)) : nullptr;
  if (!view) {  // the device cannot write dst: compute into res, then copy
    int rc = gbs_gemm(c, stream);
    return rc != GBS_OK ? rc : gbs_get_result(c, dst, stream);
  }
  c->out = view;
  const int rc = gbs_gemm(c, stream);
  c->out = nullptr;
  if (rc != GBS_OK) return rc;
  c->res_stale = true;
  if (host) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_gemm_to: stream sync");
  }
  return GBS_OK;
}

int gbs_get_result(gbs_ctx *c, int32_t *dst, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_get_result: ctx is NULL");
  const uint64_t n = c->lhs.nrows * c->rhs.nrows;
  if (n == 0) return GBS_OK;
  if (!dst) return fail(GBS_EINVAL, "gbs_get_result: dst is NULL");
  if (c->res_stale)
    return fail(GBS_ESTATE, "gbs_get_result: the last GEMM wrote its result to the caller's buffer (gbs_gemm_to)");
  DeviceGuard g(c->device);
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(dst, c->res, n * 4, cudaMemcpyDefault, s);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_get_result: copy");
  if (!is_device_ptr(dst)) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_get_result: stream sync");
  }
  return GBS_OK;
}

int gbs_get_planes(gbs_ctx *c, int side, uint64_t *dst, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_get_planes: ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, "gbs_get_planes: bad side");
  const Mat &m = side ? c->rhs : c->lhs;
  if (m.words() == 0) return GBS_OK;
  if (!dst) return fail(GBS_EINVAL, "gbs_get_planes: dst is NULL");
  DeviceGuard g(c->device);
  cudaStream_t s = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(dst, m.planes, m.words() * 8, cudaMemcpyDefault, s);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_get_planes: copy");
  if (!is_device_ptr(dst)) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_get_planes: stream sync");
  }
  return GBS_OK;
}

static int to_dst(int32_t *dst, uint64_t n, cudaStream_t s,
                  cudaError_t (*fill)(const Mat &, int32_t *, cudaStream_t), const Mat &m, const char *who) {
  if (n == 0) return GBS_OK;
  if (!dst) return fail(GBS_EINVAL, std::string(who) + ": dst is NULL");
  if (is_device_ptr(dst)) {
    cudaError_t e = fill(m, dst, s);
    return e == cudaSuccess ? GBS_OK : cuda_fail(e, who);
  }
  int32_t *tmp = nullptr;
  if (dev_alloc((void **)&tmp, n * 4) != cudaSuccess) {
    cudaGetLastError();
    return fail(GBS_ENOMEM, std::string(who) + ": temporary allocation failed");
  }
  cudaError_t e = fill(m, tmp, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst, tmp, n * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(tmp);
  return e == cudaSuccess ? GBS_OK : cuda_fail(e, who);
}

int gbs_sum_rows(gbs_ctx *c, int side, int32_t *dst, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_sum_rows: ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, "gbs_sum_rows: bad side");
  DeviceGuard g(c->device);
  const Mat &m = side ? c->rhs : c->lhs;
  return to_dst(dst, m.nrows, as_stream(stream), launch_rowsum, m, "gbs_sum_rows");
}

int gbs_export(gbs_ctx *c, int side, int32_t *dst, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_export: ctx is NULL");
  if (side != GBS_LHS && side != GBS_RHS) return fail(GBS_EINVAL, "gbs_export: bad side");
  DeviceGuard g(c->device);
  const Mat &m = side ? c->rhs : c->lhs;
  return to_dst(dst, m.nrows * m.ncols, as_stream(stream), launch_export, m, "gbs_export");
}

}  // extern "C"
