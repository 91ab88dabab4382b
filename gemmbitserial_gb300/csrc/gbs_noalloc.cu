// gbs_noalloc.cu -- a one-shot bit-serial GEMM that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc: code that runs while a
// stream is being captured into a CUDA graph in global capture mode (where an
// allocation invalidates the capture), real-time loops that must not take the
// allocator's locks or synchronisation, and hosts that give the library a
// fixed memory budget up front.  gbs_gemm_noalloc serves them: the caller
// passes device inputs and a device output, and every intermediate (the
// packed bit planes of both operands and the row sums of the bipolar x regular
// correction) lives in g_noalloc_scratch, a file-scope device array of fixed
// size that every GPU loading the library holds until the process exits.
//
// The array's host-side name is only a stand-in for the symbol, so host code
// never passes it to a kernel: the first call on each device looks up its
// device address with cudaGetSymbolAddress (with that device current) and
// caches it.  That first call should therefore come before any stream capture.
//
// All calls share the one array and it keeps the last call's contents.  The
// pack kernels write every plane word the GEMM reads (padding included) and
// the row-sum kernel writes every row sum it reads, so nothing has to start
// at zero.  Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array: order them on one stream.
#include <mutex>

#include "gbs_internal.h"

namespace gbs {
namespace {

// 16 MiB: enough for the packed planes of e.g. a 2048 x 4096 x 2048 GEMM of
// 3-bit x 2-bit operands (5 MiB) or 4096 x 4096 x 4096 at 2 x 2 bits (8 MiB).
constexpr uint64_t kScratchWords = 2ull << 20;
static __device__ __align__(256) uint64_t g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
uint64_t *g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

int scratch_address(int dev, uint64_t **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (dev < 0 || dev >= kMaxDevices) return fail(GBS_EUNSUPPORTED, "gbs_gemm_noalloc: device index out of range");
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_gemm_noalloc: cudaGetSymbolAddress");
    g_scratch_addr[dev] = static_cast<uint64_t *>(p);
  }
  *out = g_scratch_addr[dev];
  return GBS_OK;
}

// True when the kernels launched on device `dev` may address `p` directly:
// managed memory, or device memory of `dev` itself.  Another GPU's memory is
// refused (reading it without peer access faults), and so is host memory.
bool on_device(const void *p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}

uint64_t round_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" uint64_t gbs_noalloc_scratch_bytes(void) { return kScratchWords * sizeof(uint64_t); }

extern "C" int gbs_gemm_noalloc(const void *lhs, int lhs_dtype, const void *rhs, int rhs_dtype, uint64_t M,
                                uint64_t K, uint64_t N, uint64_t lhsBits, uint64_t rhsBits, int lhsSigned,
                                int rhsSigned, int32_t *res, void *stream) {
  if (lhsBits < 1 || lhsBits > (uint64_t)kMaxBits || rhsBits < 1 || rhsBits > (uint64_t)kMaxBits)
    return fail(GBS_EINVAL, "gbs_gemm_noalloc: bit widths must be in [1, 8]");
  if (lhs_dtype < GBS_I8 || lhs_dtype > GBS_F32 || rhs_dtype < GBS_I8 || rhs_dtype > GBS_F32)
    return fail(GBS_EINVAL, "gbs_gemm_noalloc: unknown dtype");
  if (M > (1ull << 31) || N > (1ull << 31) || K > (1ull << 31))
    return fail(GBS_EINVAL, "gbs_gemm_noalloc: shape too large");
  if (M == 0 || N == 0) return GBS_OK;
  // The whole working set must fit the fixed array: planes of both operands
  // (rows padded to 256, columns to 256 bits) plus M + N int32 row sums.
  gbs_ctx c;  // describes the operands; owns nothing
  auto init = [&](Mat &m, uint64_t bits, uint64_t rows, int sgn) {
    m.nbits = bits;
    m.nrows = rows;
    m.ncols = K;
    m.issigned = sgn ? 1 : 0;
    m.nrows_a = round_up(rows, kRowAlign);
    m.ncols_a = round_up(K, kColAlign);
    m.drows = m.nrows_a;
    m.dcols = m.ncols_a;
    m.imported = true;
  };
  init(c.lhs, lhsBits, M, lhsSigned);
  init(c.rhs, rhsBits, N, rhsSigned);
  const uint64_t need_words = c.lhs.words() + c.rhs.words() + (M + N + 1) / 2;
  if (need_words > kScratchWords)
    return fail(GBS_EINVAL, "gbs_gemm_noalloc: this GEMM needs " + std::to_string(need_words * 8) +
                                " bytes of scratch; the fixed array holds " + std::to_string(kScratchWords * 8));
  if ((K && (!lhs || !rhs)) || !res) return fail(GBS_EINVAL, "gbs_gemm_noalloc: NULL pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_gemm_noalloc: cudaGetDevice");
  if ((K && (!on_device(lhs, dev) || !on_device(rhs, dev))) || !on_device(res, dev))
    return fail(GBS_EINVAL, "gbs_gemm_noalloc: inputs and result must be memory of the current device");
  uint64_t *scratch = nullptr;
  int rc = scratch_address(dev, &scratch);
  if (rc != GBS_OK) return rc;
  c.device = dev;
  c.lhs.planes = scratch;
  c.rhs.planes = scratch + c.lhs.words();
  c.rowsum = reinterpret_cast<int32_t *>(scratch + c.lhs.words() + c.rhs.words());
  c.res = res;
  cudaStream_t s = (cudaStream_t)stream;

  e = launch_pack(c.lhs, lhs, lhs_dtype, 0, s);
  if (e == cudaSuccess) e = launch_pack(c.rhs, rhs, rhs_dtype, 0, s);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_gemm_noalloc: pack kernel");
  Epilogue ep;
  make_epilogue(&c, ep, c.rowsum);
  if (ep.ra || ep.rb) {
    e = launch_rowsum(c.lhs.bipolar() ? c.rhs : c.lhs, c.rowsum, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_gemm_noalloc: row-sum kernel");
  }
  GemmShape sh;
  sh.A = c.lhs.planes;
  sh.B = c.rhs.planes;
  sh.C = res;
  sh.M = M;
  sh.N = N;
  sh.wpr = c.lhs.wpr();
  sh.a_plane = c.lhs.nrows_a * sh.wpr;
  sh.b_plane = c.rhs.nrows_a * sh.wpr;
  sh.a_rows = c.lhs.nrows_a;
  sh.b_rows = c.rhs.nrows_a;
  sh.wa = (int)lhsBits;
  sh.wb = (int)rhsBits;
  sh.tile_cls = -1;
  e = launch_gemm_popc(sh, ep, s);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_gemm_noalloc: forward kernel");
  return GBS_OK;
}
