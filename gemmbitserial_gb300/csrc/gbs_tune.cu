// gbs_tune.cu -- pipe peaks and the per-shape pipe choice.
//
// gbs_pipe_peaks measures, on the current device, the sustained rate of the
// two pipes the forward GEMM can use, in AND+popcount bit operations per
// second (one bit of one plane pair of one output):
//   * POPC: a shared-memory-fed 4x4 register tile of popc(a & b) over 64-bit
//     words, the inner loop of the CUDA-core kernel;
//   * BMMA: back-to-back mma.sync.m16n8k256 b1 AND.popc with independent
//     accumulators.
// Both loops run on every SM (4 CTAs of 256 threads each) for ~10-20 ms.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "gbs_internal.h"

namespace gbs {
namespace {

__global__ void __launch_bounds__(256) peak_popc(const uint64_t *in, int *out, int iters) {
  __shared__ uint64_t sa[64 * 16], sb[64 * 16];
  for (int i = threadIdx.x; i < 64 * 16; i += blockDim.x) {
    sa[i] = in[i & 1023];
    sb[i] = in[(i * 7) & 1023];
  }
  __syncthreads();
  uint32_t acc[4][4] = {};
  const int tm = threadIdx.x & 15, tn = threadIdx.x >> 4;
  for (int it = 0; it < iters; it++) {
#pragma unroll 4
    for (int k = 0; k < 64; k++) {
      uint64_t a[4], b[4];
#pragma unroll
      for (int m = 0; m < 4; m++) a[m] = sa[k * 16 + ((tm + m) & 15)];
#pragma unroll
      for (int n = 0; n < 4; n++) b[n] = sb[k * 16 + ((tn + n) & 15)];
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int n = 0; n < 4; n++) acc[m][n] += __popcll(a[m] & b[n]);
    }
  }
  uint32_t s = 0;
  for (int m = 0; m < 4; m++)
    for (int n = 0; n < 4; n++) s += acc[m][n];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (int)s;
}

__global__ void __launch_bounds__(256) peak_bmma(const uint64_t *in64, int *out, int iters) {
  const uint32_t *in = reinterpret_cast<const uint32_t *>(in64);
  const int t = threadIdx.x;
  uint32_t a0 = in[t & 127], a1 = in[(t + 1) & 127], a2 = in[(t + 2) & 127], a3 = in[(t + 3) & 127];
  uint32_t b0 = in[(t + 4) & 127], b1 = in[(t + 5) & 127];
  int c[4][4] = {};
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 4; j++)
      asm volatile(
          "mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.and.popc {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
          "{%0,%1,%2,%3};"
          : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  int s = 0;
  for (int j = 0; j < 4; j++) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[blockIdx.x * blockDim.x + t] = s;
}

// 8 independent FMA chains per thread, all SMs busy.
__global__ void __launch_bounds__(256) peak_fma(const float *in, float *out, int iters) {
  float x[8];
#pragma unroll
  for (int j = 0; j < 8; j++) x[j] = in[(threadIdx.x + j) & 255];
  const float a = in[1] * 1e-3f, b = in[2] * 1e-3f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = fmaf(x[j], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; j++) s += x[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

namespace {

// ---------------------------------------------------------------- tuner store
// Key: shape class (log4 buckets of M, N and K, capped), widths and encodings
// (0 unsigned, 1 signed, 2 bipolar).  Value: the fastest pipe and variant
// measured by gbs_tune on this device.
constexpr const char *kStoreVersion = "gbs-tuner v1 sm_103a";

typedef std::tuple<int, int, int, int, int, int, int> TuneKey;
struct TuneChoice {
  int pipe, variant;
  double us;
};
std::map<TuneKey, TuneChoice> g_store;
std::mutex g_store_mu;
bool g_env_loaded = false;

int bucket(uint64_t x) {
  int b = 0;
  while (x >= 4 && b < 8) {
    x >>= 2;
    b++;
  }
  return b;
}
int enc_of(const Mat &m) { return m.bipolar() ? 2 : (m.issigned ? 1 : 0); }

TuneKey key_of(const gbs_ctx *c) {
  return TuneKey(bucket(c->lhs.nrows), bucket(c->rhs.nrows), bucket(c->lhs.ncols), (int)c->lhs.nbits,
                 (int)c->rhs.nbits, enc_of(c->lhs), enc_of(c->rhs));
}

int load_store(const char *path, bool replace);

void load_env_store() {
  if (g_env_loaded) return;
  g_env_loaded = true;
  const char *p = getenv("GBS_TUNER_STORE");
  if (p && *p) load_store(p, false);
}

}  // namespace

// Measured on GB300: the CUDA-core POPC pipe sustains ~160 T bit-op/s and the
// b1 mma.sync pipe about half that (gbs_pipe_peaks), while tcgen05 e4m3
// multiply-adds run at ~1.75 P/s (gbs_tc_peaks).  Without a tuner entry,
// every shape the tensor-core pipe covers exactly goes there; the rest
// (8-bit widths, more than 5 planes, K beyond the fp32-exact bound, skinny
// shapes) use the CUDA cores.  A tuner entry for the shape class wins when
// its pipe applies to this context.
int choose_pipe(const gbs_ctx *c) {
  {
    std::lock_guard<std::mutex> lock(g_store_mu);
    load_env_store();
    auto it = g_store.find(key_of(c));
    if (it != g_store.end()) {
      const int p = it->second.pipe;
      if (p == GBS_PIPE_POPC || p == GBS_PIPE_BMMA) return p;
      if ((p == GBS_PIPE_TC || p == GBS_PIPE_TC_PAIRS || p == GBS_PIPE_TC_SMEM) && tc_exact(c, p)) return p;
      if (p == GBS_PIPE_TC && tc_wide(c)) return p;
    }
  }
  return ((tc_exact(c, GBS_PIPE_TC) || tc_wide(c)) && tcg_preferred(c)) ? GBS_PIPE_TC : GBS_PIPE_POPC;
}

int tuned_variant(const gbs_ctx *c, int pipe) {
  std::lock_guard<std::mutex> lock(g_store_mu);
  auto it = g_store.find(key_of(c));
  return (it != g_store.end() && it->second.pipe == pipe) ? it->second.variant : -1;
}

namespace {

int load_store(const char *path, bool replace) {
  FILE *f = fopen(path, "r");
  if (!f) return fail(GBS_EINVAL, std::string("gbs_tuner_load: cannot open ") + path);
  char line[256];
  if (!fgets(line, sizeof(line), f) || strncmp(line, kStoreVersion, strlen(kStoreVersion)) != 0) {
    fclose(f);
    return fail(GBS_EINVAL, "gbs_tuner_load: store written by another version; entries ignored");
  }
  std::map<TuneKey, TuneChoice> fresh;
  int n = 0;
  while (fgets(line, sizeof(line), f)) {
    int k[7], pipe, variant;
    double us;
    if (sscanf(line, "%d %d %d %d %d %d %d %d %d %lf", &k[0], &k[1], &k[2], &k[3], &k[4], &k[5], &k[6], &pipe,
               &variant, &us) != 10)
      continue;
    if (pipe < GBS_PIPE_POPC || pipe > GBS_PIPE_TC_SMEM) continue;
    fresh[TuneKey(k[0], k[1], k[2], k[3], k[4], k[5], k[6])] = TuneChoice{pipe, variant, us};
    n++;
  }
  fclose(f);
  if (replace) g_store.clear();
  for (auto &kv : fresh) g_store[kv.first] = kv.second;
  return GBS_OK;
}

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" int gbs_pipe_peaks(double *popc_bitops, double *bmma_bitops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "gbs_pipe_peaks: no device");
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  uint64_t *in = nullptr;
  int *out = nullptr;
  const int blocks = sms * 4, threads = 256;
  if (dev_alloc((void **)&in, 1024 * 8) != cudaSuccess || dev_alloc((void **)&out, blocks * threads * 4) != cudaSuccess) {
    cudaGetLastError();
    if (in) cudaFree(in);
    return fail(GBS_ENOMEM, "gbs_pipe_peaks: allocation failed");
  }
  uint64_t h[1024];
  for (int i = 0; i < 1024; i++) h[i] = 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
  cudaMemcpy(in, h, sizeof(h), cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto timed = [&](auto launch) {
    launch(4);
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
      cudaEventRecord(e0);
      launch(0);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) best = ms;
    }
    return (double)best * 1e-3;
  };
  const int it_popc = 48, it_bmma = 2048;
  double tp = timed([&](int small) { peak_popc<<<blocks, threads>>>(in, out, small ? small : it_popc); });
  double tb = timed([&](int small) { peak_bmma<<<blocks, threads>>>(in, out, small ? small : it_bmma); });
  count_launch(8);
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(in);
  cudaFree(out);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_pipe_peaks");
  const double warps = (double)blocks * threads / 32.0;
  if (popc_bitops) *popc_bitops = warps * 32.0 * it_popc * 64.0 * 16.0 * 64.0 / tp;
  if (bmma_bitops) *bmma_bitops = warps * it_bmma * 4.0 * 16.0 * 8.0 * 256.0 / tb;
  return GBS_OK;
}

extern "C" int gbs_fma_peak(double *flops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "gbs_fma_peak: no device");
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 8192;
  float *in = nullptr, *out = nullptr;
  if (dev_alloc((void **)&in, 256 * 4) != cudaSuccess || dev_alloc((void **)&out, blocks * threads * 4) != cudaSuccess) {
    cudaGetLastError();
    if (in) cudaFree(in);
    return fail(GBS_ENOMEM, "gbs_fma_peak: allocation failed");
  }
  float h[256];
  for (int i = 0; i < 256; i++) h[i] = 1.0f + 0.001f * (float)i;
  cudaMemcpy(in, h, sizeof(h), cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  peak_fma<<<blocks, threads>>>(in, out, 16);
  cudaDeviceSynchronize();
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0);
    peak_fma<<<blocks, threads>>>(in, out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  count_launch(4);
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(in);
  cudaFree(out);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_fma_peak");
  if (flops) *flops = 2.0 * blocks * threads * (double)iters * 8.0 / (best * 1e-3);
  return GBS_OK;
}

extern "C" int gbs_tune(gbs_ctx *c, int reps, int *best_pipe, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_tune: ctx is NULL");
  if (!c->lhs.imported || !c->rhs.imported) return fail(GBS_ESTATE, "gbs_tune: import both operands first");
  if (reps < 1) reps = 3;
  cudaStream_t s = (cudaStream_t)stream;
  struct Cand {
    int pipe, variant;
  };
  Cand cands[24];
  int nc = 0;
  for (int v = -1; v <= 2; v++) cands[nc++] = Cand{GBS_PIPE_POPC, v};  // -1: built-in tile rule
  if (c->lhs.nrows <= (uint64_t)kRowsMaxM) cands[nc++] = Cand{GBS_PIPE_POPC, kRowsCls};
  cands[nc++] = Cand{GBS_PIPE_BMMA, -1};
  if (tc_wide(c)) cands[nc++] = Cand{GBS_PIPE_TC, -1};  // 5-8-bit operands: part products on the digit pipe
  if (tc_exact(c, GBS_PIPE_TC)) {
    cands[nc++] = Cand{GBS_PIPE_TC, -1};  // built-in rule: SM pairs, or the persistent kernel for a side < 256
    cands[nc++] = Cand{GBS_PIPE_TC, 128};
    cands[nc++] = Cand{GBS_PIPE_TC, 256};
    cands[nc++] = Cand{GBS_PIPE_TC, kPairVariantPersistent};
    cands[nc++] = Cand{GBS_PIPE_TC, kPairVariantStreamK};
    // SM-pair tiles: width 256 / 128 x K split 1, 2, 4
    for (int v : {2561, 2562, 2564, 1281, 1282, 1284}) cands[nc++] = Cand{GBS_PIPE_TC, v};
  }
  if (tc_exact(c, GBS_PIPE_TC_SMEM)) {
    cands[nc++] = Cand{GBS_PIPE_TC_SMEM, 256};
    cands[nc++] = Cand{GBS_PIPE_TC_PAIRS, 128};
  }
  const int saved_pipe = c->pipe, saved_variant = c->variant;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  TuneChoice best{GBS_PIPE_POPC, -1, 1e30};
  int rc = GBS_OK;
  for (int i = 0; i < nc && rc == GBS_OK; i++) {
    c->pipe = cands[i].pipe;
    c->variant = cands[i].variant;
    rc = gbs_gemm(c, stream);  // warm-up (also builds tensor maps)
    if (rc != GBS_OK) break;
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps && rc == GBS_OK; r++) rc = gbs_gemm(c, stream);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "gbs_tune: timing");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double us = 1e3 * ms / reps;
    if (us < best.us) best = TuneChoice{cands[i].pipe, cands[i].variant, us};
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->pipe = saved_pipe;
  c->variant = saved_variant;
  if (rc != GBS_OK) return rc;
  {
    std::lock_guard<std::mutex> lock(g_store_mu);
    g_store[key_of(c)] = best;
  }
  if (best_pipe) *best_pipe = best.pipe;
  return GBS_OK;
}

extern "C" int gbs_tuner_lookup(const gbs_ctx *c, int *pipe, int *variant, double *us) {
  if (!c || !pipe || !variant || !us) return fail(GBS_EINVAL, "gbs_tuner_lookup: NULL argument");
  std::lock_guard<std::mutex> lock(g_store_mu);
  load_env_store();
  auto it = g_store.find(key_of(c));
  if (it == g_store.end()) return fail(GBS_ESTATE, "gbs_tuner_lookup: no entry for this shape class");
  *pipe = it->second.pipe;
  *variant = it->second.variant;
  *us = it->second.us;
  return GBS_OK;
}

extern "C" int gbs_tuner_save(const char *path) {
  if (!path) return fail(GBS_EINVAL, "gbs_tuner_save: path is NULL");
  std::lock_guard<std::mutex> lock(g_store_mu);
  FILE *f = fopen(path, "w");
  if (!f) return fail(GBS_EINVAL, std::string("gbs_tuner_save: cannot open ") + path);
  fprintf(f, "%s\n", kStoreVersion);
  for (auto &kv : g_store) {
    const TuneKey &k = kv.first;
    fprintf(f, "%d %d %d %d %d %d %d %d %d %.3f\n", std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k),
            std::get<4>(k), std::get<5>(k), std::get<6>(k), kv.second.pipe, kv.second.variant, kv.second.us);
  }
  fclose(f);
  return GBS_OK;
}

extern "C" int gbs_tuner_load(const char *path, int replace) {
  if (!path) return fail(GBS_EINVAL, "gbs_tuner_load: path is NULL");
  std::lock_guard<std::mutex> lock(g_store_mu);
  return load_store(path, replace != 0);
}

extern "C" int gbs_tuner_entries(void) {
  std::lock_guard<std::mutex> lock(g_store_mu);
  return (int)g_store.size();
}

extern "C" int gbs_tuner_clear(void) {
  std::lock_guard<std::mutex> lock(g_store_mu);
  g_store.clear();
  return GBS_OK;
}
