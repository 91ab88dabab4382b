// gbs_grouped.cu -- many independent bit-serial GEMMs in one persistent launch.
//
// The reference runs a list of GEMMs as a host loop of gemmBitSerial calls
// over a vector of contexts (benchmark.cpp:192-206, 217-219).  A group does the
// same work with
//   * one grouped pack launch for every operand (optional),
//   * one grouped row-sum launch when some problem is bipolar x regular,
//   * one persistent GEMM launch whose CTAs drain a device tile queue (an
//     atomic counter over a tile table sorted by decreasing cost),
// and can capture that sequence once into a CUDA graph for replay.  Each
// problem keeps its own context, so results land in each context's res.
//
// Problems go to one of two persistent kernels: the tensor-core kernel over
// e4m3 digit matrices (gbs_gemm_tcg.cu) where it is exact and cheaper, the
// CUDA-core popcount kernel otherwise.  GBS_GROUP_PIPE=popc or =tc in the
// environment forces one kernel (tc: wherever it is exact).  Digit matrices
// are rebuilt by one grouped expansion launch after every import.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbs_internal.h"

struct gbs_group {
  int device = 0;
  std::vector<gbs_ctx *> ctxs;
  gbs::GroupProblem *d_probs = nullptr;
  gbs::GroupTile *d_tiles = nullptr;
  uint32_t ntiles = 0;
  uint32_t *d_scratch = nullptr;  // [0] tile counter, [1] popcount-kernel error bits, [2] tensor-core error bits
  gbs::PackJob *d_rs_jobs = nullptr;
  int nrs = 0;
  uint64_t rs_warps = 0;
  gbs::PackJob *d_pack_jobs = nullptr;
  int npack = 0;
  uint64_t pack_warps = 0;
  size_t smem = 0;
  int grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  gbs::TcgPlan tc;  // problems on the tensor-core kernel
  std::vector<char> is_tc;  // per problem: on the tensor-core kernel
  // with both kernel types, the tensor-core kernel runs on a stream forked
  // from the caller's (and joined back), so the two share the SMs
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  uint64_t launches_per_replay = 0;
  uint32_t popc_tiles = 0;
};

namespace gbs {
namespace {

// Largest dynamic shared memory per CTA that still lets two CTAs share an SM.
constexpr size_t kGroupSmemCap = 113 * 1024;

bool device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void free_group(gbs_group *g) {
  tcg_plan_free(&g->tc);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->join) cudaEventDestroy(g->join);
  if (g->side) cudaStreamDestroy(g->side);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->d_probs) cudaFree(g->d_probs);
  if (g->d_tiles) cudaFree(g->d_tiles);
  if (g->d_scratch) cudaFree(g->d_scratch);
  if (g->d_rs_jobs) cudaFree(g->d_rs_jobs);
  if (g->d_pack_jobs) cudaFree(g->d_pack_jobs);
  delete g;
}

template <typename T>
cudaError_t upload(T **dst, const std::vector<T> &v) {
  cudaError_t e = dev_alloc((void **)dst, v.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  return cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// Builds the pack-job table for (lhs_srcs[p], rhs_srcs[p]) of every problem.
int build_pack_jobs(gbs_group *g, const void *const *lhs, const void *const *rhs, const int *dtypes) {
  std::vector<PackJob> jobs;
  uint64_t warps = 0;
  size_t ti = 0;  // index among the tensor-core problems
  for (size_t p = 0; p < g->ctxs.size(); p++) {
    const uint8_t digit_sides = g->is_tc[p] ? g->tc.sides[ti++] : 0;
    for (int side = 0; side < 2; side++) {
      const void *src = side ? rhs[p] : lhs[p];
      const int dt = dtypes ? dtypes[2 * p + side] : GBS_I8;
      if (dt < GBS_I8 || dt > GBS_F32) return fail(GBS_EINVAL, "gbs_group: unknown dtype");
      const Mat &m = side ? g->ctxs[p]->rhs : g->ctxs[p]->lhs;
      if (m.nrows_a == 0 || m.wpr() == 0) continue;
      if (m.nrows && m.ncols && (!src || !device_ptr(src)))
        return fail(GBS_EINVAL, "gbs_group: sources must be device pointers (problem " + std::to_string(p) + ")");
      PackJob j;
      memset(&j, 0, sizeof(j));
      j.src = src;
      j.planes = m.planes;
      j.nrows = m.nrows;
      j.ncols = m.ncols;
      j.nrows_a = m.nrows_a;
      j.wpr = m.wpr();
      j.nbits = (int)m.nbits;
      j.issigned = m.issigned;
      j.dtype = dt;
      j.vec = (dt == GBS_I8 || dt == GBS_U8) && m.ncols % 16 == 0 && ((uintptr_t)src % 16) == 0;
      j.segs = (uint32_t)pack_segs_per_row(m.wpr());
      j.dcols = m.dcols;
      if ((digit_sides >> side) & 1) {  // tensor-core problem: the import writes the digit matrices it reads
        j.digits = g->ctxs[p]->digits[side];
        tc_digit_table(m, j.dtab);
      }
      if ((digit_sides >> (2 + side)) & 1) j.nibbles = g->ctxs[p]->nibbles[side];  // ... and nibble matrices
      j.warp0 = warps;
      warps += m.nrows_a * j.segs;
      jobs.push_back(j);
    }
  }
  if (g->d_pack_jobs) cudaFree(g->d_pack_jobs);
  g->d_pack_jobs = nullptr;
  if (upload(&g->d_pack_jobs, jobs) != cudaSuccess) {
    cudaGetLastError();
    return fail(GBS_ENOMEM, "gbs_group: pack table upload failed");
  }
  g->npack = (int)jobs.size();
  g->pack_warps = warps;
  return GBS_OK;
}

cudaError_t enqueue_gemm(gbs_group *g, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  const bool both = g->popc_tiles && g->tc.ntiles;
  if (both) {  // the tensor-core kernel on the side stream
    e = cudaEventRecord(g->fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(g->side, g->fork, 0);
    if (e == cudaSuccess) e = tcg_gemm(g->tc, g->d_scratch + 2, g->side);
    if (e == cudaSuccess) e = cudaEventRecord(g->join, g->side);
    if (e != cudaSuccess) return e;
  }
  if (g->popc_tiles) {
    e = cudaMemsetAsync(g->d_scratch, 0, sizeof(uint32_t), s);  // tile counter only
    if (e == cudaSuccess && g->nrs) e = launch_rowsum_grouped(g->d_rs_jobs, g->nrs, g->rs_warps, s);
    if (e == cudaSuccess)
      e = launch_gemm_popc_grouped(g->d_probs, (int)g->ctxs.size(), g->d_tiles, g->popc_tiles, g->d_scratch,
                                   g->d_scratch + 1, g->smem, g->grid, s);
  }
  if (both) {
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g->join, 0);
  } else if (e == cudaSuccess) {
    e = tcg_gemm(g->tc, g->d_scratch + 2, s);
  }
  return e;
}

// True when a digit or nibble matrix some tensor-core problem reads is older than its planes.
bool digits_stale(const gbs_group *g) {
  for (size_t i = 0; i < g->tc.ctxs.size(); i++)
    for (int side = 0; side < 2; side++) {
      if (((g->tc.sides[i] >> side) & 1) && !g->tc.ctxs[i]->digits_valid[side]) return true;
      if (((g->tc.sides[i] >> (2 + side)) & 1) && !g->tc.ctxs[i]->nibbles_valid[side]) return true;
    }
  return false;
}

// After a grouped pack: the digit and nibble matrices it wrote match the new
// planes, any other of the group's contexts is stale.
void mark_packed_digits(const gbs_group *g) {
  for (gbs_ctx *c : g->ctxs)
    for (int side = 0; side < 2; side++) c->digits_valid[side] = c->nibbles_valid[side] = false;
  for (size_t i = 0; i < g->tc.ctxs.size(); i++)
    for (int side = 0; side < 2; side++) {
      g->tc.ctxs[i]->digits_valid[side] = ((g->tc.sides[i] >> side) & 1) != 0;
      g->tc.ctxs[i]->nibbles_valid[side] = ((g->tc.sides[i] >> (2 + side)) & 1) != 0;
    }
}

// 0 = per-problem choice, 1 = popcount kernel only, 2 = tensor-core kernel wherever exact.
int group_pipe_mode() {
  const char *v = getenv("GBS_GROUP_PIPE");
  if (!v) return 0;
  if (!strcmp(v, "popc")) return 1;
  if (!strcmp(v, "tc")) return 2;
  return 0;
}

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" {

int gbs_group_create(gbs_ctx *const *ctxs, int count, gbs_group **out) {
  if (!out) return fail(GBS_EINVAL, "gbs_group_create: out is NULL");
  *out = nullptr;
  if (count < 0 || (count > 0 && !ctxs)) return fail(GBS_EINVAL, "gbs_group_create: bad context list");
  gbs_group *g = new gbs_group();
  if (cudaGetDevice(&g->device) != cudaSuccess) {
    delete g;
    return cuda_fail(cudaGetLastError(), "gbs_group_create: no device");
  }
  std::vector<GroupProblem> probs;
  std::vector<GroupTile> tiles;
  std::vector<uint64_t> cost;
  std::vector<PackJob> rs;
  uint64_t rs_warps = 0;
  size_t smem = 16;
  const int mode = group_pipe_mode();
  std::vector<gbs_ctx *> tc_ctxs;
  for (int p = 0; p < count; p++) {
    gbs_ctx *c = ctxs[p];
    if (!c) {
      delete g;
      return fail(GBS_EINVAL, "gbs_group_create: context " + std::to_string(p) + " is NULL");
    }
    if (c->device != g->device) {
      delete g;
      return fail(GBS_EINVAL, "gbs_group_create: contexts must live on the current device");
    }
    g->ctxs.push_back(c);
    g->is_tc.push_back(mode != 1 && tcg_eligible(c) && (mode == 2 || tcg_preferred(c)) ? 1 : 0);
    if (g->is_tc.back()) {
      tc_ctxs.push_back(c);
      GroupProblem none;  // keeps the popcount table indexed by problem
      memset(&none, 0, sizeof(none));
      probs.push_back(none);
      continue;
    }
    Epilogue e;
    make_epilogue(c, e, c->rowsum);
    GroupProblem P;
    memset(&P, 0, sizeof(P));
    P.A = c->lhs.planes;
    P.B = c->rhs.planes;
    P.C = c->res;
    P.ra = e.ra;
    P.rb = e.rb;
    P.M = c->lhs.nrows;
    P.N = c->rhs.nrows;
    P.wpr = c->lhs.wpr();
    P.a_plane = c->lhs.nrows_a * P.wpr;
    P.b_plane = c->rhs.nrows_a * P.wpr;
    P.a_rows = c->lhs.nrows_a;
    P.b_rows = c->rhs.nrows_a;
    P.wa = (int)c->lhs.nbits;
    P.wb = (int)c->rhs.nbits;
    P.use_xor = e.use_xor;
    P.neg_i = e.neg_i;
    P.neg_j = e.neg_j;
    P.shift = e.shift;
    P.c0 = e.c0;
    // kSkinnyTile outputs per tile, a warp each, where every BM x BN class would
    // leave most of its tile empty: fewer than 16 rhs rows (the classes' BN is
    // 64 or more), or a tiny output of more than 16 lhs rows; at most 16 lhs
    // rows take the rows class below (a warp per output waits on memory once
    // per output, a rows tile once per 128-byte step of 256 outputs)
    const bool rows_fit = P.M <= (uint64_t)kRowsMaxM && popc_rows_smem(P.wa, kRowsKC) <= kGroupSmemCap;
    if (P.N < 16 || (P.M * P.N <= 4096 && !rows_fit)) {
      P.cls = kSkinnyCls;
      probs.push_back(P);
      const uint64_t nt = (P.M * P.N + kSkinnyTile - 1) / kSkinnyTile;
      for (uint64_t i = 0; i < nt; i++) {
        tiles.push_back(GroupTile{(uint32_t)p, (uint32_t)i, 0u, (uint32_t)kSkinnyCls});
        cost.push_back(std::max<uint64_t>(1, (uint64_t)P.wa * P.wb * P.wpr / 512));
      }
    } else if (rows_fit) {
      // at most 16 lhs rows: the rows class, one rhs row per thread (no popcounts on padding rows)
      P.cls = kRowsCls;
      smem = std::max(smem, popc_rows_smem(P.wa, kRowsKC));
      probs.push_back(P);
      const uint64_t bnr = (uint64_t)rows_tile_n(P.M), nt = (P.N + bnr - 1) / bnr;
      for (uint64_t j = 0; j < nt; j++) {
        tiles.push_back(GroupTile{(uint32_t)p, 0u, (uint32_t)j, (uint32_t)kRowsCls});
        cost.push_back((uint64_t)P.wa * P.wb * P.wpr);
      }
    } else {
      P.cls = popc_tile_class(P.M, P.wa, P.wb, kGroupSmemCap);
      smem = std::max(smem, popc_stage_smem(P.cls, P.wa, P.wb, kGroupKC));
      probs.push_back(P);
      const uint64_t bm = tile_bm(P.cls), bn = tile_bn(P.cls);
      const uint64_t mt = (P.M + bm - 1) / bm, nt = (P.N + bn - 1) / bn;
      for (uint64_t i = 0; i < mt; i++)
        for (uint64_t j = 0; j < nt; j++) {
          tiles.push_back(GroupTile{(uint32_t)p, (uint32_t)i, (uint32_t)j, (uint32_t)P.cls});
          cost.push_back((uint64_t)P.wa * P.wb * P.wpr);
        }
    }
    if (e.ra || e.rb) {  // bipolar x regular: row sums of the regular operand
      const Mat &reg = c->lhs.bipolar() ? c->rhs : c->lhs;
      PackJob j;
      memset(&j, 0, sizeof(j));
      j.planes = reg.planes;
      j.rowsum = c->rowsum;
      j.nrows = reg.nrows;
      j.ncols = reg.ncols;
      j.nrows_a = reg.nrows_a;
      j.wpr = reg.wpr();
      j.nbits = (int)reg.nbits;
      j.issigned = reg.issigned;
      j.warp0 = rs_warps;
      rs_warps += reg.nrows;
      if (reg.nrows) rs.push_back(j);
    }
  }
  // Longest tiles first: the queue then balances like LPT scheduling.
  std::vector<size_t> order(tiles.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  std::vector<GroupTile> sorted(tiles.size());
  for (size_t i = 0; i < order.size(); i++) sorted[i] = tiles[order[i]];

  if (!tc_ctxs.empty()) {
    const int rc = tcg_plan_build(&g->tc, tc_ctxs.data(), (int)tc_ctxs.size());
    if (rc != GBS_OK) {
      free_group(g);
      return rc;
    }
  }
  cudaError_t e = upload(&g->d_probs, probs);
  if (e == cudaSuccess) e = upload(&g->d_tiles, sorted);
  if (e == cudaSuccess) e = upload(&g->d_rs_jobs, rs);
  if (e == cudaSuccess) e = dev_alloc((void **)&g->d_scratch, 3 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(g->d_scratch, 0, 3 * sizeof(uint32_t));
  if (e == cudaSuccess) e = prepare_gemm_popc_grouped(smem);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cudaGetLastError();
    free_group(g);
    return fail(GBS_ENOMEM, "gbs_group_create: device allocation or upload failed");
  }
  g->popc_tiles = (uint32_t)sorted.size();
  g->ntiles = g->popc_tiles + g->tc.ntiles;
  g->nrs = (int)rs.size();
  g->rs_warps = rs_warps;
  g->smem = smem;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device);
  g->grid = std::max(1, std::min<int>((int)g->popc_tiles, sms * grouped_blocks_per_sm(smem)));
  *out = g;
  return GBS_OK;
}

int gbs_group_free(gbs_group *g) {
  if (!g) return GBS_OK;
  cudaDeviceSynchronize();
  free_group(g);
  return GBS_OK;
}

int gbs_group_import(gbs_group *g, const void *const *lhs_srcs, const void *const *rhs_srcs, const int *dtypes,
                     void *stream) {
  if (!g || !lhs_srcs || !rhs_srcs) return fail(GBS_EINVAL, "gbs_group_import: NULL argument");
  int rc = build_pack_jobs(g, lhs_srcs, rhs_srcs, dtypes);
  if (rc != GBS_OK) return rc;
  cudaError_t e = launch_pack_grouped(g->d_pack_jobs, g->npack, g->pack_warps, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_group_import: pack kernel");
  for (gbs_ctx *c : g->ctxs) {
    c->lhs.imported = c->rhs.imported = true;
    c->vt_valid[0] = c->vt_valid[1] = false;
  }
  mark_packed_digits(g);
  return GBS_OK;
}

int gbs_group_gemm(gbs_group *g, void *stream) {
  if (!g) return fail(GBS_EINVAL, "gbs_group_gemm: group is NULL");
  for (gbs_ctx *c : g->ctxs)
    if (!c->lhs.imported || !c->rhs.imported) return fail(GBS_ESTATE, "gbs_group_gemm: import every operand first");
  cudaError_t e = cudaSuccess;
  if (digits_stale(g)) e = tcg_expand(g->tc, (cudaStream_t)stream);
  if (e == cudaSuccess) e = enqueue_gemm(g, (cudaStream_t)stream);
  if (e == cudaSuccess)
    for (gbs_ctx *c : g->ctxs) c->res_stale = false;
  return e == cudaSuccess ? GBS_OK : cuda_fail(e, "gbs_group_gemm");
}

int gbs_group_capture(gbs_group *g, const void *const *lhs_srcs, const void *const *rhs_srcs, const int *dtypes,
                      void *stream) {
  if (!g) return fail(GBS_EINVAL, "gbs_group_capture: group is NULL");
  if (!stream)  // CUDA cannot capture the legacy default stream
    return fail(GBS_EINVAL, "gbs_group_capture: capture needs a created stream, not the legacy default stream");
  const bool with_pack = lhs_srcs && rhs_srcs;
  if (with_pack) {
    int rc = build_pack_jobs(g, lhs_srcs, rhs_srcs, dtypes);
    if (rc != GBS_OK) return rc;
  } else {
    for (gbs_ctx *c : g->ctxs)
      if (!c->lhs.imported || !c->rhs.imported)
        return fail(GBS_ESTATE, "gbs_group_capture: without sources, import every operand first");
  }
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  g->exec = nullptr;
  g->graph = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  if (!with_pack && digits_stale(g)) {  // the graph then holds the GEMMs only
    cudaError_t xe = tcg_expand(g->tc, s);
    if (xe != cudaSuccess) return cuda_fail(xe, "gbs_group_capture: digit expansion");
  }
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_group_capture: begin capture");
  cudaError_t ke = cudaSuccess;
  if (with_pack) ke = launch_pack_grouped(g->d_pack_jobs, g->npack, g->pack_warps, s);
  if (ke == cudaSuccess) ke = enqueue_gemm(g, s);
  e = cudaStreamEndCapture(s, &g->graph);
  if (ke != cudaSuccess) return cuda_fail(ke, "gbs_group_capture: enqueue");
  if (e != cudaSuccess) return cuda_fail(e, "gbs_group_capture: end capture");
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_group_capture: instantiate");
  g->launches_per_replay = (with_pack && g->npack ? 1 : 0) + (g->popc_tiles ? 1 + (g->nrs ? 1 : 0) : 0) +
                           (g->tc.ntiles ? 1 : 0);
  if (with_pack) {
    for (gbs_ctx *c : g->ctxs) c->lhs.imported = c->rhs.imported = true;
    mark_packed_digits(g);  // each replay packs them
  }
  return GBS_OK;
}

int gbs_group_replay(gbs_group *g, void *stream) {
  if (!g || !g->exec) return fail(GBS_ESTATE, "gbs_group_replay: capture the group first");
  cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_group_replay");
  if (g->npack) {  // the replay packs new planes: cached adjoint operands and other derived copies are stale
    for (gbs_ctx *c : g->ctxs) c->vt_valid[0] = c->vt_valid[1] = false;
    mark_packed_digits(g);
  }
  for (gbs_ctx *c : g->ctxs) c->res_stale = false;
  count_launch(g->launches_per_replay);
  return GBS_OK;
}

int gbs_group_status(gbs_group *g, void *stream) {
  if (!g) return fail(GBS_EINVAL, "gbs_group_status: group is NULL");
  uint32_t err[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(err, g->d_scratch + 1, sizeof(err), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbs_group_status");
  if (err[0]) return fail(GBS_EINVAL, "gbs_group_status: the grouped kernel rejected tile descriptors (bits " +
                                          std::to_string(err[0]) + ")");
  if (err[1] & 4u) return fail(GBS_EINVAL, "gbs_group_status: the tensor-core kernel rejected tile descriptors");
  if (err[1]) return fail(GBS_ECUDA, "gbs_group_status: a tensor-core pipeline wait timed out (bits " +
                                         std::to_string(err[1]) + ")");
  return GBS_OK;
}

int gbs_group_stats(const gbs_group *g, uint64_t *ntiles, uint64_t *smem_bytes, uint64_t *grid) {
  if (!g) return fail(GBS_EINVAL, "gbs_group_stats: group is NULL");
  if (ntiles) *ntiles = g->ntiles;
  if (smem_bytes) *smem_bytes = g->smem;
  if (grid) *grid = (uint64_t)g->grid;
  return GBS_OK;
}

int gbs_group_split(const gbs_group *g, uint64_t *popc_problems, uint64_t *tc_problems, uint64_t *tc_tiles) {
  if (!g) return fail(GBS_EINVAL, "gbs_group_split: group is NULL");
  if (popc_problems) *popc_problems = g->ctxs.size() - g->tc.ctxs.size();
  if (tc_problems) *tc_problems = g->tc.ctxs.size();
  if (tc_tiles) *tc_tiles = g->tc.ntiles;
  return GBS_OK;
}

int gbs_debug_group_tc_kernel(const gbs_group *g) {
  if (!g) return -fail(GBS_EINVAL, "gbs_debug_group_tc_kernel: group is NULL");  // negative: not a kernel code
  if (!g->tc.ntiles) return 0;
  return g->tc.nibbles ? 2 : 1;
}

int gbs_debug_group_poison_tile(gbs_group *g, uint32_t tile) {
  if (!g || tile >= g->ntiles) return fail(GBS_EINVAL, "gbs_debug_group_poison_tile: bad tile");
  cudaError_t e;
  if (tile < g->popc_tiles) {
    GroupTile bad{0xffffffffu, 0u, 0u, 0u};
    e = cudaMemcpy(g->d_tiles + tile, &bad, sizeof(bad), cudaMemcpyHostToDevice);
  } else {
    TcgTile bad{0xffffffffu, 0u, 0u, 0u};
    e = cudaMemcpy(g->tc.d_tiles + (tile - g->popc_tiles), &bad, sizeof(bad), cudaMemcpyHostToDevice);
  }
  return e == cudaSuccess ? GBS_OK : cuda_fail(e, "gbs_debug_group_poison_tile");
}

}  // extern "C"
