// gbs_wide.cu -- the tensor-core digit pipe for operands of 5 to 8 bits.
//
// An operand of w > 4 bits does not fit one e4m3 digit exactly, so it is
// split by planes into a low part (planes [0, lo), unsigned, lo = w - hi) and
// a high part (planes [lo, w), signed when the operand is, hi = max(2, w - 4)
// bits: never a lone signed plane, which would read as bipolar).  Each part
// holds at most 4 significant bits, so every (lhs part, rhs part) product is
// an ordinary digit GEMM, exact while K * max|a part| * max|b part| < 2^24:
//   A.B = sum_{pa, pb} 2^(lo_A pa + lo_B pb) (A_pa . B_pb)
// the plane-weight identity of gemmBitSerial_generic_usingBinary
// (arch-generic.hpp:179-192) grouped by part instead of by single plane.  Each
// part product runs on a sub-context whose planes alias the parent's (no
// copy), whose digit matrices are the parent's per-part buffers, and whose
// result is its own; one combine kernel sums the shifted partial results in
// 32-bit wrap-around arithmetic, as the reference's int32 accumulators do.
#include <algorithm>
#include <cstring>

#include "gbs_internal.h"

namespace gbs {

struct WidePlan {
  int parts[2] = {1, 1};    // parts per side (1 or 2)
  int lo_bits[2] = {0, 0};  // bits of a side's low part (the high part's weight is 2^lo_bits)
  uint8_t *digits[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [side][part] digit matrices
  gbs_ctx *sub[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};      // [lhs part][rhs part]
};

namespace {

int hi_bits(int w) { return w > 4 ? std::max(2, w - 4) : 0; }

// Part `part` of operand m (part 0 is the whole operand when it has <= 4 bits).
Mat part_of(const Mat &m, int part) {
  const int w = (int)m.nbits, hi = hi_bits(w), lo = w - hi;
  Mat p = m;
  if (w <= 4) return p;
  if (part == 0) {
    p.nbits = (uint64_t)lo;
    p.issigned = 0;
  } else {
    p.nbits = (uint64_t)hi;
    p.planes = m.planes + (uint64_t)lo * m.nrows_a * m.wpr();
  }
  return p;
}

uint64_t part_max_abs(const Mat &m) {
  if (m.bipolar()) return 1;
  return m.issigned ? (1ull << (m.nbits - 1)) : ((1ull << m.nbits) - 1);
}

// out[i] = sum_k in_k[i] << shift_k (mod 2^32), 4 elements per thread
__global__ void __launch_bounds__(256) combine_kernel(int32_t *__restrict__ out, const int32_t *__restrict__ in0,
                                                      const int32_t *__restrict__ in1, const int32_t *__restrict__ in2,
                                                      const int32_t *__restrict__ in3, int nin, uint32_t sh1,
                                                      uint32_t sh2, uint32_t sh3, uint64_t n) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (n + 3) / 4; q += stride) {
    const uint64_t i0 = 4 * q;
    if (i0 + 4 <= n) {
      uint4 a = *reinterpret_cast<const uint4 *>(in0 + i0);
      auto add = [&](const int32_t *in, uint32_t sh) {
        const uint4 b = *reinterpret_cast<const uint4 *>(in + i0);
        a.x += b.x << sh;
        a.y += b.y << sh;
        a.z += b.z << sh;
        a.w += b.w << sh;
      };
      if (nin > 1) add(in1, sh1);
      if (nin > 2) add(in2, sh2);
      if (nin > 3) add(in3, sh3);
      *reinterpret_cast<uint4 *>(out + i0) = a;
    } else {
      for (uint64_t i = i0; i < n; i++) {
        uint32_t v = (uint32_t)in0[i];
        if (nin > 1) v += (uint32_t)in1[i] << sh1;
        if (nin > 2) v += (uint32_t)in2[i] << sh2;
        if (nin > 3) v += (uint32_t)in3[i] << sh3;
        out[i] = (int32_t)v;
      }
    }
  }
}

// Sub-contexts and part digit buffers of a wide context, built on first use.
int build_plan(gbs_ctx *c, int variant) {
  WidePlan *p = new WidePlan();
  c->wide = p;
  const Mat *side_m[2] = {&c->lhs, &c->rhs};
  for (int side = 0; side < 2; side++) {
    const int w = (int)side_m[side]->nbits;
    p->parts[side] = w > 4 ? 2 : 1;
    p->lo_bits[side] = w - hi_bits(w);
    const size_t bytes = std::max<size_t>(side_m[side]->drows * side_m[side]->dcols, 16);
    for (int k = 0; k < p->parts[side]; k++) {
      cudaError_t e = dev_alloc((void **)&p->digits[side][k], bytes);
      if (e == cudaSuccess) e = cudaMemset(p->digits[side][k], 0, bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GBS_ENOMEM, "gbs_gemm: digit matrices of the wide-operand parts could not be allocated");
      }
    }
  }
  for (int pa = 0; pa < p->parts[0]; pa++)
    for (int pb = 0; pb < p->parts[1]; pb++) {
      gbs_ctx *s = new gbs_ctx();
      p->sub[pa][pb] = s;
      s->device = c->device;
      s->lhs = part_of(c->lhs, pa);
      s->rhs = part_of(c->rhs, pb);
      s->lhs.imported = s->rhs.imported = true;
      s->pipe = GBS_PIPE_TC;
      s->variant = variant;
      s->digits[0] = p->digits[0][pa];
      s->digits[1] = p->digits[1][pb];
      if (dev_alloc((void **)&s->res, std::max<size_t>(c->lhs.nrows * c->rhs.nrows * 4, 16)) != cudaSuccess) {
        cudaGetLastError();
        return fail(GBS_ENOMEM, "gbs_gemm: partial results of the wide-operand parts could not be allocated");
      }
    }
  return GBS_OK;
}

}  // namespace

bool tc_wide(const gbs_ctx *c) {
  const Mat &A = c->lhs, &B = c->rhs;
  if (A.nbits <= 4 && B.nbits <= 4) return false;
  if (A.nbits > 8 || B.nbits > 8 || A.nrows == 0 || B.nrows == 0 || A.ncols == 0 || !tc_encoder_available())
    return false;
  uint64_t ma = 0, mb = 0;
  for (int k = 0; k < (A.nbits > 4 ? 2 : 1); k++) ma = std::max(ma, part_max_abs(part_of(A, k)));
  for (int k = 0; k < (B.nbits > 4 ? 2 : 1); k++) mb = std::max(mb, part_max_abs(part_of(B, k)));
  return (double)A.ncols * (double)ma * (double)mb < 16777216.0 && A.drows * A.nbits < (1ull << 31) &&
         B.drows * B.nbits < (1ull << 31);
}

void wide_plan_free(WidePlan *p) {
  if (!p) return;
  for (auto &row : p->sub)
    for (gbs_ctx *s : row) {
      if (!s) continue;
      if (s->res) cudaFree(s->res);
      if (s->plan1) {
        tcg_plan_free(s->plan1);
        delete s->plan1;
      }
      if (s->sk_ws) cudaFree(s->sk_ws);
      if (s->sk_flags) cudaFree(s->sk_flags);
      for (uint8_t *nb : s->nibbles)
        if (nb) cudaFree(nb);
      delete s;  // its planes alias the parent's, its digit matrices are the plan's
    }
  for (auto &side : p->digits)
    for (uint8_t *d : side)
      if (d) cudaFree(d);
  delete p;
}

cudaError_t launch_gemm_wide(gbs_ctx *c, cudaStream_t s, int variant) {
  if (!c->wide) {
    if (build_plan(c, variant) != GBS_OK) return cudaErrorMemoryAllocation;
  }
  WidePlan &p = *c->wide;
  // digit matrices of every part of a side whose planes changed since the last expansion
  const Mat *side_m[2] = {&c->lhs, &c->rhs};
  for (int side = 0; side < 2; side++) {
    if (c->digits_valid[side]) continue;
    for (auto &row : p.sub)  // the parts' own nibble matrices (one-problem plans) are stale too
      for (gbs_ctx *sub : row)
        if (sub) sub->nibbles_valid[side] = false;
    for (int k = 0; k < p.parts[side]; k++) {
      cudaError_t e = launch_expand(make_expand_job(part_of(*side_m[side], k), p.digits[side][k]), s);
      if (e != cudaSuccess) return e;
    }
    c->digits_valid[side] = true;
  }
  const int32_t *parts[4] = {nullptr, nullptr, nullptr, nullptr};
  uint32_t shift[4] = {0, 0, 0, 0};
  int n = 0;
  for (int pa = 0; pa < p.parts[0]; pa++)
    for (int pb = 0; pb < p.parts[1]; pb++) {
      gbs_ctx *sub = p.sub[pa][pb];
      sub->variant = variant;
      sub->digits_valid[0] = sub->digits_valid[1] = true;
      sub->out = nullptr;
      cudaError_t e = launch_gemm_tc_hbm(sub, s, variant);
      if (e != cudaSuccess) return e;
      parts[n] = sub->res;
      shift[n] = (uint32_t)(p.lo_bits[0] * pa + p.lo_bits[1] * pb);
      n++;
    }
  // the unshifted part product first: shift[0] is 0 by construction
  const uint64_t total = c->lhs.nrows * c->rhs.nrows;
  const uint64_t threads = (total + 3) / 4;
  const unsigned blocks = (unsigned)std::min<uint64_t>((threads + 255) / 256, 152 * 32);
  combine_kernel<<<blocks, 256, 0, s>>>(result_ptr(c), parts[0], parts[1], parts[2], parts[3], n, shift[1], shift[2],
                                        shift[3], total);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs
