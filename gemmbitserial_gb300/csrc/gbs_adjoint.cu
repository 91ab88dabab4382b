// gbs_adjoint.cu -- FP32 adjoint of the bit-serial GEMM (quantisation-aware training).
//
// No reference counterpart: the reference has no backward pass.  The forward
// res[n, m] = sum_k A[m, k] * B[n, k] is bilinear, so for an upstream
// gradient dC (FP32, in the transposed result layout dC[n*M + m]):
//   dA[m, k] = sum_n dC[n, m] * B[n, k]      (M x K, row-major)
//   dB[n, k] = sum_m dC[n, m] * A[m, k]      (N x K, row-major: the rhs layout)
// where A and B are the VALUES the packed planes encode: sum_j s_j 2^j bit_j
// with s_j = -1 for a signed MSB plane, or 2*bit - 1 for a bipolar operand
// (gemmbitserial.hpp:313-333 defines the same decoding for exportRegular).
//
// Both are one kernel, Out[r, k] = sum_s X(s, r) * V[s, k], where V is decoded
// from planes (rows s) into shared memory and X is dC read either as X[s][r]
// (dA: s = n, r = m, contiguous in r) or as X[r][s] (dB: r = n, s = m,
// contiguous in s).  CTA tile 128 (r) x 128 (k), 8 values of s per stage,
// 256 threads with 8 x 8 outputs each (two 4-wide groups per dimension for
// conflict-free float4 shared reads), FP32 FMA accumulation in registers.
#include <cstdlib>
#include <cstring>

#include "gbs_internal.h"

namespace gbs {
namespace {

constexpr int BR = 128, BKc = 128, BS = 8, NT = 256;

struct AdjArgs {
  const float *X;         // dC
  const uint64_t *planes; // operand decoded into V (rows s)
  float *out;             // R x K row-major
  uint64_t R, S, K, M;    // M: row length of dC (lhs rows of the forward)
  uint64_t plane_words, wpr;
  int nbits, neg_msb, bipolar;
};

// dC element for reduction index s and output row r.
template <bool DA>
__device__ __forceinline__ float x_at(const AdjArgs &a, uint64_t s, uint64_t r) {
  // DA: X(s, r) = dC[s*M + r];  DB: X(s, r) = dC[r*M + s]
  return DA ? a.X[s * a.M + r] : a.X[r * a.M + s];
}

template <bool DA>
__global__ void __launch_bounds__(NT, 1) adjoint_kernel(AdjArgs a) {
  __shared__ __align__(16) float sX[2][BS][BR];
  __shared__ __align__(16) float sV[2][BS][BKc];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const uint64_t r0 = (uint64_t)blockIdx.y * BR, k0 = (uint64_t)blockIdx.x * BKc;
  const int nchunks = (int)((a.S + BS - 1) / BS);

  // X tile: 1024 floats per stage, 4 per thread.  DA: thread -> (s = tid/32,
  // r = (tid%32)*4), contiguous r.  DB: thread -> (r = tid/2, s = (tid%2)*4),
  // contiguous s, stored transposed.
  auto fetch_x = [&](uint64_t s0, float (&t)[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) t[i] = 0.f;
    if (DA) {
      const uint64_t gs = s0 + (tid >> 5), gr = r0 + (tid & 31) * 4;
      if (gs < a.S) {
        if (gr + 3 < a.R && (a.M & 3) == 0) {
          const float4 v = *reinterpret_cast<const float4 *>(a.X + gs * a.M + gr);
          t[0] = v.x; t[1] = v.y; t[2] = v.z; t[3] = v.w;
        } else {
#pragma unroll
          for (int i = 0; i < 4; i++) t[i] = gr + i < a.R ? x_at<DA>(a, gs, gr + i) : 0.f;
        }
      }
    } else {
      const uint64_t gr = r0 + (tid >> 1), gs = s0 + (tid & 1) * 4;
      if (gr < a.R) {
        if (gs + 3 < a.S && (a.M & 3) == 0) {
          const float4 v = *reinterpret_cast<const float4 *>(a.X + gr * a.M + gs);
          t[0] = v.x; t[1] = v.y; t[2] = v.z; t[3] = v.w;
        } else {
#pragma unroll
          for (int i = 0; i < 4; i++) t[i] = gs + i < a.S ? x_at<DA>(a, gs + i, gr) : 0.f;
        }
      }
    }
  };
  auto store_x = [&](int st, const float (&t)[4]) {
    if (DA) {
      *reinterpret_cast<float4 *>(&sX[st][tid >> 5][(tid & 31) * 4]) = make_float4(t[0], t[1], t[2], t[3]);
    } else {
#pragma unroll
      for (int i = 0; i < 4; i++) sX[st][(tid & 1) * 4 + i][tid >> 1] = t[i];
    }
  };
  // V tile: rows s0..s0+7, columns k0..k0+127; thread -> (s = tid/32, k = (tid%32)*4):
  // fetch the 4 bits of each plane, decode to values on store.
  auto fetch_v = [&](uint64_t s0, uint32_t (&bits)[kMaxBits]) {
    const uint64_t gs = s0 + (tid >> 5), gk = k0 + (tid & 31) * 4;
    const uint64_t w = gk >> 6;
    const int sh = (int)(gk & 63);
    const bool ok = gs < a.S && w < a.wpr;
#pragma unroll
    for (int b = 0; b < kMaxBits; b++)
      bits[b] = (ok && b < a.nbits) ? (uint32_t)(a.planes[b * a.plane_words + gs * a.wpr + w] >> sh) & 0xfu : 0u;
  };
  auto store_v = [&](int st, const uint32_t (&bits)[kMaxBits]) {
    float v[4];
    if (a.bipolar) {
#pragma unroll
      for (int i = 0; i < 4; i++) v[i] = ((bits[0] >> i) & 1u) ? 1.f : -1.f;
    } else {
      int iv[4] = {0, 0, 0, 0};
#pragma unroll
      for (int b = 0; b < kMaxBits; b++) {
        if (b >= a.nbits) break;
        const int wgt = (b == a.neg_msb) ? -(1 << b) : (1 << b);
#pragma unroll
        for (int i = 0; i < 4; i++) iv[i] += ((bits[b] >> i) & 1u) ? wgt : 0;
      }
#pragma unroll
      for (int i = 0; i < 4; i++) v[i] = (float)iv[i];
    }
    *reinterpret_cast<float4 *>(&sV[st][tid >> 5][(tid & 31) * 4]) = make_float4(v[0], v[1], v[2], v[3]);
  };

  // Two-level FP32 accumulation: FMAs go into part[][] for kFold stages (32
  // reduction terms), which is then added into acc[][].  The running sum then
  // sees S/32 roundings instead of S, which keeps the normwise error of a
  // 2048-4096 term reduction near 3e-7 of the largest result.
  constexpr int kFold = 4;
  float acc[8][8], part[8][8];
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[i][j] = part[i][j] = 0.f;

  float xt[4];
  uint32_t vb[kMaxBits];
  if (nchunks > 0) {
    fetch_x(0, xt);
    fetch_v(0, vb);
    store_x(0, xt);
    store_v(0, vb);
  }
  __syncthreads();
  for (int c = 0; c < nchunks; c++) {
    const int st = c & 1;
    const bool more = c + 1 < nchunks;
    if (more) {  // global loads of the next stage overlap this stage's FMAs
      fetch_x((uint64_t)(c + 1) * BS, xt);
      fetch_v((uint64_t)(c + 1) * BS, vb);
    }
#pragma unroll
    for (int s = 0; s < BS; s++) {
      const float4 x0 = *reinterpret_cast<const float4 *>(&sX[st][s][ty * 4]);
      const float4 x1 = *reinterpret_cast<const float4 *>(&sX[st][s][64 + ty * 4]);
      const float4 v0 = *reinterpret_cast<const float4 *>(&sV[st][s][tx * 4]);
      const float4 v1 = *reinterpret_cast<const float4 *>(&sV[st][s][64 + tx * 4]);
      const float xr[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
      const float vk[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) part[i][j] = fmaf(xr[i], vk[j], part[i][j]);
    }
    if ((c + 1) % kFold == 0 || !more) {
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) {
          acc[i][j] += part[i][j];
          part[i][j] = 0.f;
        }
    }
    if (more) {
      store_x(st ^ 1, xt);
      store_v(st ^ 1, vb);
    }
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint64_t gr = r0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
    if (gr >= a.R) continue;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const uint64_t gk = k0 + half * 64 + tx * 4;
      float *dst = a.out + gr * a.K + gk;
      const float *src = &acc[i][half * 4];
      if (gk + 3 < a.K && (a.K & 3) == 0) {
        *reinterpret_cast<float4 *>(dst) = make_float4(src[0], src[1], src[2], src[3]);
      } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (gk + j < a.K) dst[j] = src[j];
      }
    }
  }
}

}  // namespace

cudaError_t launch_adjoint(const Mat &op, const float *dC, uint64_t M, uint64_t N, bool da, float *out,
                           cudaStream_t s) {
  AdjArgs a;
  a.X = dC;
  a.planes = op.planes;
  a.out = out;
  a.M = M;
  a.R = da ? M : N;
  a.S = da ? N : M;
  a.K = op.ncols;
  a.plane_words = op.nrows_a * op.wpr();
  a.wpr = op.wpr();
  a.nbits = (int)op.nbits;
  a.bipolar = op.bipolar() ? 1 : 0;
  a.neg_msb = (op.issigned && !op.bipolar()) ? (int)op.nbits - 1 : -1;
  if (a.R == 0 || a.K == 0) return cudaSuccess;
  if (a.S == 0) return cudaMemsetAsync(out, 0, a.R * a.K * sizeof(float), s);
  dim3 grid((unsigned)((a.K + BKc - 1) / BKc), (unsigned)((a.R + BR - 1) / BR));
  if (da) adjoint_kernel<true><<<grid, NT, 0, s>>>(a);
  else adjoint_kernel<false><<<grid, NT, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gbs

using namespace gbs;

extern "C" int gbs_adjoint(gbs_ctx *c, const float *dC, float *dA, float *dB, void *stream) {
  if (!c) return fail(GBS_EINVAL, "gbs_adjoint: ctx is NULL");
  if (!c->lhs.imported || !c->rhs.imported) return fail(GBS_ESTATE, "gbs_adjoint: import both operands first");
  const uint64_t M = c->lhs.nrows, N = c->rhs.nrows;
  if ((dA || dB) && M && N && !dC) return fail(GBS_EINVAL, "gbs_adjoint: dC is NULL");
  for (const void *p : {(const void *)dC, (const void *)dA, (const void *)dB}) {
    if (!p) continue;
    // the kernels move rows of 4 floats as 16-byte vectors
    if ((uintptr_t)p % 16 != 0) return fail(GBS_EINVAL, "gbs_adjoint: dC, dA and dB must be 16-byte aligned");
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
        (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
      cudaGetLastError();
      return fail(GBS_EINVAL, "gbs_adjoint: dC, dA and dB must be device pointers");
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  const char *mode = getenv("GBS_ADJOINT_PIPE");
  if (!(mode && !strcmp(mode, "simt")) && adjoint_tc_available()) return adjoint_tc(c, dC, dA, dB, s);
  if (dA) {
    cudaError_t e = launch_adjoint(c->rhs, dC, M, N, true, dA, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_adjoint: dA kernel");
  }
  if (dB) {
    cudaError_t e = launch_adjoint(c->lhs, dC, M, N, false, dB, s);
    if (e != cudaSuccess) return cuda_fail(e, "gbs_adjoint: dB kernel");
  }
  return GBS_OK;
}
