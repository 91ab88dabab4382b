// gbs_tc_common.cuh -- device primitives shared by the tensor-core kernels:
// mbarriers with bounded waits, TMA tile loads, tcgen05 descriptors and MMA
// issue, and the bit-plane -> e4m3 digit decode.
#pragma once
#include <cuda.h>
#include <stdint.h>

namespace gbs {

// Iterations of mbarrier try_wait before a wait gives up (each try_wait may
// also suspend the thread for a short, hardware-chosen time).
constexpr uint32_t kTcWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.b32 %0, 1, 0, P;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: true when the phase completed; false on abort or timeout.
// A timeout raises the CTA's abort flag and sets bit 0 of *err.
__device__ __forceinline__ bool mbar_wait_err(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                              uint32_t *err) {
  for (uint32_t it = 0; it < kTcWaitLimit; ++it) {
    if (mbar_try(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  *abort_flag = 1;
  atomicOr(err, 1u);
  return false;
}
// Bounded wait that ignores the abort flag: drains work this thread issued.
// A timeout sets bit 1 of *err.
__device__ __forceinline__ void mbar_drain_err(uint32_t bar, uint32_t parity, uint32_t *err) {
  for (uint32_t it = 0; it < kTcWaitLimit; ++it)
    if (mbar_try(bar, parity)) return;
  atomicOr(err, 2u);
}

// Programmatic dependent launch.  A kernel launched with the
// programmatic-stream-serialization attribute may start while the kernel
// before it in the stream is still running: it sets up (barriers, TMEM) and
// then calls griddep_wait(), which returns once the previous grids have
// completed and their memory is visible; nothing before it may read or write
// global memory.  griddep_launch_dependents() lets the next such kernel in
// the stream be scheduled as soon as every CTA of this one has issued it (its
// CTAs then take SMs as ours leave and wait likewise).
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Rows [row, row + box) (row a multiple of 16) x digits [128 k, 128 k + 128)
// of a digit matrix through its blocked 4-D map (tc_map_u8): the box lands
// in shared memory as box x 128 bytes, rows in order, 128-byte swizzled.
__device__ __forceinline__ void tma_load_digits(uint32_t dst, const CUtensorMap *map, int k, uint32_t row,
                                                uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(k), "r"((int)(row >> 4)), "r"(bar)
      : "memory");
}

// NC consecutive result columns n0 .. n0+NC-1 of result row m (res[n*M + m];
// a warp's lanes on consecutive m): one base pointer and a fixed column
// stride, whole blocks without per-column predicates.  A 64-bit index and a
// predicate per element measured up to ~2.5x slower in a persistent kernel.
template <int NC>
__device__ __forceinline__ void store_result_cols(int32_t *C, uint64_t M, uint64_t N, uint64_t m, uint64_t n0,
                                                  const int32_t (&o)[NC]) {
  if (m >= M) return;
  int32_t *p = C + n0 * M + m;
  if (n0 + NC <= N) {
#pragma unroll
    for (int j = 0; j < NC; j++) p[(uint64_t)j * M] = o[j];
  } else {
#pragma unroll
    for (int j = 0; j < NC; j++)
      if (n0 + j < N) p[(uint64_t)j * M] = o[j];
  }
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// The same for 64-byte rows: 64-byte swizzle, 8-row groups 512 bytes apart.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

__device__ __forceinline__ void mma_f8(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ uint32_t bfe4(uint32_t x, int sh) {
  uint32_t r;
  asm("bfe.u32 %0, %1, %2, 4;" : "=r"(r) : "r"(x), "r"(sh));
  return r;
}

// e4m3 bytes of 4 consecutive columns of one tile row: codes from the tile's
// planes (bits at column offset `sh` of each plane's 32-bit word), then a
// byte-permute lookup in the tile's 16-entry table.  Plane p's nibble is
// spread straight to bit p of each byte (multiplier and mask shifted by p).
template <int CNT>
__device__ __forceinline__ uint32_t decode4(const uint32_t (&pw)[4], int sh, const uint32_t (&tab)[4]) {
  uint32_t c = 0;
#pragma unroll
  for (int p = 0; p < CNT; p++) c |= (bfe4(pw[p], sh) * (0x00204081u << p)) & (0x01010101u << p);
  if (CNT == 1) return c;  // caller maps 0/1 bytes itself
  const uint32_t t = c | (c >> 4);                        // byte 0 = c0 | c1<<4, byte 2 = c2 | c3<<4
  const uint32_t sel = __byte_perm(t, 0u, 0x0020u);        // nibbles c0 c1 c2 c3 in the low 16 bits
  if (CNT <= 3) return __byte_perm(tab[0], tab[1], sel);
  const uint32_t lo = __byte_perm(tab[0], tab[1], sel & 0x7777u);
  const uint32_t hi = __byte_perm(tab[2], tab[3], sel & 0x7777u);
  const uint32_t m = ((c >> 3) & 0x01010101u) * 0xFFu;     // codes 8..15 take the high table
  return (lo & ~m) | (hi & m);
}


}  // namespace gbs
