// gbs_gemm_bmma.cu -- forward bit-serial GEMM on the tensor pipe (mma.sync b1).
#include "gbs_internal.h"

namespace gbs {

bool bmma_supported(int, int, int) { return false; }

cudaError_t launch_gemm_bmma(const GemmShape &, const Epilogue &, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace gbs
