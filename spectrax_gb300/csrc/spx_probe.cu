// spx_probe.cu — FP64 issue-rate probe used as the compute roofline denominator.
//
// Each thread runs 8 independent FMA chains; the result is written out so the
// work cannot be removed.  FLOP/s = 2 * 8 * iters * threads / time.
#include "spx_plan.h"

namespace spx {
__global__ void __launch_bounds__(256) k_fp64_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace spx

extern "C" int spx_probe_fp64(void* out, int blocks, int iters, void* stream) {
  if (!out || blocks <= 0 || iters <= 0) { spx::set_error("spx_probe_fp64: bad argument"); return SPX_E_ARG; }
  spx::k_fp64_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>((double*)out, iters, 0.999999, 1e-7);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}
