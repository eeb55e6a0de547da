// spx_plan.h — host-side plan object shared by the translation units of the library.
#pragma once
#include <string>
#include <vector>
#include "spx_core.cuh"

struct spx_plan {
  spx::DevPlan host;            // host copy of the device header
  std::vector<double2> tab;     // host copy of the table
  std::vector<double> coef;     // fused 1D1V path: coef_1v for every (species, plane)
  std::vector<unsigned char> gen;   // general path: GenPlane for every (species, plane), as bytes
  spx::DevPlan* d_plan = nullptr;
  double2* d_tab = nullptr;
  void* d_block = nullptr;      // single allocation holding d_plan, d_tab and d_ticket
  unsigned int* d_ticket = nullptr;  // zero between launches: tickets of spx_vjp_param ([0] completion,
                                     // [64 + g] group g of 8 Hermite tiles)
  int device = 0;
  int nsm = 0;
  size_t smem_tab = 0;          // bytes of the table in shared memory
  size_t smem_1v = 0;           // dynamic smem of the fused 1D1V kernel
  size_t smem_gen = 0;          // dynamic smem of the general kernels
  size_t ws_bytes = 0;          // scratch of spx_rhs
  int threads = 256;            // CTA width of the right-hand-side kernels (<= 256)
  bool herm_ok = false;         // fused 1D1V path, odd Nx, antisymmetric k table: packed transforms valid
  // general layout whose plane does not fit in one CTA's shared memory: spx_rhs
  // runs the multi-pass kernels (line batches of big_nl lines, smem_big bytes)
  bool big = false;
  int big_nl = 0;
  size_t smem_big = 0;
};

namespace spx {
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
// Fill `pl` (everything but the device pointers) from a problem; returns SPX_OK or an error code.
// mgrid (fused 1D1V path): 0 = products on the Nx-point grid, 1 = the stepper's
// product grid may be any cheaper length, 2 = only one no longer than Nx.
int build_plan_host(const spx_problem* pb, int nsm, spx_plan* pl, int tile = 0, int mgrid = 1);
// Launch helpers used by several entry points.
int launch_rhs(const spx_plan* pl, const double2* y, double2* dy, double2* ws, cudaStream_t st);
// Opt-in shared memory per block of the current device (0 on failure).
int smem_optin();
// SPX_OK when the calling thread's current device is the one the plan was created
// on; otherwise SPX_E_ARG (the plan's tables, and any per-device scratch, live there).
int check_plan_device(const spx_plan* pl, const char* who);
}  // namespace spx

namespace spx {
// Launch with a programmatic dependency on the previous kernel in the stream, so
// its prologue overlaps the tail of that kernel.
template <class... Args>
inline cudaError_t launch_pdl(void (*k)(Args...), int grid, int threads, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}
}  // namespace spx

#define SPX_CUDA(call)                                         \
  do {                                                         \
    cudaError_t e__ = (call);                                  \
    if (e__ != cudaSuccess) return spx::cuda_fail(e__, #call); \
  } while (0)
