// spx_noalloc.cu — allocation-free variant of the 1D1V vector-Jacobian product.
//
// spx_vjp needs a caller-provided workspace for its per-tile partial sums of the
// field gradient.  Some callers cannot allocate device memory at the point where
// they need the VJP: code that records the adjoint sweep into a CUDA stream
// capture (cudaMalloc is not a capturable operation), real-time loops that must
// not allocate after start-up, and host frameworks that own every device byte
// through their own pool.  spx_vjp_noalloc keeps that scratch in a fixed
// file-scope __device__ array instead, so the call itself allocates nothing.
//
// Limits and sharing rules:
//  * the scratch holds SPX_VJP_NOALLOC_MAX_ENTRIES complex128 values (1 MiB);
//    problems that need more (Ns * tiles * Nx entries) are rejected with
//    SPX_E_UNSUPPORTED;
//  * every GPU that loads this library keeps the array until the process exits;
//  * all calls share the one array, so calls whose kernels overlap on the GPU
//    (different streams, or different host threads) race; serialise them;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) and sets the kernels' shared-memory limits; make
//    that first call before any stream capture.
//  * nothing needs to start at zero: every call writes each scratch entry it
//    later reads, so the contents left by an earlier call are never used.
#include <mutex>

#include "spx_plan.h"
#include "spx_rhs.cuh"

namespace spx {

// Scratch for the per-(species, tile) partial field-gradient lines.
static __device__ __align__(256) double2 g_vjp_scratch[SPX_VJP_NOALLOC_MAX_ENTRIES];

__global__ void __launch_bounds__(NTHREADS, 2) k_vjp1v_static(const DevPlan* __restrict__ gP,
                                                           const double2* __restrict__ gtab,
                                                           const double2* __restrict__ y,
                                                           const double2* __restrict__ w,
                                                           double2* __restrict__ g,
                                                           double2* __restrict__ part) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const int s = blockIdx.x / P.ntiles, tile = blockIdx.x % P.ntiles;
  const int m0 = tile * P.tile;
  const int nt = min(P.tile, P.pb.Nn - m0);
  const int N = P.ax[1].n;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)(2 * P.tile + 2) * N;
  double* scoef = reinterpret_cast<double*>(sB + (size_t)(2 * P.tile + 2) * N);
  if (nt <= 0) {
    for (int x = threadIdx.x; x < N; x += blockDim.x)
      part[((size_t)s * P.ntiles + tile) * N + x] = make_double2(0.0, 0.0);
    return;
  }
  vjp1v_tile(P, stab, y, w, g, part, s, tile, m0, nt, sA, sB, scoef);
}

__global__ void __launch_bounds__(NTHREADS, 2) k_vjp1v_fields_static(const DevPlan* __restrict__ gP,
                                                                  const double2* __restrict__ gtab,
                                                                  const double2* __restrict__ w,
                                                                  double2* __restrict__ g,
                                                                  const double2* __restrict__ part) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const int N = P.ax[1].n;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)P.pb.Ns * N;
  vjp1v_fields(P, stab, w, g, part, sA, sB);
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double2* g_scratch_dev[kMaxDevices] = {};   // device address of g_vjp_scratch, per device

// Once per device, with that device current: look up the array's device
// address (the host-side name is only a stand-in) and allow the kernels their
// dynamic shared memory.
int setup_device(int dev, double2** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (dev < 0 || dev >= kMaxDevices) { set_error("spx_vjp_noalloc: device ordinal out of range"); return SPX_E_ARG; }
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_vjp_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_vjp_scratch)");
    const int optin = smem_optin();
    if (optin <= 0) { set_error("spx_vjp_noalloc: cannot query shared memory limit"); return SPX_E_CUDA; }
    cudaFuncAttributes fa;
    SPX_CUDA(cudaFuncGetAttributes(&fa, k_vjp1v_static));
    SPX_CUDA(cudaFuncSetAttribute(k_vjp1v_static, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes));
    SPX_CUDA(cudaFuncGetAttributes(&fa, k_vjp1v_fields_static));
    SPX_CUDA(cudaFuncSetAttribute(k_vjp1v_fields_static, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes));
    g_scratch_dev[dev] = static_cast<double2*>(p);
  }
  *out = g_scratch_dev[dev];
  return SPX_OK;
}
}  // namespace

}  // namespace spx

using namespace spx;

extern "C" int spx_vjp_noalloc(const spx_plan* pl, const void* y, const void* w, void* g, void* stream) {
  if (!pl || !y || !w || !g) { set_error("spx_vjp_noalloc: null argument"); return SPX_E_ARG; }
  if (g == y || g == w) { set_error("spx_vjp_noalloc: output must not alias an input"); return SPX_E_ARG; }
  if (((uintptr_t)y | (uintptr_t)w | (uintptr_t)g) & 15) {
    set_error("spx_vjp_noalloc: pointers must be 16-byte aligned"); return SPX_E_ARG;
  }
  const DevPlan& P = pl->host;
  if (P.path != 0) {
    set_error("spx_vjp_noalloc: only the 1D1V layout (Ny = Nz = Nm = Np = 1) is supported");
    return SPX_E_UNSUPPORTED;
  }
  const size_t need = (size_t)P.pb.Ns * P.ntiles * P.ax[1].n;
  if (need > (size_t)SPX_VJP_NOALLOC_MAX_ENTRIES) {
    set_error("spx_vjp_noalloc: problem needs " + std::to_string(need) +
              " scratch entries (Ns * Hermite tiles * Nx), more than the fixed maximum of " +
              std::to_string((long long)SPX_VJP_NOALLOC_MAX_ENTRIES) + "; use spx_vjp with a workspace");
    return SPX_E_UNSUPPORTED;
  }
  // the scratch address is per device: the plan's device must be current
  if (int rd = check_plan_device(pl, "spx_vjp_noalloc")) return rd;
  double2* scratch = nullptr;
  int rc = setup_device(pl->device, &scratch);
  if (rc != SPX_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_vjp1v_static<<<P.pb.Ns * P.ntiles, pl->threads, pl->smem_1v, st>>>(
      pl->d_plan, pl->d_tab, static_cast<const double2*>(y), static_cast<const double2*>(w),
      static_cast<double2*>(g), scratch);
  k_vjp1v_fields_static<<<1, pl->threads, pl->smem_1v, st>>>(pl->d_plan, pl->d_tab,
                                                          static_cast<const double2*>(w),
                                                          static_cast<double2*>(g), scratch);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}
