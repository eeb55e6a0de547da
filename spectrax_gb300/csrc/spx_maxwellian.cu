// spx_maxwellian.cu — Hermite-Fourier coefficients of drifting Maxwellians, on
// the device (spectrax/_initialize_maxwellian.py:15-66), for large initial states.
//
// The reference samples, per species s and Hermite mode (n, m, p),
//   C(x) = sqrt(2^(n+m+p) / (n! m! p!)) / (a_x^(n+1) a_y^(m+1) a_z^(p+1))
//          (U_x(x) - u_x)^n (U_y(x) - u_y)^m (U_z(x) - u_z)^p
// on the real-space grid and takes fftshift(fftn(C, norm="forward")) over
// (y, x, z).  Here one CTA per (species, mode) plane evaluates the samples as
//   c0 * ((U_x - u_x)/a_x)^n ((U_y - u_y)/a_y)^m ((U_z - u_z)/a_z)^p,
// c0 = sqrt(2^(n+m+p) / (n! m! p!)) / (a_x a_y a_z) from log-gamma on the host
// (finite where n! overflows), straight into shared memory, runs the forward
// transform of the FFT engine (a plan that keeps every mode, so nothing is
// pruned), scales by 1/N and writes the centred (fftshift) order.  Extra real
// planes (the fields E, B sampled on the grid) go through the same transform.
#include <cmath>
#include <cuda_runtime.h>
#include <vector>

#include "spx_core.cuh"
#include "spx_plan.h"
#include "spx_rhs.cuh"

namespace spx {

__global__ void __launch_bounds__(GEN_THREADS, 1) k_spectrum(const DevPlan* __restrict__ gP,
                                                             const double2* __restrict__ gtab,
                                                             const double* __restrict__ Us,
                                                             const double* __restrict__ c0,
                                                             const double* __restrict__ xr,
                                                             double2* __restrict__ out) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const int pl = P.plane;
  const int nplanes = P.pb.Ns * P.nh;
  const int id = blockIdx.x;
  if (id < nplanes) {
    const int s = id / P.nh, h = id % P.nh;
    const int Nn = P.pb.Nn, Nm = P.pb.Nm;
    const int n = h % Nn, m = (h / Nn) % Nm, p = h / (Nn * Nm);
    const double ia0 = 1.0 / P.pb.alpha_s[3 * s], ia1 = 1.0 / P.pb.alpha_s[3 * s + 1],
                 ia2 = 1.0 / P.pb.alpha_s[3 * s + 2];
    const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
    const double c = c0[id];
    const double* U = Us + (size_t)s * 3 * pl;
    for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) {
      const double wx = (U[pt] - u0) * ia0, wy = (U[pl + pt] - u1) * ia1, wz = (U[2 * pl + pt] - u2) * ia2;
      double v = c;
      for (int k = 0; k < n; ++k) v *= wx;
      for (int k = 0; k < m; ++k) v *= wy;
      for (int k = 0; k < p; ++k) v *= wz;
      sA[padded(P, pt)] = make_double2(v, 0.0);
    }
  } else {
    const double* X = xr + (size_t)(id - nplanes) * pl;
    for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) sA[padded(P, pt)] = make_double2(X[pt], 0.0);
  }
  __syncthreads();
  const double2* f = fft_planes_t<false, true>(sA, sB, P, stab);
  const double sc = 1.0 / (double)pl;
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    const int sidx = std_index(cy, Ny) * P.prow + std_index(cx, Nx) * Nz + std_index(cz, Nz);
    out[(size_t)id * pl + pt] = cscale(sc, f[sidx]);
  }
}

}  // namespace spx

using namespace spx;

extern "C" {

int spx_maxwellian(const spx_plan* pl, const double* Us, const double* xreal, int32_t nreal, void* out,
                   void* stream) {
  if (!pl || !Us || !out || nreal < 0 || (nreal > 0 && !xreal)) {
    set_error("spx_maxwellian: bad argument");
    return SPX_E_ARG;
  }
  if (int rd = check_plan_device(pl, "spx_maxwellian")) return rd;
  const DevPlan& P = pl->host;
  for (int a = 0; a < 3; ++a)
    if (P.ax[a].n > 1 && 2 * P.ax[a].cut + 1 < P.ax[a].n) {
      set_error("spx_maxwellian: the plan must keep every Fourier mode (cut >= N/2 on every axis)");
      return SPX_E_ARG;
    }
  const size_t smem = pl->smem_tab + 2 * (size_t)P.pplane * sizeof(double2);
  if ((int)smem > smem_optin()) { set_error("spx_maxwellian: a plane does not fit in shared memory"); return SPX_E_UNSUPPORTED; }
  static bool attr = false;
  if (!attr) {
    cudaFuncAttributes fa;
    SPX_CUDA(cudaFuncGetAttributes(&fa, k_spectrum));
    SPX_CUDA(cudaFuncSetAttribute(k_spectrum, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin() - (int)fa.sharedSizeBytes));
    attr = true;
  }
  // c0 per (species, mode): sqrt(2^(n+m+p) / (n! m! p!)) / (a_x a_y a_z), via log-gamma
  const int nplanes = P.pb.Ns * P.nh;
  std::vector<double> c0(std::max(1, nplanes));
  for (int id = 0; id < nplanes; ++id) {
    const int s = id / P.nh, h = id % P.nh;
    const int n = h % P.pb.Nn, m = (h / P.pb.Nn) % P.pb.Nm, p = h / (P.pb.Nn * P.pb.Nm);
    const double lg = 0.5 * ((n + m + p) * std::log(2.0) - std::lgamma(n + 1.0) - std::lgamma(m + 1.0) -
                             std::lgamma(p + 1.0));
    c0[id] = std::exp(lg) / (P.pb.alpha_s[3 * s] * P.pb.alpha_s[3 * s + 1] * P.pb.alpha_s[3 * s + 2]);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* d = nullptr;
  SPX_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), c0.size() * sizeof(double), st));
  cudaError_t e = cudaMemcpyAsync(d, c0.data(), c0.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_spectrum<<<nplanes + nreal, GEN_THREADS, smem, st>>>(pl->d_plan, pl->d_tab, Us, d, xreal,
                                                           static_cast<double2*>(out));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // c0 (host) is copied before returning
  cudaFreeAsync(d, st);
  if (e != cudaSuccess) return cuda_fail(e, "spx_maxwellian");
  return SPX_OK;
}

}  // extern "C"
