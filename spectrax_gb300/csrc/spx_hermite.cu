// spx_hermite.cu — normalised Hermite basis on a velocity grid, for the
// reconstruction of f(x, v) from Hermite-Fourier coefficients
// (spectrax/_inverse_transform.py:97-125).
//
// The reference evaluates the physicists' polynomials H_n(xi) with a Clenshaw
// sum (orthax hermval, :20-38) and divides by sqrt(pi) 2^(n/2) sqrt(n!) per axis
// (:79-84).  H_n itself overflows double precision for large n at moderate xi,
// so here each point runs the three-term recurrence of the normalised functions
//     psi_0 = 1,  psi_1 = sqrt(2) xi,
//     psi_{n+1} = sqrt(2/(n+1)) xi psi_n - sqrt(n/(n+1)) psi_{n-1},
// psi_n = H_n / sqrt(2^n n!), and writes b_n(xi) = psi_n(xi) / sqrt(pi): the same
// numbers where the reference's are finite.  One thread per grid point, the
// recurrence coefficients are computed once on the host.
#include <cmath>
#include <cuda_runtime.h>
#include <vector>

#include "spx_core.cuh"
#include "spx_plan.h"

namespace spx {

// out[n * nv + j] = b_n(xi[j]), n < N; c1[n] = sqrt(2/(n+1)), c2[n] = sqrt(n/(n+1))
__global__ void __launch_bounds__(NTHREADS) k_hermite_basis(int N, const double* __restrict__ xi, long long nv,
                                                            const double* __restrict__ c1,
                                                            const double* __restrict__ c2,
                                                            double* __restrict__ out) {
  const double rpi = 0.56418958354775628695;   // 1 / sqrt(pi)
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nv; j += (long long)gridDim.x * blockDim.x) {
    const double x = xi[j];
    double pm = 0.0, p = 1.0;                  // psi_{n-1}, psi_n
    for (int n = 0; n < N; ++n) {
      out[(size_t)n * nv + j] = p * rpi;
      const double pn = fma(c1[n] * x, p, -c2[n] * pm);
      pm = p;
      p = pn;
    }
  }
}

}  // namespace spx

using namespace spx;

extern "C" {

int spx_hermite_basis(int32_t N, const double* xi, int64_t nv, double* out, void* stream) {
  if (N < 0 || nv < 0 || (nv > 0 && (!xi || !out))) { set_error("spx_hermite_basis: bad argument"); return SPX_E_ARG; }
  if (N == 0 || nv == 0) return SPX_OK;
  // recurrence coefficients (host, IEEE square roots), in one small device buffer
  std::vector<double> c(2 * (size_t)N);
  for (int n = 0; n < N; ++n) {
    c[n] = std::sqrt(2.0 / (double)(n + 1));
    c[N + n] = std::sqrt((double)n / (double)(n + 1));
  }
  double* d = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SPX_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), c.size() * sizeof(double), st));
  cudaError_t e = cudaMemcpyAsync(d, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const int grid = (int)std::min<long long>((nv + NTHREADS - 1) / NTHREADS, 152LL * 8);
    k_hermite_basis<<<grid, NTHREADS, 0, st>>>(N, xi, nv, d, d + N, out);
    e = cudaGetLastError();
  }
  // the host vector must outlive the copy; the buffer is freed in stream order
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(d, st);
  if (e != cudaSuccess) return cuda_fail(e, "spx_hermite_basis");
  return SPX_OK;
}

}  // extern "C"
