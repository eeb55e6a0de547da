// spx_fxv.cu — f(x, v) from Hermite-Fourier coefficients (spectrax/_inverse_transform.py:97-125).
//
// The reference takes C = Re ifftn(ifftshift(Ck)) over (y, x, z) (1/N, no mask) and
// contracts it over the Hermite modes with the product basis
// b_n(xi_x) b_m(xi_y) b_p(xi_z) (mode index (p Nm + m) Nn + n), times
// exp(-(xi_x^2 + xi_y^2 + xi_z^2)).  Here:
//  * k_real_planes: one CTA per coefficient plane runs the inverse transform of
//    the FFT engine in shared memory (a plan that keeps every mode, so nothing is
//    pruned) and writes the real part / N in natural order;
//  * k_fxv_gemm: an FP64 GEMM over 64 x 64 output tiles (rows = (lead, point),
//    columns = velocity points), 16 modes per shared-memory step, 4 x 4 outputs per
//    thread; the basis entries are formed from the three per-axis bases while the
//    tile is staged and the Gaussian is applied in the epilogue.
#include <cuda_runtime.h>

#include "spx_core.cuh"
#include "spx_plan.h"
#include "spx_rhs.cuh"

namespace spx {

__global__ void __launch_bounds__(GEN_THREADS, 1) k_real_planes(const DevPlan* __restrict__ gP,
                                                                const double2* __restrict__ gtab,
                                                                const double2* __restrict__ Ck,
                                                                double* __restrict__ out) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const int pl = P.plane;
  const double2* src = Ck + (size_t)blockIdx.x * pl;
  // centred (fftshift) order in, standard order in shared memory (ifftshift)
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    sA[std_index(cy, Ny) * P.prow + std_index(cx, Nx) * Nz + std_index(cz, Nz)] = src[pt];
  }
  __syncthreads();
  const double2* r = fft_planes_t<true, false>(sA, sB, P, stab);
  const double sc = 1.0 / (double)pl;
  double* dst = out + (size_t)blockIdx.x * pl;
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) dst[pt] = sc * r[padded(P, pt)].x;
}

constexpr int FXV_TM = 64, FXV_TN = 64, FXV_TK = 16, FXV_THREADS = 256;

// f[(l, pt), v] = exp(-|xi_v|^2) sum_m C[(l, m), pt] bx[n, v] by[mm, v] bz[p, v],
// m = (p Nm + mm) Nn + n; C: nlead x modes x plane (real), rows = nlead * plane.
__global__ void __launch_bounds__(FXV_THREADS) k_fxv_gemm(const double* __restrict__ C, long long nlead, int modes,
                                                         int plane, int Nn, int Nm,
                                                         const double* __restrict__ bx,
                                                         const double* __restrict__ by,
                                                         const double* __restrict__ bz,
                                                         const double* __restrict__ xi, long long nv,
                                                         double* __restrict__ f) {
  __shared__ double As[FXV_TK][FXV_TM];
  __shared__ double Bs[FXV_TK][FXV_TN];
  const long long rows = nlead * (long long)plane;
  const long long r0 = (long long)blockIdx.x * FXV_TM, v0 = (long long)blockIdx.y * FXV_TN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;   // 16 x 16 threads, 4 x 4 outputs each
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < modes; k0 += FXV_TK) {
    for (int i = threadIdx.x; i < FXV_TK * FXV_TM; i += FXV_THREADS) {
      const int kk = i / FXV_TM, rr = i % FXV_TM;
      const long long r = r0 + rr;
      const int m = k0 + kk;
      double a = 0.0;
      if (r < rows && m < modes) {
        const long long l = r / plane, pt = r % plane;
        a = C[((size_t)l * modes + m) * plane + pt];
      }
      As[kk][rr] = a;
    }
    for (int i = threadIdx.x; i < FXV_TK * FXV_TN; i += FXV_THREADS) {
      const int kk = i / FXV_TN, cc = i % FXV_TN;
      const long long v = v0 + cc;
      const int m = k0 + kk;
      double b = 0.0;
      if (v < nv && m < modes) {
        const int n = m % Nn, mm = (m / Nn) % Nm, p = m / (Nn * Nm);
        b = bx[(size_t)n * nv + v] * by[(size_t)mm * nv + v] * bz[(size_t)p * nv + v];
      }
      Bs[kk][cc] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < FXV_TK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const long long v = v0 + tx + 16 * j;
    if (v >= nv) continue;
    const double x = xi[v], y = xi[nv + v], z = xi[2 * nv + v];
    const double g = exp(-(x * x + y * y + z * z));
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long r = r0 + ty + 16 * i;
      if (r < rows) f[(size_t)r * nv + v] = acc[i][j] * g;
    }
  }
}

}  // namespace spx

using namespace spx;

extern "C" {

size_t spx_fxv_workspace_bytes(const spx_plan* pl, int64_t nlead) {
  if (!pl || nlead < 0) return 0;
  return (size_t)nlead * pl->host.nh * pl->host.plane * sizeof(double);
}

int spx_fxv(const spx_plan* pl, const void* Ck, int64_t nlead, const double* bx, const double* by, const double* bz,
            const double* xi, int64_t nv, double* f, void* ws, size_t ws_bytes, void* stream) {
  if (!pl || !Ck || !bx || !by || !bz || !xi || !f || !ws || nlead < 1 || nv < 1) {
    set_error("spx_fxv: bad argument");
    return SPX_E_ARG;
  }
  if (int rd = check_plan_device(pl, "spx_fxv")) return rd;
  const DevPlan& P = pl->host;
  if (P.pb.Ns != 1) { set_error("spx_fxv: the plan must have one species (Ns = 1)"); return SPX_E_ARG; }
  for (int a = 0; a < 3; ++a)
    if (P.ax[a].n > 1 && 2 * P.ax[a].cut + 1 < P.ax[a].n) {
      set_error("spx_fxv: the plan must keep every Fourier mode (cut >= N/2 on every axis)");
      return SPX_E_ARG;
    }
  if (ws_bytes < spx_fxv_workspace_bytes(pl, nlead)) { set_error("spx_fxv: workspace too small"); return SPX_E_WORKSPACE; }
  if (((uintptr_t)Ck | (uintptr_t)ws) & 15) { set_error("spx_fxv: Ck and ws must be 16-byte aligned"); return SPX_E_ARG; }
  const size_t smem = pl->smem_tab + 2 * (size_t)P.pplane * sizeof(double2);
  if ((int)smem > smem_optin()) { set_error("spx_fxv: a plane does not fit in shared memory"); return SPX_E_UNSUPPORTED; }
  static bool attr = false;
  if (!attr) {
    cudaFuncAttributes fa;
    SPX_CUDA(cudaFuncGetAttributes(&fa, k_real_planes));
    SPX_CUDA(cudaFuncSetAttribute(k_real_planes, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin() - (int)fa.sharedSizeBytes));
    attr = true;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* C = static_cast<double*>(ws);
  const long long nplanes = nlead * (long long)P.nh;
  if (nplanes > 0x7fffffffLL) { set_error("spx_fxv: too many planes"); return SPX_E_UNSUPPORTED; }
  k_real_planes<<<(unsigned)nplanes, GEN_THREADS, smem, st>>>(pl->d_plan, pl->d_tab, static_cast<const double2*>(Ck), C);
  const long long rows = nlead * (long long)P.plane;
  dim3 grid((unsigned)((rows + FXV_TM - 1) / FXV_TM), (unsigned)((nv + FXV_TN - 1) / FXV_TN));
  if (grid.y > 65535) { set_error("spx_fxv: too many velocity points"); return SPX_E_UNSUPPORTED; }
  k_fxv_gemm<<<grid, FXV_THREADS, 0, st>>>(C, nlead, P.nh, P.plane, P.pb.Nn, P.pb.Nm, bx, by, bz, xi, nv, f);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

}  // extern "C"
