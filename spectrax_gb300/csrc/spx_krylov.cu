// spx_krylov.cu — Krylov-basis kernels of the implicit midpoint's restarted GMRES.
//
// The reference solves each Newton system with jax.scipy's GMRES
// (spectrax/midpoint_solver.py:37-98).  Here the basis V (rows of n complex128
// entries, row i at V + i*n) lives on the device; per Arnoldi step the new
// vector w is orthogonalised against the first k rows by classical Gram-Schmidt
// with one re-orthogonalisation pass:
//     h = V[:k]^H w;  w -= V[:k]^T h;  h2 = V[:k]^H w;  w -= V[:k]^T h2
// and the host receives h + h2 and ||w|| in one copy.  Only the k rows built so
// far are read (no work on the unused rows of the basis), the middle update and
// projection share one pass (three streaming passes in all for k <= 32), and
// the block partial sums are reduced in a fixed order, so results do not depend
// on scheduling.  The kernels are HBM-bound: one pass moves k*n*16 bytes (plus w).
#include <algorithm>
#include <cuda_runtime.h>

#include "spx_core.cuh"
#include "spx_plan.h"

namespace spx {

constexpr int KRY_GROUP = 8;   // rows per register group

static int kry_blocks(long long n) {
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 152;
  }
  const long long need = (n + NTHREADS - 1) / NTHREADS;
  return (int)std::max<long long>(1, std::min<long long>(need, 4LL * nsm));
}

// part[b*SPX_KRYLOV_MAX_ROWS + i] = sum over block b's entries of conj(V_i[e]) w[e], i < k
__global__ void __launch_bounds__(NTHREADS) k_kry_dots(const double2* __restrict__ V, long long n, int k,
                                                       const double2* __restrict__ w,
                                                       double2* __restrict__ part) {
  __shared__ double2 red[NTHREADS / 32][KRY_GROUP];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (int g0 = 0; g0 < k; g0 += KRY_GROUP) {
    double2 acc[KRY_GROUP];
#pragma unroll
    for (int r = 0; r < KRY_GROUP; ++r) acc[r] = make_double2(0.0, 0.0);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
      const double2 x = w[e];
#pragma unroll
      for (int r = 0; r < KRY_GROUP; ++r) {
        if (g0 + r < k) {
          const double2 v = __ldcs(V + (size_t)(g0 + r) * n + e);
          acc[r].x = fma(v.x, x.x, fma(v.y, x.y, acc[r].x));
          acc[r].y = fma(v.x, x.y, fma(-v.y, x.x, acc[r].y));
        }
      }
    }
#pragma unroll
    for (int r = 0; r < KRY_GROUP; ++r) {
      for (int off = 16; off > 0; off >>= 1) {
        acc[r].x += __shfl_down_sync(0xffffffffu, acc[r].x, off);
        acc[r].y += __shfl_down_sync(0xffffffffu, acc[r].y, off);
      }
      if (lane == 0) red[wid][r] = acc[r];
    }
    __syncthreads();
    if (threadIdx.x < KRY_GROUP && g0 + (int)threadIdx.x < k) {
      double2 s = make_double2(0.0, 0.0);
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s = cadd(s, red[q][threadIdx.x]);
      part[(size_t)blockIdx.x * SPX_KRYLOV_MAX_ROWS + g0 + threadIdx.x] = s;
    }
    __syncthreads();
  }
}

// out[i] = sum_b part[b*SPX_KRYLOV_MAX_ROWS + i], i < k: warp i sums its column, lane
// l the blocks b = l, l + 32, ... in order, then a fixed shuffle tree (deterministic)
constexpr int KRY_RED_THREADS = 1024;
__global__ void __launch_bounds__(KRY_RED_THREADS) k_kry_reduce(const double2* __restrict__ part, int nb, int k,
                                                                double2* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x >> 5; i < k; i += blockDim.x >> 5) {
    double2 s = make_double2(0.0, 0.0);
    for (int b = lane; b < nb; b += 32) s = cadd(s, part[(size_t)b * SPX_KRYLOV_MAX_ROWS + i]);
    for (int off = 16; off > 0; off >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, off);
      s.y += __shfl_down_sync(0xffffffffu, s.y, off);
    }
    if (lane == 0) out[i] = s;
  }
}

// x[e] += sign * sum_{i<k} c[i] V_i[e]; npart[b] = block b's sum of |x_new|^2 when npart != nullptr
__global__ void __launch_bounds__(NTHREADS) k_kry_update(const double2* __restrict__ V, long long n, int k,
                                                         const double2* __restrict__ c, double sign,
                                                         double2* __restrict__ x, double* __restrict__ npart) {
  __shared__ double2 sc[SPX_KRYLOV_MAX_ROWS];
  __shared__ double red[NTHREADS / 32];
  for (int i = threadIdx.x; i < k; i += blockDim.x) sc[i] = cscale(sign, c[i]);
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  double nrm = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
    double2 a = x[e];
    for (int g0 = 0; g0 < k; g0 += KRY_GROUP) {
      double2 v[KRY_GROUP];
#pragma unroll
      for (int r = 0; r < KRY_GROUP; ++r)
        v[r] = (g0 + r < k) ? __ldcs(V + (size_t)(g0 + r) * n + e) : make_double2(0.0, 0.0);
#pragma unroll
      for (int r = 0; r < KRY_GROUP; ++r)
        if (g0 + r < k) a = cfma(v[r], sc[g0 + r], a);
    }
    x[e] = a;
    nrm = fma(a.x, a.x, fma(a.y, a.y, nrm));
  }
  if (!npart) return;
  for (int off = 16; off > 0; off >>= 1) nrm += __shfl_down_sync(0xffffffffu, nrm, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nrm;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    npart[blockIdx.x] = s;
  }
}

// The middle two passes of CGS2 in one: x[e] -= sum_{i<k} c[i] V_i[e], then
// part[b*SPX_KRYLOV_MAX_ROWS + i] = block b's sum of conj(V_i[e]) x_new[e].  Each
// thread re-reads its own rows right after the update (L1), so the rows stream
// from memory once for both.  k <= 32 (four unrolled groups of eight rows).
__global__ void __launch_bounds__(NTHREADS) k_kry_update_dots(const double2* __restrict__ V, long long n, int k,
                                                              const double2* __restrict__ c,
                                                              double2* __restrict__ x, double2* __restrict__ part) {
  __shared__ double2 sc[32];
  __shared__ double2 red[NTHREADS / 32][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x < 32) sc[threadIdx.x] = threadIdx.x < k ? cscale(-1.0, c[threadIdx.x]) : make_double2(0.0, 0.0);
  __syncthreads();
  double2 acc[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) acc[i] = make_double2(0.0, 0.0);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
    double2 a = x[e];
#pragma unroll
    for (int g0 = 0; g0 < 32; g0 += KRY_GROUP) {
      if (g0 < k) {
        double2 v[KRY_GROUP];
#pragma unroll
        for (int r = 0; r < KRY_GROUP; ++r)
          v[r] = (g0 + r < k) ? V[(size_t)(g0 + r) * n + e] : make_double2(0.0, 0.0);
#pragma unroll
        for (int r = 0; r < KRY_GROUP; ++r)
          if (g0 + r < k) a = cfma(v[r], sc[g0 + r], a);
      }
    }
    x[e] = a;
#pragma unroll
    for (int g0 = 0; g0 < 32; g0 += KRY_GROUP) {
      if (g0 < k) {
#pragma unroll
        for (int r = 0; r < KRY_GROUP; ++r) {
          if (g0 + r < k) {
            const double2 v = __ldcs(V + (size_t)(g0 + r) * n + e);
            acc[g0 + r].x = fma(v.x, a.x, fma(v.y, a.y, acc[g0 + r].x));
            acc[g0 + r].y = fma(v.x, a.y, fma(-v.y, a.x, acc[g0 + r].y));
          }
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    if (i < k) {
      for (int off = 16; off > 0; off >>= 1) {
        acc[i].x += __shfl_down_sync(0xffffffffu, acc[i].x, off);
        acc[i].y += __shfl_down_sync(0xffffffffu, acc[i].y, off);
      }
      if (lane == 0) red[wid][i] = acc[i];
    }
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double2 sum = make_double2(0.0, 0.0);
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) sum = cadd(sum, red[q][threadIdx.x]);
    part[(size_t)blockIdx.x * SPX_KRYLOV_MAX_ROWS + threadIdx.x] = sum;
  }
}

// out[i] = h[i] + h2[i] (i < k), out[k] = (||w||, 0); warp 0 sums the norm
// partials (lane l: b = l, l + 32, ... in order, then a fixed shuffle tree)
__global__ void k_kry_finish(const double2* __restrict__ h, const double2* __restrict__ h2,
                             const double* __restrict__ npart, int nb, int k, double2* __restrict__ out) {
  const int i = threadIdx.x;
  if (i < k) out[i] = cadd(h[i], h2[i]);
  if (i < 32) {
    double s = 0.0;
    for (int b = i; b < nb; b += 32) s += npart[b];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (i == 0) out[k] = make_double2(sqrt(s), 0.0);
  }
}

// ---------------------------------------------------------------- implicit midpoint glue
// r[e] = y1[e] - y0[e] - dt f[e] (stored when r != nullptr); npart[b] = block b's
// sum of |r / (atol + rtol max(|y0|, |y1|))|^2, bpart[b] its count of non-finite r.
// With f = f(y_mid) this is the Newton residual of spectrax/midpoint_solver.py:48-50,
// with f = f(y0) the solver's error estimate y1 - y1_init (:51).
__global__ void __launch_bounds__(NTHREADS) k_mid_residual(long long n, const double2* __restrict__ y0,
                                                           const double2* __restrict__ y1,
                                                           const double2* __restrict__ f, double dt, double rtol,
                                                           double atol, double2* __restrict__ r,
                                                           double* __restrict__ npart, double* __restrict__ bpart) {
  __shared__ double red[2][NTHREADS / 32];
  const long long stride = (long long)gridDim.x * blockDim.x;
  double sq = 0.0, bad = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
    const double2 a = y0[e], b = y1[e], g = f[e];
    const double2 v = make_double2(fma(-dt, g.x, b.x - a.x), fma(-dt, g.y, b.y - a.y));
    if (r) r[e] = v;
    const double m0 = fma(a.x, a.x, a.y * a.y), m1 = fma(b.x, b.x, b.y * b.y);
    const double inv = 1.0 / fma(rtol, sqrt(fmax(m0, m1)), atol);
    const double rx = v.x * inv, ry = v.y * inv;
    sq = fma(rx, rx, fma(ry, ry, sq));
    if (!(isfinite(v.x) && isfinite(v.y))) bad += 1.0;
  }
  for (int off = 16; off > 0; off >>= 1) {
    sq += __shfl_down_sync(0xffffffffu, sq, off);
    bad += __shfl_down_sync(0xffffffffu, bad, off);
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = sq; red[1][threadIdx.x >> 5] = bad; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, c = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { s += red[0][q]; c += red[1][q]; }
    npart[blockIdx.x] = s;
    bpart[blockIdx.x] = c;
  }
}

// out[0] = sum of npart, out[1] = sum of bpart (lanes take blocks in order, then a
// fixed shuffle tree: deterministic)
__global__ void k_mid_sum2(const double* __restrict__ npart, const double* __restrict__ bpart, int nb,
                           double* __restrict__ out) {
  const int lane = threadIdx.x;
  double s = 0.0, c = 0.0;
  for (int b = lane; b < nb; b += 32) { s += npart[b]; c += bpart[b]; }
  for (int off = 16; off > 0; off >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, off);
    c += __shfl_down_sync(0xffffffffu, c, off);
  }
  if (lane == 0) { out[0] = s; out[1] = c; }
}

// y1 += sign * delta (when delta != nullptr); ymid = (y0 + y1) / 2
__global__ void __launch_bounds__(NTHREADS) k_mid_update(long long n, const double2* __restrict__ y0,
                                                         double2* __restrict__ y1,
                                                         const double2* __restrict__ delta, double sign,
                                                         double2* __restrict__ ymid) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += stride) {
    double2 b = y1[e];
    if (delta) {
      const double2 d = delta[e];
      b = make_double2(fma(sign, d.x, b.x), fma(sign, d.y, b.y));
      y1[e] = b;
    }
    const double2 a = y0[e];
    ymid[e] = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
  }
}

}  // namespace spx

using namespace spx;

extern "C" {

size_t spx_krylov_ws_bytes(int64_t n) {
  const size_t nb = (size_t)kry_blocks(n);
  return nb * SPX_KRYLOV_MAX_ROWS * sizeof(double2) + 2 * SPX_KRYLOV_MAX_ROWS * sizeof(double2) +
         nb * sizeof(double);
}

int spx_krylov_cgs2(const void* V, int64_t n, int32_t k, void* w, void* out, void* ws, size_t ws_bytes,
                    void* stream) {
  if (!V || !w || !out || !ws || n <= 0) { set_error("spx_krylov_cgs2: bad argument"); return SPX_E_ARG; }
  if (k < 1 || k > SPX_KRYLOV_MAX_ROWS) { set_error("spx_krylov_cgs2: k out of range"); return SPX_E_ARG; }
  if (((uintptr_t)V | (uintptr_t)w | (uintptr_t)out | (uintptr_t)ws) & 15) {
    set_error("spx_krylov_cgs2: pointers must be 16-byte aligned"); return SPX_E_ARG;
  }
  if (ws_bytes < spx_krylov_ws_bytes(n)) { set_error("spx_krylov_cgs2: workspace too small"); return SPX_E_WORKSPACE; }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = kry_blocks(n);
  const double2* Vp = static_cast<const double2*>(V);
  double2* wp = static_cast<double2*>(w);
  double2* part = static_cast<double2*>(ws);
  double2* h = part + (size_t)nb * SPX_KRYLOV_MAX_ROWS;
  double2* h2 = h + SPX_KRYLOV_MAX_ROWS;
  double* npart = reinterpret_cast<double*>(h2 + SPX_KRYLOV_MAX_ROWS);
  k_kry_dots<<<nb, NTHREADS, 0, st>>>(Vp, n, k, wp, part);
  k_kry_reduce<<<1, KRY_RED_THREADS, 0, st>>>(part, nb, k, h);
  if (k <= 32) {
    k_kry_update_dots<<<nb, NTHREADS, 0, st>>>(Vp, n, k, h, wp, part);
  } else {
    k_kry_update<<<nb, NTHREADS, 0, st>>>(Vp, n, k, h, -1.0, wp, nullptr);
    k_kry_dots<<<nb, NTHREADS, 0, st>>>(Vp, n, k, wp, part);
  }
  k_kry_reduce<<<1, KRY_RED_THREADS, 0, st>>>(part, nb, k, h2);
  k_kry_update<<<nb, NTHREADS, 0, st>>>(Vp, n, k, h2, -1.0, wp, npart);
  k_kry_finish<<<1, SPX_KRYLOV_MAX_ROWS, 0, st>>>(h, h2, npart, nb, k, static_cast<double2*>(out));
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_midpoint_residual(int64_t n, const void* y0, const void* y1, const void* f, double dt, double rtol,
                          double atol, void* r, double* sums, void* ws, size_t ws_bytes, void* stream) {
  if (!y0 || !y1 || !f || !sums || !ws || n <= 0) { set_error("spx_midpoint_residual: bad argument"); return SPX_E_ARG; }
  if (((uintptr_t)y0 | (uintptr_t)y1 | (uintptr_t)f | (uintptr_t)r | (uintptr_t)ws) & 15) {
    set_error("spx_midpoint_residual: pointers must be 16-byte aligned"); return SPX_E_ARG;
  }
  if (ws_bytes < spx_krylov_ws_bytes(n)) { set_error("spx_midpoint_residual: workspace too small"); return SPX_E_WORKSPACE; }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = kry_blocks(n);
  // the first 2 nb doubles of the Krylov workspace (its block-partial area)
  double* npart = static_cast<double*>(ws);
  double* bpart = npart + nb;
  k_mid_residual<<<nb, NTHREADS, 0, st>>>(n, static_cast<const double2*>(y0), static_cast<const double2*>(y1),
                                          static_cast<const double2*>(f), dt, rtol, atol, static_cast<double2*>(r),
                                          npart, bpart);
  k_mid_sum2<<<1, 32, 0, st>>>(npart, bpart, nb, sums);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_midpoint_update(int64_t n, const void* y0, void* y1, const void* delta, double sign, void* ymid,
                        void* stream) {
  if (!y0 || !y1 || !ymid || n <= 0) { set_error("spx_midpoint_update: bad argument"); return SPX_E_ARG; }
  if (((uintptr_t)y0 | (uintptr_t)y1 | (uintptr_t)delta | (uintptr_t)ymid) & 15) {
    set_error("spx_midpoint_update: pointers must be 16-byte aligned"); return SPX_E_ARG;
  }
  k_mid_update<<<kry_blocks(n), NTHREADS, 0, static_cast<cudaStream_t>(stream)>>>(
      n, static_cast<const double2*>(y0), static_cast<double2*>(y1), static_cast<const double2*>(delta), sign,
      static_cast<double2*>(ymid));
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_krylov_axpy(const void* V, int64_t n, int32_t k, const void* c, void* x, void* stream) {
  if (!V || !c || !x || n <= 0) { set_error("spx_krylov_axpy: bad argument"); return SPX_E_ARG; }
  if (k < 1 || k > SPX_KRYLOV_MAX_ROWS) { set_error("spx_krylov_axpy: k out of range"); return SPX_E_ARG; }
  if (((uintptr_t)V | (uintptr_t)c | (uintptr_t)x) & 15) {
    set_error("spx_krylov_axpy: pointers must be 16-byte aligned"); return SPX_E_ARG;
  }
  k_kry_update<<<kry_blocks(n), NTHREADS, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const double2*>(V), n, k, static_cast<const double2*>(c), 1.0, static_cast<double2*>(x), nullptr);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

}  // extern "C"
