// spx_adjoint.cu — building blocks of the discrete adjoint of the Dopri8 step.
//
//  * spx_rk_step_store: one fixed Runge-Kutta step that keeps every stage input
//    Y_j and stage derivative K_j = f(Y_j) (the backward sweep linearises at Y_j);
//  * spx_lincomb: out = sum_i c_i v_i (real c_i), the adjoint recursion's combinations;
//  * spx_param_dots: accumulates Re sum_e g_e (df/dtheta)_e for the parameters
//    theta = (nu, k, u_x of each species) of a 1D1V problem.
#include <algorithm>
#include <cstring>

#include "spx_plan.h"
#include "spx_rhs.cuh"
#include "spx_tableau.cuh"

namespace spx {

__constant__ double aCoef[13][13];   // a(i, j)
__constant__ double aB[13];
__constant__ int aMask[13];

// Stage epilogue: store K_j, write the next stage input Y_{j+1} = y + h sum_{l<=j} a(j+1, l) K_l.
struct EpiStore2 {
  const double2* y;
  double2* Kb;
  double2* Yb;
  double2* ynext;   // written by the last stage: y + h sum b_l K_l
  long long len;
  int stage;
  double h;
  __device__ __forceinline__ void operator()(size_t e, double2 v) const {
    Kb[(size_t)stage * len + e] = v;
    double2 acc = y[e];
    if (stage < rk::S - 1) {
      const int row = stage + 1;
      const int mask = aMask[row];
      for (int j = 0; j < stage; ++j)
        if (mask & (1 << j)) acc = crfma(h * aCoef[row][j], Kb[(size_t)j * len + e], acc);
      acc = crfma(h * aCoef[row][stage], v, acc);
      Yb[(size_t)(stage + 1) * len + e] = acc;
    } else {
      for (int j = 0; j < stage; ++j)
        if (aB[j] != 0.0) acc = crfma(h * aB[j], Kb[(size_t)j * len + e], acc);
      acc = crfma(h * aB[stage], v, acc);
      ynext[e] = acc;
    }
  }
};

__global__ void __launch_bounds__(NTHREADS) k_rk_stage_1v(const DevPlan* __restrict__ gP,
                                                          const double2* __restrict__ gtab,
                                                          const double2* y, double2* Yb, double2* Kb,
                                                          double2* ynext, double h, int stage) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const long long len = P.nc + 6LL * P.plane;
  EpiStore2 epi{y, Kb, Yb, ynext, len, stage, h};
  const double2* in = Yb + (size_t)stage * len;
  const int nblk = P.pb.Ns * P.ntiles;
  if ((int)blockIdx.x == nblk) {
    maxwell_range(P, stab, in, 0, P.plane, epi);
    return;
  }
  const int s = blockIdx.x / P.ntiles, tile = blockIdx.x % P.ntiles;
  const int n0 = tile * P.tile;
  const int nt = min(P.tile, P.pb.Nn - n0);
  if (nt <= 0) return;
  const int N = P.ax[1].n;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)(2 * P.tile + 2) * N;
  double* scoef = reinterpret_cast<double*>(sB + (size_t)(2 * P.tile + 2) * N);
  rhs1v_tile(P, stab, in, s, n0, nt, sA, sB, scoef, epi);
}

struct LinTerms {
  const double2* v[16];
  double c[16];
  int n;
};

__global__ void k_lincomb(LinTerms t, double2* __restrict__ out, long long len) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < t.n; ++k) acc = crfma(t.c[k], t.v[k][i], acc);
    out[i] = acc;
  }
}

// acc[0] += Re sum g . (-col C)            (d/dnu)
// acc[1] += Re sum g . f_K(y)               (k d/dk: the parts of f linear in K)
// acc[2+s] += Re sum g . (d f / d u_x,s)
__global__ void __launch_bounds__(NTHREADS) k_param_dots_1v(const DevPlan* __restrict__ gP,
                                                            const double2* __restrict__ gtab,
                                                            const double2* __restrict__ y,
                                                            const double2* __restrict__ g,
                                                            double* __restrict__ acc) {
  __shared__ DevPlan P;
  __shared__ double red[NTHREADS / 32][2 + SPX_MAX_SPECIES];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const int N = P.ax[1].n, Nn = P.pb.Nn, Ns = P.pb.Ns;
  const long long nC = P.nc;
  double loc[2 + SPX_MAX_SPECIES];
  for (int k = 0; k < 2 + SPX_MAX_SPECIES; ++k) loc[k] = 0.0;
  const double iO = 1.0 / P.pb.Omega_cs[0];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nC + 6LL * N;
       e += (long long)gridDim.x * blockDim.x) {
    const double2 ge = g[e];
    if (e < nC) {
      const int c = (int)(e % N);
      const int n = (int)((e / N) % Nn);
      const int s = (int)(e / ((long long)N * Nn));
      const double a0 = P.pb.alpha_s[3 * s], u0 = P.pb.u_s[3 * s];
      const double2 C0 = y[e];
      const double2 Cp = (n + 1 < Nn) ? y[e + N] : make_double2(0.0, 0.0);
      const double2 Cm = (n >= 1) ? y[e - N] : make_double2(0.0, 0.0);
      const double K = ktab(P, stab, 1, c).x;
      // nu: -col(n) C
      const double col = colc(Nn, n);
      loc[0] += -col * (ge.x * C0.x - ge.y * C0.y);
      // streaming -i K a0 t  with t = sqrt((n+1)/2) C+ + sqrt(n/2) C- + (u0/a0) C
      double2 t = cscale(u0 / a0, C0);
      t = crfma(sqrt((n + 1) * 0.5), Cp, t);
      t = crfma(sqrt(n * 0.5), Cm, t);
      const double w = K * a0;
      const double2 fk = make_double2(w * t.y, -w * t.x);
      loc[1] += ge.x * fk.x - ge.y * fk.y;
      // u_x,s: -i K C
      const double2 fu = make_double2(K * C0.y, -K * C0.x);
      loc[2 + s] += ge.x * fu.x - ge.y * fu.y;
    } else {
      const int f = (int)((e - nC) / N), c = (int)((e - nC) % N);
      const double K = ktab(P, stab, 1, c).x;
      const double2* F = y + nC;
      // curl parts with K = (Kx, 0, 0): dE_y = -i Kx B_z, dE_z = i Kx B_y, dB_y = i Kx E_z, dB_z = -i Kx E_y
      double2 fk = make_double2(0.0, 0.0);
      if (f == 1) { const double2 b = F[5 * N + c]; fk = make_double2(K * b.y, -K * b.x); }
      else if (f == 2) { const double2 b = F[4 * N + c]; fk = make_double2(-K * b.y, K * b.x); }
      else if (f == 4) { const double2 ez = F[2 * N + c]; fk = make_double2(-K * ez.y, K * ez.x); }
      else if (f == 5) { const double2 ey = F[N + c]; fk = make_double2(K * ey.y, -K * ey.x); }
      loc[1] += ge.x * fk.x - ge.y * fk.y;
      if (f == 0) {
        // dE_x = -J_x / Omega_0 with J_x containing q a0 a1 a2 u_x C_{s,000}
        for (int s = 0; s < Ns; ++s) {
          const double pre = P.pb.qs[s] * P.pb.alpha_s[3 * s] * P.pb.alpha_s[3 * s + 1] * P.pb.alpha_s[3 * s + 2];
          const double2 C000 = y[(size_t)s * Nn * N + c];
          loc[2 + s] += -pre * iO * (ge.x * C000.x - ge.y * C000.y);
        }
      }
    }
  }
  // block reduction of the 2 + Ns sums
  for (int k = 0; k < 2 + Ns; ++k) {
    double v = loc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2 + Ns) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
    atomicAdd(acc + threadIdx.x, v);
  }
}

static int adj_setup() {
  static bool done = false;
  if (done) return SPX_OK;
  double c[13][13];
  double b[13];
  int m[13];
  std::memset(c, 0, sizeof(c));
  for (int i = 0; i < 13; ++i) {
    m[i] = 0;
    for (int j = 0; j < i; ++j) {
      c[i][j] = rk::A(i, j);
      if (c[i][j] != 0.0) m[i] |= 1 << j;
    }
    b[i] = rk::B(i);
  }
  SPX_CUDA(cudaMemcpyToSymbol(aCoef, c, sizeof(c)));
  SPX_CUDA(cudaMemcpyToSymbol(aB, b, sizeof(b)));
  SPX_CUDA(cudaMemcpyToSymbol(aMask, m, sizeof(m)));
  const int optin = smem_optin();
  cudaFuncAttributes fa;
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_rk_stage_1v));
  SPX_CUDA(cudaFuncSetAttribute(k_rk_stage_1v, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_param_dots_1v));
  SPX_CUDA(cudaFuncSetAttribute(k_param_dots_1v, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  done = true;
  return SPX_OK;
}

}  // namespace spx

using namespace spx;

extern "C" {

int spx_rk_step_store(const spx_plan* pl, const void* y, double h, void* Ystages, void* Kstages, void* ynext,
                      void* stream) {
  if (!pl || !y || !Ystages || !Kstages || !ynext) { set_error("spx_rk_step_store: null argument"); return SPX_E_ARG; }
  if (pl->host.path != 0) {
    set_error("spx_rk_step_store: only the 1D1V layout (Ny = Nz = Nm = Np = 1) is supported");
    return SPX_E_UNSUPPORTED;
  }
  int rc = adj_setup();
  if (rc != SPX_OK) return rc;
  const DevPlan& P = pl->host;
  const long long len = P.nc + 6LL * P.plane;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2* Yb = static_cast<double2*>(Ystages);
  if (static_cast<const void*>(Yb) != y)
    SPX_CUDA(cudaMemcpyAsync(Yb, y, sizeof(double2) * len, cudaMemcpyDeviceToDevice, st));
  for (int stage = 0; stage < rk::S; ++stage)
    k_rk_stage_1v<<<P.pb.Ns * P.ntiles + 1, pl->threads, pl->smem_1v, st>>>(
        pl->d_plan, pl->d_tab, static_cast<const double2*>(y), Yb, static_cast<double2*>(Kstages),
        static_cast<double2*>(ynext), h, stage);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_lincomb(int64_t len, int32_t nterms, const void* const* vecs, const double* coefs, void* out,
                void* stream) {
  if (len < 0 || nterms < 0 || nterms > 16 || !out || (nterms && (!vecs || !coefs))) {
    set_error("spx_lincomb: bad argument (at most 16 terms)");
    return SPX_E_ARG;
  }
  LinTerms t;
  std::memset(&t, 0, sizeof(t));
  t.n = nterms;
  for (int i = 0; i < nterms; ++i) {
    t.v[i] = static_cast<const double2*>(vecs[i]);
    t.c[i] = coefs[i];
  }
  const int threads = 256;
  const long long blocks = std::min<long long>((len + threads - 1) / threads, 152LL * 8);
  k_lincomb<<<(int)std::max<long long>(blocks, 1), threads, 0, static_cast<cudaStream_t>(stream)>>>(
      t, static_cast<double2*>(out), len);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_param_dots(const spx_plan* pl, const void* y, const void* g, double* acc, void* stream) {
  if (!pl || !y || !g || !acc) { set_error("spx_param_dots: null argument"); return SPX_E_ARG; }
  if (pl->host.path != 0) {
    set_error("spx_param_dots: only the 1D1V layout is supported");
    return SPX_E_UNSUPPORTED;
  }
  int rc = adj_setup();
  if (rc != SPX_OK) return rc;
  const DevPlan& P = pl->host;
  const long long len = P.nc + 6LL * P.plane;
  const int blocks = (int)std::min<long long>((len + NTHREADS - 1) / NTHREADS, 152LL * 2);
  k_param_dots_1v<<<std::max(blocks, 1), NTHREADS, pl->smem_tab, static_cast<cudaStream_t>(stream)>>>(
      pl->d_plan, pl->d_tab, static_cast<const double2*>(y), static_cast<const double2*>(g), acc);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

}  // extern "C"
