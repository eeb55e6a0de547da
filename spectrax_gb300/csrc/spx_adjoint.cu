// spx_adjoint.cu — building blocks of the discrete adjoint of the Dopri8 step.
//
//  * spx_rk_step_store: one fixed Runge-Kutta step that keeps every stage input
//    Y_j and stage derivative K_j = f(Y_j) (the backward sweep linearises at Y_j),
//    with the same staged stage kernels as the device Dopri8 solver, so a
//    recomputed step reproduces the forward solve's arithmetic;
//  * spx_lincomb: out = sum_i c_i v_i (real c_i), the adjoint recursion's combinations;
//  * spx_param_dots: accumulates Re sum_e g_e (df/dtheta)_e for the parameters
//    theta = (nu, k, u_x of each species) of a 1D1V problem.
#include <algorithm>
#include <cstring>

#include "spx_plan.h"
#include "spx_rhs.cuh"
#include "spx_stage.cuh"
#include "spx_tableau.cuh"

namespace spx {

__constant__ double aCoef[13][13];   // a(i, j)
__constant__ double aB[13];
__constant__ int aMask[13];

// Status of the staged recomputation (SPX_ST_WAIT_TIMEOUT if a bounded wait gave up).
__device__ int g_rk_status;

// Stage term list for a fixed step h: stage i < 12 forms y + h sum_j a(i+1, j) K_j
// (j < i, nonzero) + h a(i+1, i) K_i; the last stage y + h sum_j b_j K_j + h b_12 K_12.
__device__ void fill_terms_fixed(EpiTerms& T, int stage, double h) {
  T.n = 0;
  if (stage < rk::S - 1) {
    const int row = stage + 1, mask = aMask[row];
    for (int j = 0; j < stage; ++j)
      if (mask & (1 << j)) { T.j[T.n] = j; T.c[T.n] = h * aCoef[row][j]; T.e[T.n] = 0.0; ++T.n; }
    T.cself = h * aCoef[row][stage];
  } else {
    for (int j = 0; j < stage; ++j)
      if (aB[j] != 0.0) { T.j[T.n] = j; T.c[T.n] = h * aB[j]; T.e[T.n] = 0.0; ++T.n; }
    T.cself = h * aB[stage];
  }
  T.eself = 0.0;
}

template <bool LAST, bool HERM>
__global__ void __launch_bounds__(NTHREADS, 2) k_rk_stage_st(const DevPlan* __restrict__ gP,
                                                            const double2* __restrict__ gtab,
                                                            const double2* y, double2* Yb, double2* Kb,
                                                            double2* ynext, double h, int stage, int npf) {
  __shared__ DevPlan P;
  __shared__ EpiTerms terms;
  __shared__ __align__(8) uint64_t bars[2];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  if (threadIdx.x == 0) fill_terms_fixed(terms, stage, h);
  pdl_wait_and_release();
  __syncthreads();
  const long long len = P.nc + 6LL * P.plane;
  StageIO io;
  io.in = Yb + (size_t)stage * len;
  io.Y = y;
  io.K = Kb;
  io.len = len;
  io.Ki = Kb + (size_t)stage * len;
  io.out = LAST ? ynext : Yb + (size_t)(stage + 1) * len;
  io.npf = npf;
  io.herm = HERM;
  io.rtol = io.atol = 0.0;
  io.adaptive = 0;
  io.timeout_status = &g_rk_status;
  io.persistent = false;
  staged_stage_1v<LAST, HERM ? 1 : 0>(P, stab, io, terms, bars, [](auto&) {});
}

struct LinTerms {
  const double2* v[16];
  double c[16];
  int n;
};

__global__ void k_lincomb(LinTerms t, double2* __restrict__ out, long long len) {
  pdl_wait_and_release();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < t.n; ++k) acc = crfma(t.c[k], t.v[k][i], acc);
    out[i] = acc;
  }
}

// Parameter sensitivities of one entry e of f(y) contracted with g:
//   loc[0] += Re g . (-col C)            (d/dnu)
//   loc[1] += Re g . f_K(y)               (k d/dk: the parts of f linear in K)
//   loc[2+s] += Re g . (d f / d u_x,s)
__device__ __forceinline__ void param_terms(const DevPlan& P, const double2* __restrict__ tab,
                                            const double2* __restrict__ y, const double2 ge, long long e,
                                            double* loc) {
  const int N = P.ax[1].n, Nn = P.pb.Nn, Ns = P.pb.Ns;
  const long long nC = P.nc;
  if (e < nC) {
    const int c = (int)(e % N);
    const int n = (int)((e / N) % Nn);
    const int s = (int)(e / ((long long)N * Nn));
    const double a0 = P.pb.alpha_s[3 * s];
    const double2 C0 = y[e];
    const double2 Cp = (n + 1 < Nn) ? y[e + N] : make_double2(0.0, 0.0);
    const double2 Cm = (n >= 1) ? y[e - N] : make_double2(0.0, 0.0);
    const double K = ktab(P, tab, 1, c).x;
    const double* cf = P.coef + ((size_t)s * Nn + n) * COEF_1V;   // coef_1v of plane (s, n)
    // nu: -col(n) C
    const double col = cf[4];
    loc[0] += -col * (ge.x * C0.x - ge.y * C0.y);
    // streaming -i K a0 t  with t = sqrt((n+1)/2) C+ + sqrt(n/2) C- + (u0/a0) C
    double2 t = cscale(P.ua[s], C0);
    t = crfma(cf[0], Cp, t);
    t = crfma(cf[1], Cm, t);
    const double w = K * a0;
    const double2 fk = make_double2(w * t.y, -w * t.x);
    loc[1] += ge.x * fk.x - ge.y * fk.y;
    // u_x,s: -i K C
    const double2 fu = make_double2(K * C0.y, -K * C0.x);
    loc[2 + s] += ge.x * fu.x - ge.y * fu.y;
  } else {
    const int f = (int)((e - nC) / N), c = (int)((e - nC) % N);
    const double K = ktab(P, tab, 1, c).x;
    const double2* F = y + nC;
    const double iO = P.iO0;
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

// Block sums of loc[0 .. nk) (every thread's values); valid in threads 0 .. nk-1.
__device__ __forceinline__ double block_sums(const double* loc, int nk, double (*red)[2 + SPX_MAX_SPECIES]) {
  for (int k = 0; k < nk; ++k) {
    double v = loc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  double v = 0.0;
  if ((int)threadIdx.x < nk)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
  return v;
}

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
  const int nk = 2 + P.pb.Ns;
  double loc[2 + SPX_MAX_SPECIES];
  for (int k = 0; k < 2 + SPX_MAX_SPECIES; ++k) loc[k] = 0.0;
  const long long len = P.nc + 6LL * P.ax[1].n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len;
       e += (long long)gridDim.x * blockDim.x)
    param_terms(P, stab, y, g[e], e, loc);
  const double v = block_sums(loc, nk, red);
  if ((int)threadIdx.x < nk) atomicAdd(acc + threadIdx.x, v);
}

// VJP of one stage plus the parameter dot products, in one launch (1D1V):
// g = J(y)^T w and acc[k] += Re sum_e w_e (df/dtheta_k)_e.  Tile CTAs run the
// VJP tile and the parameter terms of their own planes, the extra CTA those of
// the field entries; every CTA writes its partial sums, and the last to arrive
// (atomic ticket) sums the tiles' transformed field partials into the field
// gradient and adds the parameter partials to acc in a fixed order.
// ws: part (Ns * ntiles * N double2) | pp (grid x (2 + SPX_MAX_SPECIES) doubles) |
// gpart (Ns * groups * N double2); the tickets live in the plan (calls on one
// plan are serialised, as its workspace is).
template <bool HERM, bool MG>
__global__ void __launch_bounds__(NTHREADS, 2) k_vjp_param_1v(const DevPlan* __restrict__ gP,
                                                              const double2* __restrict__ gtab,
                                                              const double2* __restrict__ y,
                                                              const double2* __restrict__ w,
                                                              double2* __restrict__ g, double2* part, double* pp,
                                                              double2* gpart, unsigned int* ticket, double* acc) {
  __shared__ DevPlan P;
  __shared__ double red[NTHREADS / 32][2 + SPX_MAX_SPECIES];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int last;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const int nblk = P.pb.Ns * P.ntiles;
  const int N = P.ax[1].n, Nn = P.pb.Nn, T = P.tile;
  const int nk = 2 + P.pb.Ns;
  // work area: sA, sB (2T+2 lines of Lw = max(Nx, product grid) each) | Uy, Uw (T+2
  // lines of Nx each) | yF3, wE (3 lines each) | coefficients
  const int Lw = MG ? max(N, P.axm.n) : N;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)(2 * T + 2) * Lw;
  double2* Uy = sB + (size_t)(2 * T + 2) * Lw;
  double2* Uw = Uy + (size_t)(T + 2) * N;
  double2* yF3 = Uw + (size_t)(T + 2) * N;
  double2* wE = yF3 + 3 * (size_t)N;
  double* scoef = reinterpret_cast<double*>(wE + 3 * (size_t)N);
  double loc[2 + SPX_MAX_SPECIES];
#pragma unroll
  for (int k = 0; k < 2 + SPX_MAX_SPECIES; ++k) loc[k] = 0.0;
  const int b = blockIdx.x;
  bool timed_out = false;
  // y (the stage input) does not depend on the previous launch (the combination
  // that forms w): its planes are requested first
  const bool tile_cta = b < nblk;
  const int s = tile_cta ? b / P.ntiles : 0, tile = tile_cta ? b % P.ntiles : 0;
  const int m0 = tile * T, nt = tile_cta ? min(T, Nn - m0) : 0;
  const size_t sbase = (size_t)s * Nn * N;
  const int lo = max(m0 - 1, 0), hi = min(m0 + nt, Nn - 1);
  const uint32_t bu = (uint32_t)((hi - lo + 1) * N * sizeof(double2));
  const uint32_t bf = (uint32_t)(N * sizeof(double2));
  const size_t d0 = (size_t)(lo - (m0 - 1)) * N;
  if (nt > 0) {
    if (threadIdx.x == 0) {
      mbar_init(&bars[0], 1);
      mbar_init(&bars[1], 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_arm(&bars[0], bu + 3 * bf);
      bulk_g2s(Uy + d0, y + sbase + (size_t)lo * N, bu, &bars[0]);
      const double2* F = y + P.nc;
      bulk_g2s(yF3, F, bf, &bars[0]);                          // E_x
      bulk_g2s(yF3 + N, F + 5 * (size_t)N, bf, &bars[0]);      // B_z
      bulk_g2s(yF3 + 2 * N, F + 4 * (size_t)N, bf, &bars[0]);  // B_y
    }
  }
  pdl_wait_and_release();
  if (tile_cta) {
    if (nt > 0) {
      if (threadIdx.x == 0) {
        mbar_arm(&bars[1], bu + 3 * bf);
        bulk_g2s(Uw + d0, w + sbase + (size_t)lo * N, bu, &bars[1]);
        bulk_g2s(wE, w + P.nc, 3 * bf, &bars[1]);                // w's E_x, E_y, E_z
      }
      if (m0 == 0)
        for (int i = threadIdx.x; i < N; i += blockDim.x) Uy[i] = Uw[i] = make_double2(0.0, 0.0);
      if (m0 + nt == Nn)
        for (int i = threadIdx.x; i < N; i += blockDim.x)
          Uy[(size_t)(nt + 1) * N + i] = Uw[(size_t)(nt + 1) * N + i] = make_double2(0.0, 0.0);
      const bool ok = mbar_wait_bounded(&bars[0], 0) && mbar_wait_bounded(&bars[1], 0);
      if (__syncthreads_or(!ok)) {
        timed_out = true;
      } else {
        double pacc[3] = {0.0, 0.0, 0.0};
        vjp1v_tile_u<HERM, MG>(P, stab, Uy, Uw, yF3, wE, g, part, s, tile, m0, nt, sA, sB, scoef, pacc);
#pragma unroll
        for (int k = 0; k < 2 + SPX_MAX_SPECIES; ++k)
          loc[k] = (k == 0) ? pacc[0] : (k == 1) ? pacc[1] : (k == 2 + s) ? pacc[2] : 0.0;
      }
    } else {
      for (int x = threadIdx.x; x < N; x += blockDim.x)
        part[((size_t)s * P.ntiles + tile) * N + x] = make_double2(0.0, 0.0);
    }
  } else {
    for (long long e = P.nc + threadIdx.x; e < P.nc + 6LL * N; e += blockDim.x) param_terms(P, stab, y, w[e], e, loc);
  }
  if (timed_out && threadIdx.x == 0) atomicExch(&g_rk_status, SPX_ST_WAIT_TIMEOUT);
  const double v = block_sums(loc, nk, red);
  if ((int)threadIdx.x < nk) pp[(size_t)b * (2 + SPX_MAX_SPECIES) + threadIdx.x] = v;
  // group of 8 tiles: the last tile of a group to finish sums the group's
  // partials (while other tiles still run); then every CTA takes the ticket
  const int ngroups = (P.ntiles + 7) / 8;
  if (tile_cta) {
    const int grp = tile >> 3, gsz = min(8, P.ntiles - grp * 8);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(ticket + 64 + s * ngroups + grp, 1u) == (unsigned)gsz - 1);
    __syncthreads();
    if (last) {
      __threadfence();
      const double2* p0 = part + ((size_t)s * P.ntiles + grp * 8) * N;
      for (int c = threadIdx.x; c < N; c += blockDim.x)
        gpart[((size_t)s * ngroups + grp) * N + c] = sum_lines8(p0 + c, gsz, N);
      if (threadIdx.x == 0) ticket[64 + s * ngroups + grp] = 0;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // field pass over the groups' transformed partials (Ns lines of scratch)
  vjp1v_fields_spectral(P, stab, w + P.nc, g + P.nc, gpart, ngroups, sA);
  // parameter partials: every thread loads its CTAs' values at once, then a
  // fixed-order block reduction per parameter
  __syncthreads();
  double part_k[2 + SPX_MAX_SPECIES];
#pragma unroll
  for (int k = 0; k < 2 + SPX_MAX_SPECIES; ++k) part_k[k] = 0.0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
#pragma unroll
    for (int k = 0; k < 2 + SPX_MAX_SPECIES; ++k)
      if (k < nk) part_k[k] += __ldcg(pp + (size_t)q * (2 + SPX_MAX_SPECIES) + k);
  }
  const double tot = block_sums(part_k, nk, red);
  if ((int)threadIdx.x < nk) acc[threadIdx.x] += tot;
  if (threadIdx.x == 0) *ticket = 0;
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
#define SPX_RK_ATTR(L, H)                                                                              \
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_rk_stage_st<L, H>));                                           \
  SPX_CUDA(cudaFuncSetAttribute(k_rk_stage_st<L, H>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                optin - (int)fa.sharedSizeBytes));
  SPX_RK_ATTR(false, false)
  SPX_RK_ATTR(true, false)
  SPX_RK_ATTR(false, true)
  SPX_RK_ATTR(true, true)
#undef SPX_RK_ATTR
#define SPX_VJP_ATTR(H, G)                                                                             \
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_vjp_param_1v<H, G>));                                          \
  SPX_CUDA(cudaFuncSetAttribute(k_vjp_param_1v<H, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                optin - (int)fa.sharedSizeBytes));
  SPX_VJP_ATTR(false, false)
  SPX_VJP_ATTR(true, false)
  SPX_VJP_ATTR(false, true)
  SPX_VJP_ATTR(true, true)
#undef SPX_VJP_ATTR
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
  return spx_rk_step_store_ex(pl, y, h, Ystages, Kstages, ynext, 0, stream);
}

int spx_rk_step_store_ex(const spx_plan* pl, const void* y, double h, void* Ystages, void* Kstages, void* ynext,
                         int32_t hermitian, void* stream) {
  if (!pl || !y || !Ystages || !Kstages || !ynext) { set_error("spx_rk_step_store: null argument"); return SPX_E_ARG; }
  if (pl->host.path != 0) {
    set_error("spx_rk_step_store: only the 1D1V layout (Ny = Nz = Nm = Np = 1) is supported");
    return SPX_E_UNSUPPORTED;
  }
  if (hermitian && !pl->herm_ok) {
    set_error("spx_rk_step_store_ex: packed transforms need an odd Nx with an antisymmetric wavenumber grid");
    return SPX_E_ARG;
  }
  if (int rd = check_plan_device(pl, "spx_rk_step_store")) return rd;
  const int herm = hermitian ? 1 : 0;
  int rc = adj_setup();
  if (rc != SPX_OK) return rc;
  const DevPlan& P = pl->host;
  const long long len = P.nc + 6LL * P.plane;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2* Yb = static_cast<double2*>(Ystages);
  if (static_cast<const void*>(Yb) != y)
    SPX_CUDA(cudaMemcpyAsync(Yb, y, sizeof(double2) * len, cudaMemcpyDeviceToDevice, st));
  cudaFuncAttributes fa;
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_rk_stage_st<true, false>));
  {
    cudaFuncAttributes fh;
    SPX_CUDA(cudaFuncGetAttributes(&fh, k_rk_stage_st<true, true>));
    if (fh.sharedSizeBytes > fa.sharedSizeBytes) fa = fh;
  }
  int npf = 0;
  const size_t smem = stage_smem_1v(pl, fa.sharedSizeBytes, &npf);
  if (npf < 1) { set_error("spx_rk_step_store: Nx / tile too large for the stage kernel"); return SPX_E_UNSUPPORTED; }
  const int grid = P.pb.Ns * P.ntiles + 1;
  for (int stage = 0; stage < rk::S; ++stage) {
    const DevPlan* dp = pl->d_plan;
    const double2* dt = pl->d_tab;
    const double2* yb = Yb;
    double2* kb = static_cast<double2*>(Kstages);
    double2* yn = static_cast<double2*>(ynext);
    const bool last = stage == rk::S - 1;
    if (herm)
      SPX_CUDA(launch_pdl(last ? k_rk_stage_st<true, true> : k_rk_stage_st<false, true>, grid, pl->threads, smem,
                          st, dp, dt, yb, Yb, kb, yn, h, stage, npf));
    else
      SPX_CUDA(launch_pdl(last ? k_rk_stage_st<true, false> : k_rk_stage_st<false, false>, grid, pl->threads, smem,
                          st, dp, dt, yb, Yb, kb, yn, h, stage, npf));
  }
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_rk_status(int32_t* status, void* stream) {
  if (!status) { set_error("spx_rk_status: null argument"); return SPX_E_ARG; }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int v = 0;
  SPX_CUDA(cudaMemcpyFromSymbolAsync(&v, g_rk_status, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  SPX_CUDA(cudaStreamSynchronize(st));
  const int zero = 0;
  SPX_CUDA(cudaMemcpyToSymbolAsync(g_rk_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st));
  SPX_CUDA(cudaStreamSynchronize(st));
  *status = v;
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
  if (int rd = check_plan_device(pl, "spx_param_dots")) return rd;
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

int spx_vjp_param(const spx_plan* pl, const void* y, const void* w, void* g, double* acc, void* ws,
                  size_t ws_bytes, void* stream) {
  return spx_vjp_param_ex(pl, y, w, g, acc, ws, ws_bytes, 0, stream);
}

int spx_vjp_param_ex(const spx_plan* pl, const void* y, const void* w, void* g, double* acc, void* ws,
                     size_t ws_bytes, int32_t hermitian, void* stream) {
  if (!pl || !y || !w || !g || !acc || !ws) { set_error("spx_vjp_param: null argument"); return SPX_E_ARG; }
  if (pl->host.path != 0) {
    set_error("spx_vjp_param: only the 1D1V layout is supported");
    return SPX_E_UNSUPPORTED;
  }
  if (int rd = check_plan_device(pl, "spx_vjp_param")) return rd;
  if (hermitian && !pl->herm_ok) {
    set_error("spx_vjp_param_ex: packed transforms need an odd Nx with an antisymmetric wavenumber grid");
    return SPX_E_ARG;
  }
  if (ws_bytes < pl->ws_bytes || (reinterpret_cast<uintptr_t>(ws) & 255)) {
    set_error("spx_vjp_param: workspace too small or not 256-byte aligned");
    return SPX_E_WORKSPACE;
  }
  int rc = adj_setup();
  if (rc != SPX_OK) return rc;
  const DevPlan& P = pl->host;
  const int grid = P.pb.Ns * P.ntiles + 1;
  char* wsb = static_cast<char*>(ws);
  const size_t part_bytes = (size_t)P.pb.Ns * P.ntiles * P.ax[1].n * sizeof(double2);
  double* pp = reinterpret_cast<double*>(wsb + part_bytes);
  double2* gpart = reinterpret_cast<double2*>(wsb + part_bytes + (size_t)grid * (2 + SPX_MAX_SPECIES) * sizeof(double));
  // the plan's ticket is zero between launches (the last CTA resets it)
  unsigned int* ticket = pl->d_ticket;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int T = P.tile, N = P.ax[1].n;
  // the transposed products on the plan's product grid where it has one without
  // the folded |k| = K term (that term's transpose is only on the Nx-point grid)
  const bool mg = P.axm.n != N && P.alias == 0;
  const int Lw = mg ? std::max(N, P.axm.n) : N;
  const size_t smem = pl->smem_tab + ((size_t)(4 * T + 4) * Lw + (size_t)(2 * T + 10) * N) * sizeof(double2) +
                      64 * sizeof(double);
  if (smem > (size_t)smem_optin()) {
    set_error("spx_vjp_param: the tile does not fit in shared memory");
    return SPX_E_UNSUPPORTED;
  }
  const DevPlan* dp = pl->d_plan;
  const double2* dt = pl->d_tab;
  // a plain launch: with a programmatic early start the CTAs of this small grid
  // (one per SM) were placed less evenly and the kernel ran longer
  auto kern = hermitian ? (mg ? k_vjp_param_1v<true, true> : k_vjp_param_1v<true, false>)
                        : (mg ? k_vjp_param_1v<false, true> : k_vjp_param_1v<false, false>);
  kern<<<grid, pl->threads, smem, st>>>(dp, dt, static_cast<const double2*>(y), static_cast<const double2*>(w),
                                        static_cast<double2*>(g), reinterpret_cast<double2*>(wsb), pp, gpart,
                                        ticket, acc);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

}  // extern "C"
