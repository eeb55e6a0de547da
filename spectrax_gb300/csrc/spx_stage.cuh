// spx_stage.cuh — one Runge-Kutta stage of the fused 1D1V path with staged
// operands, shared by the device Dopri8 solver and the adjoint's step
// recomputation.
//
// A tile CTA stages its input planes n0-1 .. n0+nt of S_i and the three field
// lines that G needs with bulk asynchronous copies (barrier 0), and the
// epilogue operands of its own planes -- y and the K_j the stage combination
// reads -- on barrier 1, so the latter arrive while the transforms run.  The
// epilogue stores K_i and S_{i+1} = y + h sum_j a(i+1, j) K_j (or y_new and the
// scaled error on the last stage).  The field CTA gathers its few lines with
// plain loads.  Every wait is bounded; a wait that gives up sets *timeout_status.
#pragma once
#include <type_traits>
#include <algorithm>

#include "spx_plan.h"
#include "spx_rhs.cuh"
#include "spx_tma.cuh"

namespace spx {

constexpr int MAX_TERMS = 10;

// Coefficients of the current launch's epilogue, in shared memory.
struct EpiTerms {
  int n;                       // number of K_j terms (j < stage)
  int j[MAX_TERMS];
  double c[MAX_TERMS];         // h a(stage+1, j)  or  h b_j
  double e[MAX_TERMS];         // last stage: h e_j
  double cself, eself;         // the current stage's own weights
};

// Epilogue of stages 0..11: store K_i and the next stage input.  The first
// `npf` operands (y, then K_j in list order) of the CTA's own entries are
// staged in shared memory `pf` (own entries each, local index il); the rest
// are read from global memory, up to five loads in flight.
struct EpiNext {
  double2* __restrict__ Ki;
  double2* __restrict__ Snext;
  const double2* __restrict__ Y;
  const double2* __restrict__ K;
  long long len;
  const EpiTerms* T;
  const double2* pf;
  int own, npf;
  uint64_t* bar;               // completes when pf is filled (nullptr: nothing staged)
  __device__ bool prepare() const {
    if (!bar) return true;
    const bool ok = mbar_wait_bounded(bar, 0);
    return !__syncthreads_or(!ok);
  }
  __device__ __forceinline__ double2 operand(int q, size_t e, int il) const {
    // q = 0: y, q >= 1: K_{j[q-1]}
    if (q < npf) return pf[(size_t)q * own + il];
    return q == 0 ? Y[e] : K[(size_t)T->j[q - 1] * len + e];
  }
  __device__ __forceinline__ void operator()(size_t e, int il, double2 v) const {
    Ki[e] = v;
    Snext[e] = next(e, il, v);
  }
  // exactly Hermitian operands: the mirrored entry e2 gets the conjugates
  __device__ __forceinline__ void pair(size_t e, int il, size_t e2, int il2, double2 v, bool two) const {
    const double2 sn = next(e, il, v);
    Ki[e] = v;
    Snext[e] = sn;
    if (two) {
      Ki[e2] = conj_bits(v);
      Snext[e2] = conj_bits(sn);
    }
  }
  __device__ __forceinline__ double2 next(size_t e, int il, double2 v) const {
    const int n = T->n;
    double2 acc;
    if (npf > n) {                       // every operand staged
      acc = pf[il];
#pragma unroll 1
      for (int t = 0; t < n; ++t) acc = crfma(T->c[t], pf[(size_t)(1 + t) * own + il], acc);
    } else {
      acc = operand(0, e, il);
#pragma unroll 1
      for (int r = 0; r < n; r += 5) {
        double2 k[5];
#pragma unroll
        for (int u = 0; u < 5; ++u)
          if (r + u < n) k[u] = operand(1 + r + u, e, il);
#pragma unroll
        for (int u = 0; u < 5; ++u)
          if (r + u < n) acc = crfma(T->c[r + u], k[u], acc);
      }
    }
    return crfma(T->cself, v, acc);
  }
};

// Epilogue of the last stage: y_new, scaled error, non-finite flag; operands
// staged as in EpiNext.
struct EpiFinal {
  double2* __restrict__ Ki;
  double2* __restrict__ Ynew;
  const double2* __restrict__ Y;
  const double2* __restrict__ K;
  long long len;
  const EpiTerms* T;
  const double2* pf;
  int own, npf;
  uint64_t* bar;
  double rtol, atol;
  int adaptive;
  double sq;
  int nonfinite;
  double2 last_yn;
  double last_sq;
  __device__ bool prepare() const {
    if (!bar) return true;
    const bool ok = mbar_wait_bounded(bar, 0);
    return !__syncthreads_or(!ok);
  }
  __device__ __forceinline__ double2 operand(int q, size_t e, int il) const {
    if (q < npf) return pf[(size_t)q * own + il];
    return q == 0 ? Y[e] : K[(size_t)T->j[q - 1] * len + e];
  }
  __device__ __forceinline__ void operator()(size_t e, int il, double2 v) {
    Ki[e] = v;
    const double2 y0 = operand(0, e, il);
    double2 yn = y0;
    double2 er = make_double2(0.0, 0.0);
    const int n = T->n;
    if (npf > n) {                       // every operand staged
#pragma unroll 1
      for (int t = 0; t < n; ++t) {
        const double2 k = pf[(size_t)(1 + t) * own + il];
        yn = crfma(T->c[t], k, yn);
        er = crfma(T->e[t], k, er);
      }
    } else {
#pragma unroll 1
      for (int r = 0; r < n; r += 5) {
        double2 k[5];
#pragma unroll
        for (int u = 0; u < 5; ++u)
          if (r + u < n) k[u] = operand(1 + r + u, e, il);
#pragma unroll
        for (int u = 0; u < 5; ++u)
          if (r + u < n) {
            yn = crfma(T->c[r + u], k[u], yn);
            er = crfma(T->e[r + u], k[u], er);
          }
      }
    }
    yn = crfma(T->cself, v, yn);
    er = crfma(T->eself, v, er);
    Ynew[e] = yn;
    last_yn = yn;
    if (!(isfinite(yn.x) && isfinite(yn.y))) nonfinite = 1;
    if (adaptive) {
      // |err / (atol + rtol max(|y0|, |y1|))|^2 with one division per entry
      const double m0 = fma(y0.x, y0.x, y0.y * y0.y), m1 = fma(yn.x, yn.x, yn.y * yn.y);
      const double inv = 1.0 / fma(rtol, sqrt(fmax(m0, m1)), atol);
      const double rx = er.x * inv, ry = er.y * inv;
      last_sq = fma(rx, rx, ry * ry);
      sq += last_sq;
    }
  }
  // exactly Hermitian operands: the mirrored entry has the conjugate y_new and
  // the same error contribution
  __device__ __forceinline__ void pair(size_t e, int il, size_t e2, int il2, double2 v, bool two) {
    (*this)(e, il, v);
    if (two) {
      Ki[e2] = conj_bits(v);
      Ynew[e2] = conj_bits(last_yn);
      if (adaptive) sq += last_sq;
    }
  }
};

// Shared-memory layout of the fused 1D1V stage kernel after the table (double2
// units, all 16-byte aligned): stage_area_1v(T, Ns, N, M) entries, i.e.
//   sA, sB : (T+1)*M each (M = the product grid axm.n)   U : (T+2)*N   F3 : 3*N
//   (the field CTA reuses the area as its (2*Ns+12)*N gather + output lines),
// then scoef : 64 doubles, then pf : npf * T * N (y and K_j of the CTA's own planes).

// Dynamic shared memory of a staged stage kernel for `plan` and the number of
// epilogue operands (y first, then K_j) staged: as many as keep two CTAs per SM
// resident, at least y; 0 if even that does not fit.  When the launch has no more
// CTAs than the GPU has SMs (one CTA per SM), every operand is staged instead:
// measured 2 % faster per attempt on the two-stream workload (130 CTAs) than
// keeping room for a second, programmatically launched CTA per SM.
inline size_t stage_smem_1v(const spx_plan* plan, size_t static_smem, int* npf_out) {
  const DevPlan& P = plan->host;
  const int T = P.tile, N = P.ax[1].n;
  const size_t base = plan->smem_tab + (size_t)stage_area_1v(T, P.pb.Ns, N, P.axm.n) * sizeof(double2) +
                      64 * sizeof(double);
  const size_t per = (size_t)T * N * sizeof(double2);
  const size_t two_per_sm = 228 * 1024 / 2 - 1024 - static_smem;
  const size_t optin = (size_t)smem_optin() - static_smem;
  const bool one_per_sm = P.pb.Ns * P.ntiles + 1 <= plan->nsm;
  const size_t budget = (!one_per_sm && base + per <= two_per_sm) ? two_per_sm : optin;
  const int npf = (int)std::min<size_t>(1 + MAX_TERMS, budget > base ? (budget - base) / per : 0);
  *npf_out = npf;
  return npf >= 1 ? base + (size_t)npf * per : 0;
}

// Inputs and outputs of one staged stage.
struct StageIO {
  const double2* in;          // stage input S_i (S_0 = y)
  const double2* Y;           // y of the step
  const double2* K;           // stage vectors, K_j at K + j * len
  long long len;
  double2* Ki;                // K_i output
  double2* out;               // S_{i+1} (stages 0..11) or y_new (last stage)
  int npf;                    // staged epilogue operands available in shared memory (y first)
  bool herm;                  // exactly Hermitian state: packed real transforms
  double rtol, atol;          // last stage: error scaling
  int adaptive;
  int* timeout_status;        // gets SPX_ST_WAIT_TIMEOUT if a staged copy never lands
  bool persistent;            // called again in the same launch: fence the async proxy before
                              // the copies, invalidate the barriers afterwards
};

// Field-CTA source reading through L2 (data other CTAs wrote in the same launch).
struct SrcL2 {
  const double2* y;
  __device__ __forceinline__ double2 operator()(size_t e) const { return __ldcg(y + e); }
};

// Runs the CTA's share of one stage (block b of Ns * ntiles tile CTAs + the
// field CTA).  `terms` must be visible to every thread; bars / red are the
// caller's shared scratch.  LAST: `tail(el)` is called by every thread of every
// CTA with the stage's EpiFinal (or an empty accumulator) for the error reduction.
// HM: 0 general transforms only, 1 packed transforms only, 2 chosen by io.herm
// at run time (both variants compiled into the caller).  MGS: 0 products on the
// Nx-point grid only, 1 on the plan's product grid only, 2 chosen at run time
// (a kernel holding both variants takes the larger register allocation).
template <bool LAST, int HM = 2, int MGS = 2, class Tail>
__device__ bool staged_stage_1v(const DevPlan& P, const double2* __restrict__ stab, const StageIO& io,
                                const EpiTerms& terms, uint64_t* bars, Tail&& tail) {
  const long long len = io.len;
  const int nblk = P.pb.Ns * P.ntiles;
  const int N = P.ax[1].n, T = P.tile, Nn = P.pb.Nn;
  const int b = blockIdx.x;
  double2* sA = const_cast<double2*>(stab) + (P.tab_len + 15) / 16 * 16;
  const int Lm = P.axm.n;
  double* scoef = reinterpret_cast<double*>(sA + (size_t)stage_area_1v(T, P.pb.Ns, N, Lm));
  double2* pf = reinterpret_cast<double2*>(scoef + 64);
  if (b == nblk) {
    // field CTA: plain gather (one CTA, small) and global epilogue operands
    __syncthreads();
    if constexpr (!LAST) {
      EpiNext epi{io.Ki, io.out, io.Y, io.K, len, &terms, nullptr, 0, 0, nullptr};
      maxwell1v_g(P, stab, SrcL2{io.in}, sA, epi);
    } else {
      EpiFinal el{io.Ki, io.out, io.Y, io.K, len, &terms, nullptr, 0, 0, nullptr,
                  io.rtol, io.atol, io.adaptive, 0.0, 0, make_double2(0.0, 0.0), 0.0};
      maxwell1v_g(P, stab, SrcL2{io.in}, sA, el);
      tail(el);
    }
    return true;
  }
  const int sp = b / P.ntiles, n0 = (b % P.ntiles) * T, nt = min(T, Nn - n0);
  if (nt <= 0) {
    if constexpr (LAST) {
      EpiFinal none{io.Ki, io.out, io.Y, io.K, len, &terms, nullptr, 0, 0, nullptr,
                    io.rtol, io.atol, io.adaptive, 0.0, 0, make_double2(0.0, 0.0), 0.0};
      __syncthreads();
      tail(none);
    }
    return true;
  }
  double2* sB = sA + (size_t)(T + 1) * Lm;
  double2* U = sB + (size_t)(T + 1) * Lm;
  double2* F3 = U + (size_t)(T + 2) * N;
  const size_t sbase = (size_t)sp * Nn * N;
  const int own = nt * N;
  const int npf = min(io.npf, 1 + terms.n);
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (io.persistent) fence_proxy_async();
    const int lo = max(n0 - 1, 0), hi = min(n0 + nt, Nn - 1);     // staged planes, inclusive
    const uint32_t bu = (uint32_t)((hi - lo + 1) * N * sizeof(double2));
    const uint32_t bf = (uint32_t)(N * sizeof(double2));
    mbar_arm(&bars[0], bu + 3 * bf);
    bulk_g2s(U + (size_t)(lo - (n0 - 1)) * N, io.in + sbase + (size_t)lo * N, bu, &bars[0]);
    const double2* F = io.in + P.nc;
    bulk_g2s(F3, F, bf, &bars[0]);                         // E_x
    bulk_g2s(F3 + N, F + 5 * (size_t)N, bf, &bars[0]);     // B_z
    bulk_g2s(F3 + 2 * N, F + 4 * (size_t)N, bf, &bars[0]); // B_y
    const uint32_t bo = (uint32_t)(own * sizeof(double2));
    mbar_arm(&bars[1], (uint32_t)npf * bo);
    const size_t o0 = sbase + (size_t)n0 * N;
    bulk_g2s(pf, io.Y + o0, bo, &bars[1]);
    for (int q = 1; q < npf; ++q)
      bulk_g2s(pf + (size_t)q * own, io.K + (size_t)terms.j[q - 1] * len + o0, bo, &bars[1]);
  }
  // planes outside [0, Nn) read as zero (disjoint from the staged ones)
  if (n0 == 0)
    for (int i = threadIdx.x; i < N; i += blockDim.x) U[i] = make_double2(0.0, 0.0);
  if (n0 + nt == Nn)
    for (int i = threadIdx.x; i < N; i += blockDim.x) U[(size_t)(nt + 1) * N + i] = make_double2(0.0, 0.0);
  const bool ok = mbar_wait_bounded(&bars[0], 0);
  if (__syncthreads_or(!ok)) {
    // the staged input never arrived: stop, give the copies a last chance
    if (threadIdx.x == 0) {
      atomicExch(io.timeout_status, SPX_ST_WAIT_TIMEOUT);
      mbar_wait_bounded(&bars[1], 0);
    }
    return false;
  }
  // the product-grid variant only where the plan has one (a uniform branch)
  const bool mg = Lm != N;
  auto tile_g = [&](auto mgc, auto& epi) {
    constexpr bool G = decltype(mgc)::value;
    if (HM == 1 || (HM == 2 && io.herm)) rhs1v_tile_u<HM != 0, G>(P, stab, sp, n0, nt, U, F3, sA, sB, scoef, epi);
    else rhs1v_tile_u<false, G>(P, stab, sp, n0, nt, U, F3, sA, sB, scoef, epi);
  };
  auto tile = [&](auto& epi) {
    if constexpr (MGS == 0) tile_g(std::false_type{}, epi);
    else if constexpr (MGS == 1) tile_g(std::true_type{}, epi);
    else if (mg) tile_g(std::true_type{}, epi);
    else tile_g(std::false_type{}, epi);
  };
  if constexpr (!LAST) {
    EpiNext epi{io.Ki, io.out, io.Y, io.K, len, &terms, pf, own, npf, &bars[1]};
    tile(epi);
  } else {
    EpiFinal el{io.Ki, io.out, io.Y, io.K, len, &terms, pf, own, npf, &bars[1],
                io.rtol, io.atol, io.adaptive, 0.0, 0, make_double2(0.0, 0.0), 0.0};
    tile(el);
    tail(el);
  }
  // a failed prepare() returns from the tile early: record it once
  bool bad = false;
  if (threadIdx.x == 0 && !mbar_try_wait(&bars[1], 0)) {
    atomicExch(io.timeout_status, SPX_ST_WAIT_TIMEOUT);
    bad = true;
  }
  if (io.persistent) {
    // the barriers are initialised again by the next stage: only complete ones are invalidated
    if (__syncthreads_or(bad)) return false;
    if (threadIdx.x == 0) {
      mbar_inval(&bars[0]);
      mbar_inval(&bars[1]);
    }
  }
  return !bad;
}

}  // namespace spx
