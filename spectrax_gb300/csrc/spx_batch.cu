// spx_batch.cu — many independent 1D1V instances in one persistent launch.
//
// Each thread-block cluster (C CTAs, C = 1..8) takes the next instance from a
// global work queue ordered by decreasing estimated cost (largest first), runs
// that instance's whole adaptive Dopri8 integration, then takes the next one.
// The C CTAs of a cluster split the instance's Hermite tiles; stages are
// separated by hardware cluster barriers (barrier.cluster, no spin loops);
// the scaled error of a step is reduced through distributed shared memory and
// every CTA runs the same controller on the same numbers, so no extra
// broadcast is needed.  Stage data written by one CTA and read by another in
// the same launch is loaded with ld.global.cg (L2-coherent).  A tile's input
// planes are staged in shared memory before its transforms; an instance whose
// initial state is exactly Hermitian (odd Nx) runs the packed real-transform
// tiles, which keep that symmetry exactly.
//
// Instances may differ in Nx, Nn, Ns, L, nu, alpha, u (spectrax's Landau scan:
// Examples/1D_Landau_damping_dr_curve.py:88-110 loops over k serially).
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "spx_plan.h"
#include "spx_rhs.cuh"
#include "spx_tableau.cuh"

namespace cg = cooperative_groups;

namespace spx {

constexpr int BATCH_MAX_TILE = 32;   // Hermite planes per tile at most

__constant__ double bCoef[14][13];
__constant__ int bMask[14];

struct BInst {
  DevPlan P;             // instance plan (tile / ntiles chosen for the batch)
  int tab_off;           // offset of the instance table in the table pool
  int en_off;            // offset of the instance energies (nsave x (2 + Ns) doubles)
  long long pool_off;    // offset (double2) of Y0 | Y1 | S0 | S1 | K0 .. K12
  long long y_off;       // offset (double2) of the instance in the packed in/out states
  long long len;
  double masses[SPX_MAX_SPECIES];
  double t, dt;          // results
  long long accepted, rejected, evals;
  int status, saved;
  int herm_ok;           // odd Nx with an antisymmetric wavenumber table, and requested
  int herm;              // result: y0 was exactly Hermitian, packed real transforms used
  unsigned long long t_begin, t_end;   // %globaltimer (ns) when the instance's cluster took / finished it
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

struct BArgs {
  BInst* inst;
  int n;
  const double2* tab;
  double2* pool;
  const double2* y_in;
  double2* y_out;
  double* energies;
  const double* save_ts;
  int nsave;
  double t1, dt0, rtol, atol;
  long long max_steps;
  int adaptive;
  int interp;             // 1: save times inside a step get the dense output (steps end only on t1)
  const int* order;
  unsigned int* next;
  int tab_max;
  int work_max;           // double2 entries of the per-tile work area (line buffers, staged planes)
};

struct Ctl {
  double t, dt;
  long long acc, rej, evals;
  int cur, k1_valid, isave, status, saved, herm;
};

// Epilogue term list of one stage (see the single-instance solver): stage i < 12
// forms y + h sum_j a(i+1, j) K_j over j < i with a(i+1, j) != 0, then
// + h a(i+1, i) K_i; the last stage forms y_new and the error over j < 12 with
// b_j != 0 or e_j != 0.  Ascending j.
struct BTerms {
  int n;
  int j[12];
  double c[12], e[12];
  double cself, eself;
};

// Called by the 32 lanes of warp 0: lane j < stage fills the term of K_j (terms
// in ascending j), so the products cost one warp-level multiply each.
__device__ void fill_bterms(BTerms& T, int stage, double h) {
  const bool last = stage == rk::S - 1;
  const int row = last ? 12 : stage;
  const unsigned mask = (unsigned)(last ? (bMask[12] | bMask[13]) : bMask[row]) & ((1u << stage) - 1u);
  const int l = threadIdx.x & 31;
  if (l < stage && (mask & (1u << l))) {
    const int t = __popc(mask & ((1u << l) - 1u));
    T.j[t] = l;
    T.c[t] = h * bCoef[row][l];
    T.e[t] = last ? h * bCoef[13][l] : 0.0;
  }
  if (l == 0) {
    T.n = __popc(mask);
    T.cself = h * bCoef[row][stage];
    T.eself = last ? h * bCoef[13][stage] : 0.0;
  }
}

// Source of a tile's stage input written earlier in this launch (L2-coherent loads).
struct SrcCG {
  const double2* y;
  __device__ __forceinline__ double2 operator()(size_t e) const { return __ldcg(y + e); }
};

// Stages 0..11: store K_i and the next stage input; operands from global memory
// (written earlier in this launch: ld.global.cg), up to five loads in flight.
struct EpiNextB {
  double2* __restrict__ Ki;
  double2* __restrict__ Snext;
  const double2* Y;
  const double2* K;
  long long len;
  const BTerms* T;
  __device__ bool prepare() const { return true; }
  __device__ __forceinline__ double2 next(size_t e, double2 v) const {
    double2 acc = __ldcg(Y + e);
    const int n = T->n;
#pragma unroll 1
    for (int r = 0; r < n; r += 5) {
      double2 k[5];
#pragma unroll
      for (int u = 0; u < 5; ++u)
        if (r + u < n) k[u] = __ldcg(K + (size_t)T->j[r + u] * len + e);
#pragma unroll
      for (int u = 0; u < 5; ++u)
        if (r + u < n) acc = crfma(T->c[r + u], k[u], acc);
    }
    return crfma(T->cself, v, acc);
  }
  __device__ __forceinline__ void operator()(size_t e, int, double2 v) const {
    Ki[e] = v;
    Snext[e] = next(e, v);
  }
  __device__ __forceinline__ void pair(size_t e, int, size_t e2, int, double2 v, bool two) const {
    const double2 sn = next(e, v);
    Ki[e] = v;
    Snext[e] = sn;
    if (two) {
      Ki[e2] = conj_bits(v);
      Snext[e2] = conj_bits(sn);
    }
  }
};

// Last stage: y_new, scaled error, non-finite flag.
struct EpiFinalB {
  double2* __restrict__ Ki;
  double2* __restrict__ Ynew;
  const double2* Y;
  const double2* K;
  long long len;
  const BTerms* T;
  double rtol, atol;
  int adaptive;
  double sq;
  int nonfinite;
  __device__ bool prepare() const { return true; }
  __device__ __forceinline__ double finish(size_t e, double2 v, double2& yn) {
    const double2 y0 = __ldcg(Y + e);
    yn = y0;
    double2 er = make_double2(0.0, 0.0);
    const int n = T->n;
#pragma unroll 1
    for (int r = 0; r < n; r += 5) {
      double2 k[5];
#pragma unroll
      for (int u = 0; u < 5; ++u)
        if (r + u < n) k[u] = __ldcg(K + (size_t)T->j[r + u] * len + e);
#pragma unroll
      for (int u = 0; u < 5; ++u)
        if (r + u < n) {
          yn = crfma(T->c[r + u], k[u], yn);
          er = crfma(T->e[r + u], k[u], er);
        }
    }
    yn = crfma(T->cself, v, yn);
    er = crfma(T->eself, v, er);
    if (!(isfinite(yn.x) && isfinite(yn.y))) nonfinite = 1;
    if (!adaptive) return 0.0;
    const double m0 = fma(y0.x, y0.x, y0.y * y0.y), m1 = fma(yn.x, yn.x, yn.y * yn.y);
    const double inv = 1.0 / fma(rtol, sqrt(fmax(m0, m1)), atol);
    const double rx = er.x * inv, ry = er.y * inv;
    return fma(rx, rx, ry * ry);
  }
  __device__ __forceinline__ void operator()(size_t e, int, double2 v) {
    double2 yn;
    sq += finish(e, v, yn);
    Ki[e] = v;
    Ynew[e] = yn;
  }
  __device__ __forceinline__ void pair(size_t e, int, size_t e2, int, double2 v, bool two) {
    double2 yn;
    const double c = finish(e, v, yn);
    sq += two ? c + c : c;
    Ki[e] = v;
    Ynew[e] = yn;
    if (two) {
      Ki[e2] = conj_bits(v);
      Ynew[e2] = conj_bits(yn);
    }
  }
};

__device__ __forceinline__ double bsum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += red[i];
  return r;
}

// Energies of spectrax/_diagnostics.py:191-219 for state Y (whole CTA; thread 0 writes).
// Energies of the state whose entries val(e) returns (valid in thread 0, which writes them).
template <class V>
__device__ void batch_energies(const DevPlan& P, V&& val, const double* masses, double* out, double* red) {
  const int N = P.ax[1].n;
  double em = 0.0;
  for (int i = threadIdx.x; i < 6 * N; i += blockDim.x) {
    const double2 f = val((size_t)P.nc + i);
    em = fma(f.x, f.x, fma(f.y, f.y, em));
  }
  em = bsum(em, red);
  if (threadIdx.x == 0) {
    const spx_problem& pb = P.pb;
    const int Hs = P.nh, kc = N / 2;
    const int offs[7] = {0, 1, pb.Nn, pb.Nn * pb.Nm, 2, 2 * pb.Nn, 2 * pb.Nn * pb.Nm};
    const double O0 = pb.Omega_cs[0];
    double ke = 0.0;
    for (int s = 0; s < pb.Ns; ++s) {
      double c[7];
      for (int k = 0; k < 7; ++k)
        c[k] = (offs[k] < Hs) ? val(((size_t)s * Hs + offs[k]) * N + kc).x : 0.0;
      const double a0 = pb.alpha_s[3 * s], a1 = pb.alpha_s[3 * s + 1], a2 = pb.alpha_s[3 * s + 2];
      const double u0 = pb.u_s[3 * s], u1 = pb.u_s[3 * s + 1], u2 = pb.u_s[3 * s + 2];
      const double pref = 0.5 * masses[s] * a0 * a1 * a2;
      const double t0 = 0.5 * (a0 * a0 + a1 * a1 + a2 * a2) + (u0 * u0 + u1 * u1 + u2 * u2);
      const double t1 = 1.41421356237309504880 * (a0 * u0 * c[1] + a1 * u1 * c[2] + a2 * u2 * c[3]);
      const double t2 = 0.70710678118654752440 * (a0 * a0 * c[4] + a1 * a1 * c[5] + a2 * a2 * c[6]);
      const double kes = pref * (t0 * c[0] + t1 + t2);
      out[2 + s] = kes;
      ke += kes;
    }
    out[0] = 0.5 * em * O0 * O0;
    out[1] = ke;
  }
}

// CTAs per SM the register allocation aims at
// (2: two CTAs per SM at up to 128 registers; measured faster on the Landau scan
// than one CTA per SM at 255 registers, despite a few hundred bytes of spills)
#ifndef SPX_BATCH_MIN_BLOCKS
#define SPX_BATCH_MIN_BLOCKS 2
#endif

__global__ void __launch_bounds__(NTHREADS, SPX_BATCH_MIN_BLOCKS) k_batch(BArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int crank = (int)cl.block_rank();
  const int C = (int)cl.num_blocks();
  __shared__ DevPlan P;
  __shared__ Ctl ctl;
  __shared__ int s_inst;
  __shared__ double s_part[2];
  __shared__ double red[NTHREADS / 32];
  __shared__ BTerms terms;
  __shared__ int s_bad;
  __shared__ double s_w[rk::S];   // dense-output weights h b_j(theta) of one save time
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  double2* sA = stab + (a.tab_max + 15) / 16 * 16;        // per-tile work area (work_max entries)
  double* scoef = reinterpret_cast<double*>(sA + a.work_max);

  for (;;) {
    if (crank == 0 && threadIdx.x == 0) {
      const unsigned int k = atomicAdd(a.next, 1u);
      s_inst = (k < (unsigned)a.n) ? a.order[k] : -1;
    }
    cl.sync();
    const int id = *cl.map_shared_rank(&s_inst, 0);
    cl.sync();                      // rank 0 keeps s_inst until every rank has read it
    if (id < 0) break;
    BInst* I = a.inst + id;
    if (crank == 0 && threadIdx.x == 0) I->t_begin = globaltimer_ns();
    load_plan(P, stab, &I->P, a.tab + I->tab_off);
    const long long len = I->len;
    double2* base = a.pool + I->pool_off;
    double2* Yb[2] = {base, base + len};
    double2* Sb[2] = {base + 2 * len, base + 3 * len};
    double2* K = base + 4 * len;
    double* en = a.energies + I->en_off;
    const int Ns = P.pb.Ns, N = P.ax[1].n;
    const int ntiles_all = Ns * P.ntiles + 1;        // + the field tile
    // copy y0 in (each rank a slice)
    for (long long i = (long long)crank * blockDim.x + threadIdx.x; i < len; i += (long long)C * blockDim.x)
      Yb[0][i] = __ldcg(a.y_in + I->y_off + i);
    if (threadIdx.x == 0) {
      ctl.t = 0.0; ctl.dt = a.dt0; ctl.acc = ctl.rej = ctl.evals = 0;
      ctl.cur = 0; ctl.k1_valid = 0; ctl.isave = 0; ctl.status = SPX_ST_RUNNING; ctl.saved = 0;
      if (0.0 >= a.t1) ctl.status = SPX_ST_DONE;
      s_bad = 0;
    }
    __syncthreads();
    // exact Hermitian test of y0 (every line of N entries: y(N-1-c) == conj y(c)),
    // each rank a slice, combined over the cluster through distributed shared memory
    if (I->herm_ok) {
      int bad = 0;
      for (long long i = (long long)crank * blockDim.x + threadIdx.x; i < len; i += (long long)C * blockDim.x) {
        const long long l = i / N;
        const int c = (int)(i - l * N);
        const double2 u = __ldcg(a.y_in + I->y_off + i), v = __ldcg(a.y_in + I->y_off + l * N + (N - 1 - c));
        if (!(u.x == v.x && u.y == -v.y)) bad = 1;
      }
      if (__syncthreads_or(bad) && threadIdx.x == 0) s_bad = 1;
    }
    __threadfence();
    cl.sync();
    if (threadIdx.x == 0) {
      int any = I->herm_ok ? 0 : 1;
      for (int r = 0; r < C; ++r) any |= *cl.map_shared_rank(&s_bad, r);
      ctl.herm = any ? 0 : 1;
    }
    cl.sync();
    // a save time at t0 = 0 is taken from y0
    {
      int hi = 0;
      while (hi < a.nsave && a.save_ts[hi] <= 0.0) ++hi;
      if (hi > 0) {
        if (crank == 0) {
          batch_energies(P, [&](size_t e) { return __ldcg(Yb[0] + e); }, I->masses, en, red);
          __syncthreads();
          if (threadIdx.x == 0)
            for (int k = 1; k < hi; ++k)
              for (int q = 0; q < 2 + Ns; ++q) en[k * (2 + Ns) + q] = en[q];
        }
        if (threadIdx.x == 0) { ctl.isave = hi; ctl.saved = hi; }
      }
    }
    __syncthreads();
    while (ctl.status == SPX_ST_RUNNING) {
      // attempt parameters (identical in every CTA of the cluster)
      const double t_stop = (ctl.isave < a.nsave && !a.interp) ? fmin(a.save_ts[ctl.isave], a.t1) : a.t1;
      const double t_old = ctl.t;
      double h = ctl.dt;
      bool landed = false;
      if (ctl.t + h * (1.0 + rk::SNAP) >= t_stop) { h = t_stop - ctl.t; landed = true; }
      const bool ok = !(h <= 0.0 || ctl.t + h == ctl.t);
      if (!ok || ctl.acc + ctl.rej >= a.max_steps) {
        __syncthreads();
        if (threadIdx.x == 0)
          ctl.status = (ctl.acc + ctl.rej >= a.max_steps) ? SPX_ST_MAX_STEPS : SPX_ST_DT_UNDERFLOW;
        __syncthreads();
        break;
      }
      const int cur = ctl.cur;
      const double2* Y = Yb[cur];
      const bool herm = ctl.herm != 0;
      for (int stage = 0; stage < rk::S; ++stage) {
        const double2* in = (stage == 0) ? Y : Sb[stage & 1];
        if (threadIdx.x < 32) fill_bterms(terms, stage, h);
        __syncthreads();
        double2* Ki = K + (size_t)stage * len;
        // one tile of this stage: the field tile (Maxwell + current) or Hermite
        // planes n0 .. n0+nt of species sp, staged into shared memory first
        auto run_tile = [&](int t, auto& epi) {
          if (t == ntiles_all - 1) {
            if (stage == 0 && ctl.k1_valid) {
              for (int i = threadIdx.x; i < 6 * N; i += blockDim.x) {
                const size_t e = (size_t)P.nc + i;
                epi(e, i, __ldcg(Ki + e));
              }
            } else {
              maxwell1v_g(P, stab, SrcCG{in}, sA, epi);
            }
            return;
          }
          const int sp = t / P.ntiles, n0 = (t % P.ntiles) * P.tile, nt = min(P.tile, P.pb.Nn - n0);
          if (nt <= 0) return;
          const size_t sbase = (size_t)sp * P.pb.Nn * N;
          if (stage == 0 && ctl.k1_valid) {
            const size_t b0 = sbase + (size_t)n0 * N;
            for (int i = threadIdx.x; i < nt * N; i += blockDim.x) epi(b0 + i, i, __ldcg(Ki + b0 + i));
            return;
          }
          double2* tB = sA + (size_t)(P.tile + 1) * P.axm.n;
          double2* U = tB + (size_t)(P.tile + 1) * P.axm.n;
          double2* F3 = U + (size_t)(P.tile + 2) * N;
          for (int i = threadIdx.x; i < (nt + 2) * N; i += blockDim.x) {
            const int n = n0 - 1 + i / N;
            U[i] = (n >= 0 && n < P.pb.Nn) ? __ldcg(in + sbase + (size_t)n * N + (i % N)) : make_double2(0.0, 0.0);
          }
          for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
            const int q = i / N;        // E_x, B_z, B_y
            F3[i] = __ldcg(in + P.nc + (size_t)(q == 0 ? 0 : (q == 1 ? 5 : 4)) * N + (i % N));
          }
          __syncthreads();
          if (herm) rhs1v_tile_u<true, true>(P, stab, sp, n0, nt, U, F3, sA, tB, scoef, epi);
          else rhs1v_tile_u<false, true>(P, stab, sp, n0, nt, U, F3, sA, tB, scoef, epi);
        };
        if (stage < rk::S - 1) {
          EpiNextB epi{Ki, Sb[(stage + 1) & 1], Y, K, len, &terms};
          for (int t = crank; t < ntiles_all; t += C) {
            run_tile(t, epi);
            __syncthreads();
          }
          __threadfence();
          cl.sync();
        } else {
          EpiFinalB el{Ki, Yb[cur ^ 1], Y, K, len, &terms, a.rtol, a.atol, a.adaptive, 0.0, 0};
          for (int t = crank; t < ntiles_all; t += C) {
            run_tile(t, el);
            __syncthreads();
          }
          const double q1 = bsum(el.sq, red);
          __syncthreads();
          const double q2 = bsum((double)el.nonfinite, red);
          if (threadIdx.x == 0) { s_part[0] = q1; s_part[1] = q2; }
          __threadfence();
          cl.sync();
          if (threadIdx.x == 0) {
            double sum = 0.0;
            int nonf = 0;
            for (int r = 0; r < C; ++r) {
              const double* pr = cl.map_shared_rank(s_part, r);
              sum += pr[0];
              nonf |= (pr[1] != 0.0);
            }
            const double enorm = sqrt(sum / (double)len);
            bool accept;
            double dt_next;
            if (a.adaptive) {
              accept = enorm < 1.0;
              dt_next = h * rk::controller_factor(enorm, accept);
              if (accept && landed && dt_next < ctl.dt) dt_next = ctl.dt;
            } else {
              accept = true;
              dt_next = ctl.dt;
            }
            ctl.evals += ctl.k1_valid ? rk::S - 1 : rk::S;
            if (accept) {
              ctl.t = landed ? t_stop : ctl.t + h;
              ctl.cur ^= 1;
              ctl.acc += 1;
              ctl.k1_valid = 0;
              if (nonf) ctl.status = SPX_ST_NONFINITE;
              else if (ctl.t >= a.t1) ctl.status = SPX_ST_DONE;
            } else {
              ctl.rej += 1;
              ctl.k1_valid = 1;
            }
            ctl.dt = dt_next;
            s_inst = accept ? 1 : 0;   // scratch flag for the save check below
          }
          __syncthreads();
          if (s_inst == 1) {
            int lo = ctl.isave, hi = lo;
            while (hi < a.nsave && a.save_ts[hi] <= ctl.t) ++hi;
            // every thread has its (lo, hi) before thread 0 moves ctl.isave below,
            // so the whole cluster takes the branch (and its cluster barrier) together
            __syncthreads();
            if (hi > lo) {
              if (crank == 0) {
                // each save time: the state itself at the step's end (or in land-on-save
                // mode), else the dense output y_old + sum_j h b_j(theta) K_j
                const double2* Yn = Yb[ctl.cur];
                const double2* Yo = Yb[ctl.cur ^ 1];
                for (int k = lo; k < hi; ++k) {
                  const double tsv = a.save_ts[k];
                  const bool exact = !a.interp || tsv == ctl.t;
                  if (threadIdx.x < rk::S)
                    s_w[threadIdx.x] = exact ? 0.0 : h * rk::dense_weight(threadIdx.x, (tsv - t_old) / h);
                  __syncthreads();
                  auto val = [&](size_t e) -> double2 {
                    if (exact) return __ldcg(Yn + e);
                    double2 v = __ldcg(Yo + e);
#pragma unroll 1
                    for (int j = 0; j < rk::S; ++j)
                      if (s_w[j] != 0.0) v = crfma(s_w[j], __ldcg(K + (size_t)j * len + e), v);
                    return v;
                  };
                  batch_energies(P, val, I->masses, en + (size_t)k * (2 + Ns), red);
                  __syncthreads();
                }
              }
              if (threadIdx.x == 0) { ctl.isave = hi; ctl.saved = hi; }
              // the next attempt's stage 0 (other ranks) overwrites K_0 read above
              __threadfence();
              cl.sync();
            }
          }
          __syncthreads();
        }
      }
    }
    // copy the final state out and record the instance results
    __threadfence();
    cl.sync();
    const double2* Yf = Yb[ctl.cur];
    for (long long i = (long long)crank * blockDim.x + threadIdx.x; i < len; i += (long long)C * blockDim.x)
      a.y_out[I->y_off + i] = __ldcg(Yf + i);
    if (crank == 0 && threadIdx.x == 0) {
      I->t_end = globaltimer_ns();
      I->t = ctl.t; I->dt = ctl.dt; I->accepted = ctl.acc; I->rejected = ctl.rej;
      I->evals = ctl.evals; I->status = ctl.status; I->saved = ctl.saved; I->herm = ctl.herm;
    }
    __syncthreads();
  }
}

}  // namespace spx

// ------------------------------------------------------------------ host side
using namespace spx;

struct spx_batch {
  int n = 0;
  int cluster = 1;
  int grid = 0;
  int nsave = 0;
  size_t smem = 0;
  void* block = nullptr;
  BArgs args{};
  std::vector<BInst> hinst;
  std::vector<long long> y_off;
  long long total_len = 0;
  int en_total = 0;
  double2* y_in = nullptr;
  double2* y_out = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static int batch_free(spx_batch* b) {
  if (!b) return SPX_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->block) cudaFree(b->block);
  delete b;
  return SPX_OK;
}

static int batch_consts() {
  static bool done = false;
  if (done) return SPX_OK;
  double c[14][13];
  int m[14];
  std::memset(c, 0, sizeof(c));
  for (int i = 0; i < 12; ++i) {
    m[i] = 0;
    for (int j = 0; j <= i; ++j) {
      c[i][j] = rk::A(i + 1, j);
      if (c[i][j] != 0.0) m[i] |= 1 << j;
    }
  }
  m[12] = m[13] = 0;
  for (int j = 0; j < 13; ++j) {
    c[12][j] = rk::B(j);
    c[13][j] = rk::E(j);
    if (c[12][j] != 0.0) m[12] |= 1 << j;
    if (c[13][j] != 0.0) m[13] |= 1 << j;
  }
  SPX_CUDA(cudaMemcpyToSymbol(bCoef, c, sizeof(c)));
  SPX_CUDA(cudaMemcpyToSymbol(bMask, m, sizeof(m)));
  done = true;
  return SPX_OK;
}

static void enqueue_batch(spx_batch* b, cudaStream_t st) {
  cudaMemsetAsync(b->args.next, 0, sizeof(unsigned int), st);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(b->grid, 1, 1);
  cfg.blockDim = dim3(NTHREADS, 1, 1);
  cfg.dynamicSmemBytes = b->smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = b->cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_batch, b->args);
}

extern "C" {

int spx_batch_create(int32_t n, const spx_problem* pbs, const spx_batch_opts* o, spx_batch** out) {
  if (!pbs || !o || !out || n <= 0) { set_error("spx_batch_create: bad argument"); return SPX_E_ARG; }
  *out = nullptr;
  if (o->cluster < 1 || o->cluster > 16) { set_error("spx_batch_create: cluster must be 1..16"); return SPX_E_ARG; }
  if (!(o->t1 >= 0.0) || !(o->dt0 > 0.0) || o->max_steps <= 0 || o->nsave < 0 || (o->nsave && !o->save_ts) ||
      o->saveat < 0 || o->saveat > 1) {
    set_error("spx_batch_create: bad options"); return SPX_E_ARG;
  }
  int rc;
  if ((rc = batch_consts()) != SPX_OK) return rc;
  int dev = 0, nsm = 0;
  SPX_CUDA(cudaGetDevice(&dev));
  SPX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  spx_batch* b = new spx_batch();
  b->n = n;
  b->cluster = o->cluster;
  b->nsave = o->nsave;
  std::vector<double2> tab;
  std::vector<double> coefs;          // every instance's coef_1v table, concatenated
  std::vector<size_t> coef_off(n);
  std::vector<double> cost(n);
  int tab_max = 0, work_max = 0;
  long long pool = 0, yoff = 0;
  int en_off = 0;
  b->hinst.resize(n);
  b->y_off.resize(n);
  for (int i = 0; i < n; ++i) {
    const spx_problem& p = pbs[i];
    if (!(p.Ny == 1 && p.Nz == 1 && p.Nm == 1 && p.Np == 1)) {
      set_error("spx_batch_create: instances must use the 1D1V layout (Ny = Nz = Nm = Np = 1)");
      batch_free(b);
      return SPX_E_UNSUPPORTED;
    }
    spx_plan tmp;
    // products on the plan's product grid (M points, M = Nx where Nx is already
    // 2^a 3^b): the kernel holds that one tile variant, which also runs M = Nx
    rc = build_plan_host(&p, nsm, &tmp, 0, 1);
    if (rc != SPX_OK) { batch_free(b); return rc; }
    BInst& I = b->hinst[i];
    std::memset(&I, 0, sizeof(I));
    I.P = tmp.host;
    // batch tiling: `tile` planes per tile (0: 8); tile < 0: per instance, the fewest
    // rounds r over the cluster's CTAs whose Ns * ntiles + 1 (the field tile) <= r C
    // tiles hold at most BATCH_MAX_TILE planes each, so small instances use every CTA
    int T;
    if (o->tile < 0) {
      T = BATCH_MAX_TILE;
      for (int r = 1; r <= 64; ++r) {
        const int per = (r * o->cluster - 1) / p.Ns;       // tiles per species in r rounds
        if (per < 1) continue;
        const int t = (p.Nn + per - 1) / per;
        if (t <= BATCH_MAX_TILE) { T = t; break; }
      }
    } else {
      T = o->tile > 0 ? o->tile : 8;
    }
    T = std::max(1, std::min(std::min(T, BATCH_MAX_TILE), p.Nn));   // the coefficient scratch holds 32 planes
    int ntiles = (p.Nn + T - 1) / T;
    T = (p.Nn + ntiles - 1) / ntiles;
    I.P.tile = T;
    I.P.ntiles = ntiles;
    I.tab_off = (int)tab.size();
    tab.insert(tab.end(), tmp.tab.begin(), tmp.tab.end());
    coef_off[i] = coefs.size();
    coefs.insert(coefs.end(), tmp.coef.begin(), tmp.coef.end());
    tab_max = std::max(tab_max, I.P.tab_len);
    // work area: two line buffers (T+1 lines of M), staged planes (T+2 of Nx), field
    // lines (3); the field tile reuses it for its (2 Ns + 12)-line gather + output area
    work_max = std::max(work_max, std::max(2 * (T + 1) * I.P.axm.n + (T + 5) * p.Nx, (2 * p.Ns + 12) * p.Nx));
    if (o->hermitian && (p.Nx & 1)) {
      bool anti = true;
      for (int c = 0; c < p.Nx; ++c)
        if (!(tmp.tab[I.P.ax[1].kofs + c].x == -tmp.tab[I.P.ax[1].kofs + p.Nx - 1 - c].x)) anti = false;
      I.herm_ok = anti ? 1 : 0;
    }
    I.len = (long long)I.P.nc + 6LL * I.P.plane;
    I.pool_off = pool;
    pool += 17 * ((I.len + 15) / 16 * 16);
    I.y_off = yoff;
    b->y_off[i] = yoff;
    yoff += I.len;
    I.en_off = en_off;
    en_off += std::max(1, o->nsave) * (2 + p.Ns);
    for (int s = 0; s < SPX_MAX_SPECIES; ++s) I.masses[s] = 1.0;
    if (o->masses)
      for (int s = 0; s < p.Ns; ++s) I.masses[s] = o->masses[(size_t)i * SPX_MAX_SPECIES + s];
    // cost: the caller's (e.g. measured durations), else an estimate: FFT work
    // per RHS x stability-limited steps ~ k_max * alpha * sqrt(2 Nn)
    const double kmax = (p.Nx / 2) * 2.0 * M_PI / p.Lx;
    cost[i] = o->costs ? o->costs[i]
                       : (double)p.Ns * p.Nn * p.Nx * std::log2((double)p.Nx + 1.0) *
                             (1.0 + kmax * std::fabs(p.alpha_s[0]) * std::sqrt(2.0 * p.Nn));
  }
  b->total_len = yoff;
  b->en_total = en_off;
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  b->smem = ((size_t)tab_max * sizeof(double2) + 255) / 256 * 256 + (size_t)work_max * sizeof(double2) +
            BATCH_MAX_TILE * 4 * sizeof(double);
  const int optin = smem_optin();
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k_batch);
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "cudaFuncGetAttributes(k_batch)"); }
  if (b->smem + fa.sharedSizeBytes > (size_t)optin) {
    set_error("spx_batch_create: instances too large for shared memory (reduce tile)");
    batch_free(b);
    return SPX_E_UNSUPPORTED;
  }
  e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  // clusters of more than 8 CTAs need the non-portable size opt-in
  if (e == cudaSuccess && o->cluster > 8) e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "cudaFuncSetAttribute(k_batch)"); }
  // persistent grid: as many clusters as can be co-resident
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(o->cluster * 1024, 1, 1);
    cfg.blockDim = dim3(NTHREADS, 1, 1);
    cfg.dynamicSmemBytes = b->smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = o->cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int ncl = 0;
    e = cudaOccupancyMaxActiveClusters(&ncl, k_batch, &cfg);
    if (e != cudaSuccess || ncl <= 0) { batch_free(b); return cuda_fail(e == cudaSuccess ? cudaErrorInvalidConfiguration : e, "cudaOccupancyMaxActiveClusters"); }
    ncl = std::min(ncl, n);
    b->grid = ncl * o->cluster;
  }
  // one device block: args-side arrays + pool
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  size_t off = 0;
  const size_t o_inst = off; off += al(sizeof(BInst) * n);
  const size_t o_tab = off; off += al(sizeof(double2) * std::max<size_t>(1, tab.size()));
  const size_t o_order = off; off += al(sizeof(int) * n);
  const size_t o_next = off; off += al(sizeof(unsigned int));
  const size_t o_ts = off; off += al(sizeof(double) * std::max(1, o->nsave));
  const size_t o_en = off; off += al(sizeof(double) * std::max(1, en_off));
  const size_t o_yin = off; off += al(sizeof(double2) * b->total_len);
  const size_t o_yout = off; off += al(sizeof(double2) * b->total_len);
  const size_t o_pool = off; off += al(sizeof(double2) * pool);
  const size_t o_coef = off; off += al(sizeof(double) * std::max<size_t>(1, coefs.size()));
  e = cudaMalloc(&b->block, off);
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "cudaMalloc(batch)"); }
  char* d = static_cast<char*>(b->block);
  BArgs& A = b->args;
  A.inst = reinterpret_cast<BInst*>(d + o_inst);
  A.n = n;
  A.tab = reinterpret_cast<const double2*>(d + o_tab);
  A.order = reinterpret_cast<const int*>(d + o_order);
  A.next = reinterpret_cast<unsigned int*>(d + o_next);
  A.save_ts = reinterpret_cast<const double*>(d + o_ts);
  A.energies = reinterpret_cast<double*>(d + o_en);
  A.y_in = reinterpret_cast<const double2*>(d + o_yin);
  A.y_out = reinterpret_cast<double2*>(d + o_yout);
  A.pool = reinterpret_cast<double2*>(d + o_pool);
  A.nsave = o->nsave;
  A.t1 = o->t1; A.dt0 = o->dt0; A.rtol = o->rtol; A.atol = o->atol;
  A.max_steps = o->max_steps; A.adaptive = o->adaptive ? 1 : 0;
  A.interp = o->saveat == 0 ? 1 : 0;
  A.tab_max = tab_max;
  A.work_max = work_max;
  b->y_in = const_cast<double2*>(A.y_in);
  b->y_out = A.y_out;
  for (int i = 0; i < n; ++i) b->hinst[i].P.coef = reinterpret_cast<const double*>(d + o_coef) + coef_off[i];
  e = cudaMemcpy(A.inst, b->hinst.data(), sizeof(BInst) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !coefs.empty())
    e = cudaMemcpy(d + o_coef, coefs.data(), sizeof(double) * coefs.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !tab.empty()) e = cudaMemcpy(d + o_tab, tab.data(), sizeof(double2) * tab.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + o_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && o->nsave) e = cudaMemcpy(d + o_ts, o->save_ts, sizeof(double) * o->nsave, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d + o_en, 0, sizeof(double) * std::max(1, en_off));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    enqueue_batch(b, b->cap);
    e = cudaStreamEndCapture(b->cap, &b->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "batch set-up"); }
  *out = b;
  return SPX_OK;
}

int spx_batch_destroy(spx_batch* b) { return batch_free(b); }

int64_t spx_batch_offset(const spx_batch* b, int32_t i) {
  if (!b || i < 0 || i > b->n) return -1;
  return i == b->n ? b->total_len : b->y_off[i];
}

int spx_batch_run(spx_batch* b, const void* y0, void* y_final, void* stream) {
  if (!b || !y0) { set_error("spx_batch_run: null argument"); return SPX_E_ARG; }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t bytes = sizeof(double2) * b->total_len;
  SPX_CUDA(cudaMemcpyAsync(b->y_in, y0, bytes, cudaMemcpyDefault, st));
  SPX_CUDA(cudaGraphLaunch(b->exec, st));
  if (y_final) SPX_CUDA(cudaMemcpyAsync(y_final, b->y_out, bytes, cudaMemcpyDefault, st));
  return SPX_OK;
}

int spx_batch_results(spx_batch* b, spx_batch_stats* stats, double* energies, void* stream) {
  if (!b) { set_error("spx_batch_results: null batch"); return SPX_E_ARG; }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (energies)
    SPX_CUDA(cudaMemcpyAsync(energies, b->args.energies, sizeof(double) * b->en_total, cudaMemcpyDefault, st));
  if (stats) {
    std::vector<BInst> h(b->n);
    SPX_CUDA(cudaMemcpyAsync(h.data(), b->args.inst, sizeof(BInst) * b->n, cudaMemcpyDeviceToHost, st));
    SPX_CUDA(cudaStreamSynchronize(st));
    unsigned long long t0 = ~0ULL;
    for (int i = 0; i < b->n; ++i) t0 = std::min(t0, h[i].t_begin);
    for (int i = 0; i < b->n; ++i) {
      stats[i].start_s = 1e-9 * (double)(h[i].t_begin - t0);
      stats[i].end_s = 1e-9 * (double)(h[i].t_end - t0);
      stats[i].t = h[i].t; stats[i].dt = h[i].dt;
      stats[i].accepted = h[i].accepted; stats[i].rejected = h[i].rejected; stats[i].rhs_evals = h[i].evals;
      stats[i].status = h[i].status; stats[i].saved = h[i].saved;
      stats[i].hermitian = h[i].herm; stats[i].pad = 0;
    }
  }
  return SPX_OK;
}

int32_t spx_batch_energy_offset(const spx_batch* b, int32_t i) {
  if (!b || i < 0 || i >= b->n) return -1;
  return b->hinst[i].en_off;
}

int32_t spx_batch_grid(const spx_batch* b) { return b ? b->grid : -1; }

}  // extern "C"
