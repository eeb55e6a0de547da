// spx_dopri8.cu — device Prince-Dormand 8(7) solver for one large instance.
//
// One step attempt is a fixed launch sequence captured once as a CUDA graph and
// replayed; the host only replays graphs and polls the status word.
//
// Fused 1D1V path (13 stage launches + save): stage i stages its input planes
// (the tile's Hermite planes n0-1 .. n0+nt of S_i and the field lines G needs)
// into shared memory with bulk copies, and on a second barrier the operands of
// its epilogue (y and the K_j of its own planes), which land while the
// transforms run.  The epilogue stores K_i and the next input
// S_{i+1} = y + h sum_j a(i+1, j) K_j; the last stage forms y_new and the
// scaled error instead, and its last CTA to arrive (atomic ticket, no
// spin-wait) reduces the per-CTA sums in a fixed order and runs the step-size
// controller on the device.
//
// General path (13 x (real-space + stage) + save): the same epilogues with
// global operands.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "spx_plan.h"
#include "spx_rhs.cuh"
#include "spx_tableau.cuh"
#include "spx_stage.cuh"
#include "spx_tma.cuh"

namespace spx {

struct D8Dev {
  double t, dt, t0, t1, rtol, atol;
  long long accepted, rejected, evals, max_steps;
  int status, adaptive, cur, k1_valid;
  int isave, nsave, save_pending, save_lo, save_hi, saved;
  unsigned int arrive;
  int herm;           // 1: the state is exactly Hermitian, stages use packed real transforms
  unsigned int att;       // attempts finished since reset (the persistent kernel's attempt barrier)
  unsigned int save_seq;  // incremented whenever an accepted step crosses save times
  int interp;             // 1: save times inside a step are interpolated (steps end only on t1)
  int wait_polls;         // poll limit of the persistent kernel's counter waits; < 0: the
                          // waits ask for a count nobody publishes (time-out test), limit -wait_polls
  double save_t0, save_h; // the accepted step a pending save interpolates ([t0, t0 + h]); h = 0: none
};

struct D8Args {
  const DevPlan* plan;
  const double2* tab;
  D8Dev* st;
  double2* Y[2];
  double2* S[2];
  double2* K;
  double2* ws;
  double* part;
  const double* save_ts;
  double2* saved;
  double* energies;
  const double* masses;
  long long len;
  int npf;            // fused 1D1V path: epilogue operands staged in shared memory (y first)
  double2* S3;        // persistent kernel: third stage-input buffer (ring S0, S1, S3)
  unsigned int* done; // persistent kernel: stages finished since reset, per CTA
};

// Element i (0 or 1) of a two-pointer kernel argument, by select: indexing the
// argument array with a runtime index would copy the argument block to local memory.
template <class T>
__device__ __forceinline__ T* pick(T* const (&p)[2], int i) { return i ? p[1] : p[0]; }

// a(i+1, j) rows for i = 0..11, then b (row 12) and e (row 13); nonzero masks
__constant__ double cCoef[14][13];
__constant__ int cMask[14];


struct Attempt {
  double h, t_stop;
  int landed, go;
};

__device__ __forceinline__ Attempt attempt_params(const D8Dev& s, const double* __restrict__ ts) {
  Attempt a;
  a.t_stop = (s.isave < s.nsave && !s.interp) ? fmin(ts[s.isave], s.t1) : s.t1;
  a.h = s.dt;
  a.landed = 0;
  if (s.t + a.h * (1.0 + rk::SNAP) >= a.t_stop) { a.h = a.t_stop - s.t; a.landed = 1; }
  const bool ok = !(a.h <= 0.0 || s.t + a.h == s.t);
  a.go = (s.status == SPX_ST_RUNNING) && (s.accepted + s.rejected < s.max_steps) && ok;
  return a;
}

// Epilogue of stages 0..11: store K_i, write the next stage input.
struct EpiStage {
  const double2* __restrict__ Y;
  double2* __restrict__ K;
  double2* __restrict__ Snext;
  long long len;
  int stage;
  const double* hc;   // h a(stage+1, j) for j <= stage, formed once per CTA
  __device__ __forceinline__ void operator()(size_t e, double2 v) const {
    K[(size_t)stage * len + e] = v;
    const int mask = cMask[stage];   // coefficients a(stage+1, j)
    double2 acc = Y[e];
    for (int j = 0; j < stage; ++j)
      if (mask & (1 << j)) acc = crfma(hc[j], K[(size_t)j * len + e], acc);
    acc = crfma(hc[stage], v, acc);
    Snext[e] = acc;
  }
};

// Epilogue of the last stage: y_new, scaled error, non-finite flag.
struct EpiLast {
  const double2* __restrict__ Y;
  const double2* __restrict__ K;
  double2* __restrict__ Ynew;
  double2* __restrict__ K12;   // the last stage's K (read by the dense output)
  long long len;
  const double* hb;   // h b_j and h e_j (j <= 12), formed once per CTA
  const double* he;
  double rtol, atol;
  int adaptive;
  double sq;
  int nonfinite;
  __device__ __forceinline__ void operator()(size_t e, double2 v) {
    const double2 y0 = Y[e];
    double2 yn = y0;
    double2 er = make_double2(0.0, 0.0);
    const int mb = cMask[12], me = cMask[13];
    for (int j = 0; j < 12; ++j) {
      const bool ub = mb & (1 << j), ue = me & (1 << j);
      if (ub || ue) {
        const double2 kj = K[(size_t)j * len + e];
        if (ub) yn = crfma(hb[j], kj, yn);
        if (ue) er = crfma(he[j], kj, er);
      }
    }
    yn = crfma(hb[12], v, yn);
    er = crfma(he[12], v, er);
    Ynew[e] = yn;
    K12[e] = v;
    if (!(isfinite(yn.x) && isfinite(yn.y))) nonfinite = 1;
    if (adaptive) {
      const double m0 = fma(y0.x, y0.x, y0.y * y0.y), m1 = fma(yn.x, yn.x, yn.y * yn.y);
      const double inv = 1.0 / fma(rtol, sqrt(fmax(m0, m1)), atol);   // one division per entry
      const double rx = er.x * inv, ry = er.y * inv;
      sq = fma(rx, rx, fma(ry, ry, sq));
    }
  }
};

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += red[i];
  return r;   // valid in thread 0
}

// Thread 0 of the last CTA of an attempt: accept/reject, advance the clock.
__device__ void finalize_step(const D8Args& a, const Attempt& at, double sum, int nonf) {
  D8Dev* st = a.st;
  const double en = sqrt(sum / (double)a.len);
  bool accept;
  double dt_next;
  if (st->adaptive) {
    accept = en < 1.0;
    dt_next = at.h * rk::controller_factor(en, accept);
    if (accept && at.landed && dt_next < st->dt) dt_next = st->dt;
  } else {
    accept = true;
    dt_next = st->dt;
  }
  st->evals += st->k1_valid ? (rk::S - 1) : rk::S;
  if (accept) {
    st->save_t0 = st->t;
    st->save_h = at.h;
    st->t = at.landed ? at.t_stop : st->t + at.h;
    st->cur ^= 1;
    st->accepted += 1;
    st->k1_valid = 0;
    int lo = st->isave, hi = lo;
    while (hi < st->nsave && __ldcg(a.save_ts + hi) <= st->t) ++hi;
    if (hi > lo) {
      st->save_pending = 1; st->save_lo = lo; st->save_hi = hi; st->isave = hi;
      st->save_seq += 1;
    }
    if (nonf) st->status = SPX_ST_NONFINITE;
    else if (st->t >= st->t1) st->status = SPX_ST_DONE;
  } else {
    st->rejected += 1;
    st->k1_valid = 1;
  }
  st->dt = dt_next;
  st->arrive = 0;
  __threadfence();
  // publish: the persistent kernel's CTAs wait for this count before the next attempt
  st_release_u32(&st->att, st->att + 1);
}

// Elements owned by CTA `b` on the fused 1D1V path (plane tiles, then the field CTA).
template <class F>
__device__ void for_each_owned_1v(const DevPlan& P, int b, F&& f) {
  const int nblk = P.pb.Ns * P.ntiles;
  if (b == nblk) {
    const size_t n = 6 * (size_t)P.plane;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) f((size_t)P.nc + i);
    return;
  }
  const int s = b / P.ntiles, tile = b % P.ntiles;
  const int n0 = tile * P.tile;
  const int nt = min(P.tile, P.pb.Nn - n0);
  const int N = P.ax[1].n;
  const size_t base = ((size_t)s * P.pb.Nn + n0) * N;
  for (int i = threadIdx.x; i < nt * N; i += blockDim.x) f(base + i);
}

template <class F>
__device__ void for_each_owned_gen(const DevPlan& P, int b, F&& f) {
  const int nplanes = P.pb.Ns * P.nh;
  const size_t pl = (size_t)P.plane;
  const size_t base = (b == nplanes) ? (size_t)P.nc : (size_t)b * pl;
  const size_t n = (b == nplanes) ? 6 * pl : pl;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) f(base + i);
}

// Common tail of an attempt: per-CTA partial sums, then an atomic ticket; the
// last CTA to arrive (no spin-wait) reduces all partials with every thread in a
// fixed order and runs the controller.
template <class EL>
__device__ void last_stage_tail(const D8Args& a, const Attempt& at, EL& el, double* red) {
  __shared__ int last;
  const double s1 = block_sum(el.sq, red);
  __syncthreads();
  const double s2 = block_sum((double)el.nonfinite, red);
  if (threadIdx.x == 0) {
    a.part[2 * blockIdx.x] = s1;
    a.part[2 * blockIdx.x + 1] = s2;
    __threadfence();
    const unsigned int ticket = atomicAdd(&a.st->arrive, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double sum = 0.0, nf = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    sum += __ldcg(a.part + 2 * b);
    nf += __ldcg(a.part + 2 * b + 1);
  }
  sum = block_sum(sum, red);
  __syncthreads();
  nf = block_sum(nf, red);
  if (threadIdx.x == 0) finalize_step(a, at, sum, nf != 0.0);
}

// ------------------------------------------------------------------ stage kernels
// Epilogue term lists: stage i < 12 forms the next input y + h sum_j a(i+1, j)
// K_j over j < i with a(i+1, j) != 0 (then + h a(i+1, i) K_i); the last stage
// forms y_new and the error over j < 12 with b_j != 0 or e_j != 0.  Ascending j.
__constant__ int cEpiN[13];
__constant__ int cEpiJ[13][MAX_TERMS];

// Called by the 32 lanes of warp 0, one term per lane (a handful of warp-level
// FP64 multiplies instead of a serial loop in one thread).
__device__ void fill_terms(EpiTerms& T, int stage, double h) {
  const bool last = stage == rk::S - 1;
  const int row = last ? 12 : stage;
  const int lane = threadIdx.x & 31;
  const int n = cEpiN[stage];
  if (lane < n) {
    const int j = cEpiJ[stage][lane];
    T.j[lane] = j;
    T.c[lane] = h * cCoef[row][j];
    T.e[lane] = last ? h * cCoef[13][j] : 0.0;
  }
  if (lane == 0) {
    T.n = n;
    T.cself = h * cCoef[row][stage];
    T.eself = last ? h * cCoef[13][stage] : 0.0;
  }
}

// One stage of the fused 1D1V path (staged_stage_1v): stage inputs and
// epilogue operands arrive by bulk copies; the last stage (LAST) forms y_new
// and the error and runs the controller in its last CTA.
// MG: the plan's products run on its own product grid (axm.n != Nx); one
// kernel per case so the Nx-grid kernel keeps its smaller register allocation
template <bool LAST, bool MG>
__global__ void __launch_bounds__(NTHREADS, 2) k_d8_stage_1v(D8Args a, int stage) {
  __shared__ DevPlan P;
  __shared__ D8Dev s;
  __shared__ double red[NTHREADS / 32];
  __shared__ EpiTerms terms;
  __shared__ Attempt sat;
  __shared__ __align__(8) uint64_t bars[2];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  // prologue independent of the previous launch; then wait for it (PDL)
  load_plan(P, stab, a.plan, a.tab);
  pdl_wait_and_release();
  // the attempt's scalars once per CTA (FP64 compares and products cost the
  // same per warp whatever the number of active lanes)
  if (threadIdx.x == 0) {
    s = *a.st;
    sat = attempt_params(s, a.save_ts);
    if (stage == 0 && blockIdx.x == 0) a.st->save_pending = 0;
  }
  __syncthreads();
  const Attempt at = sat;
  if (!at.go) {
    if (LAST && blockIdx.x == 0 && threadIdx.x == 0 && s.status == SPX_ST_RUNNING)
      a.st->status = (s.accepted + s.rejected >= s.max_steps) ? SPX_ST_MAX_STEPS : SPX_ST_DT_UNDERFLOW;
    return;
  }
  if (threadIdx.x < 32) fill_terms(terms, stage, at.h);
  __syncthreads();   // every thread reads terms.n when it sizes the staged operands
  const long long len = a.len;
  const double2* Y = pick(a.Y, s.cur);
  double2* Ki = a.K + (size_t)stage * len;
  if (!LAST && stage == 0 && s.k1_valid) {
    // rejected attempt: K_0 = f(y) is kept; rebuild the next input y + h a(1,0) K_0
    __syncthreads();
    const int nblk = P.pb.Ns * P.ntiles, N = P.ax[1].n, b = blockIdx.x;
    double2* Sn = pick(a.S, 1);
    auto one = [&](size_t e) { Sn[e] = crfma(terms.cself, Ki[e], Y[e]); };
    if (b == nblk) {
      for (int i = threadIdx.x; i < 6 * N; i += blockDim.x) one((size_t)P.nc + i);
    } else {
      const int sp = b / P.ntiles, n0 = (b % P.ntiles) * P.tile, nt = min(P.tile, P.pb.Nn - n0);
      const size_t base = ((size_t)sp * P.pb.Nn + n0) * N;
      for (int i = threadIdx.x; i < nt * N; i += blockDim.x) one(base + i);
    }
    return;
  }
  StageIO io;
  io.in = (stage == 0) ? Y : pick(a.S, stage & 1);
  io.Y = Y;
  io.K = a.K;
  io.len = len;
  io.Ki = Ki;
  io.out = LAST ? pick(a.Y, s.cur ^ 1) : pick(a.S, (stage + 1) & 1);
  io.npf = a.npf;
  io.herm = s.herm != 0;
  io.rtol = s.rtol;
  io.atol = s.atol;
  io.adaptive = s.adaptive;
  io.timeout_status = &a.st->status;
  io.persistent = false;
  staged_stage_1v<LAST, 2, MG ? 1 : 0>(P, stab, io, terms, bars, [&](auto& el) { last_stage_tail(a, at, el, red); });
}

// ------------------------------------------------------------------ persistent 1D1V solver
// All attempts of a replay in one cooperative launch (every CTA resident): a CTA
// starts stage i as soon as the CTAs whose data it reads have finished stage i-1
// (per-CTA completion counters, release/acquire), instead of waiting for the
// whole grid at a kernel boundary.  Stage inputs rotate through three buffers;
// the field CTA, whose output every tile reads, also waits until every tile has
// finished stage i-2, so no buffer is overwritten while a slower CTA reads it.
// After stage 12 the last CTA runs the controller and bumps st->att; every CTA
// waits for that (attempt barrier), then performs pending saves.  Every wait is
// bounded and ends the solve with SPX_ST_WAIT_TIMEOUT.

// Copy of the controller state through L2 (other CTAs wrote it in this launch).
__device__ __forceinline__ void load_state_l2(D8Dev& s, const D8Dev* st) {
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(st);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&s);
  for (int i = 0; i < (int)(sizeof(D8Dev) / 8); ++i) dst[i] = __ldcg(src + i);
}

// Energies of spectrax/_diagnostics.py:191-219 (EM, kinetic total, kinetic per
// species) of the state whose entries val(e) returns, into e[0 .. 2 + Ns), by one
// CTA (the result is valid in thread 0, which writes it).
template <class V>
__device__ void save_energies(const DevPlan& P, const double* masses, V&& val, double* out, double* red) {
  const spx_problem& pb = P.pb;
  const size_t pl = (size_t)P.plane;
  double em = 0.0;
  for (size_t i = threadIdx.x; i < 6 * pl; i += blockDim.x) {
    const double2 f = val((size_t)P.nc + i);
    em = fma(f.x, f.x, fma(f.y, f.y, em));
  }
  em = block_sum(em, red);
  if (threadIdx.x == 0) {
    const int Ns = pb.Ns;
    const int Hs = P.nh;
    const int kc = ((P.ax[0].n / 2) * P.ax[1].n + P.ax[1].n / 2) * P.ax[2].n + P.ax[2].n / 2;
    const int offs[7] = {0, 1, pb.Nn, pb.Nn * pb.Nm, 2, 2 * pb.Nn, 2 * pb.Nn * pb.Nm};
    const double O0 = pb.Omega_cs[0];
    double ke_tot = 0.0;
    for (int sp = 0; sp < Ns; ++sp) {
      double c[7];
      for (int k = 0; k < 7; ++k)
        c[k] = (offs[k] >= 0 && offs[k] < Hs) ? val(((size_t)sp * Hs + offs[k]) * pl + kc).x : 0.0;
      const double a0 = pb.alpha_s[3 * sp], a1 = pb.alpha_s[3 * sp + 1], a2 = pb.alpha_s[3 * sp + 2];
      const double u0 = pb.u_s[3 * sp], u1 = pb.u_s[3 * sp + 1], u2 = pb.u_s[3 * sp + 2];
      const double pref = 0.5 * masses[sp] * a0 * a1 * a2;
      const double t0 = 0.5 * (a0 * a0 + a1 * a1 + a2 * a2) + (u0 * u0 + u1 * u1 + u2 * u2);
      const double t1 = 1.41421356237309504880 * (a0 * u0 * c[1] + a1 * u1 * c[2] + a2 * u2 * c[3]);
      const double t2 = 0.70710678118654752440 * (a0 * a0 * c[4] + a1 * a1 * c[5] + a2 * a2 * c[6]);
      out[2 + sp] = pref * (t0 * c[0] + t1 + t2);
      ke_tot += out[2 + sp];
    }
    out[0] = 0.5 * em * O0 * O0;
    out[1] = ke_tot;
  }
}

// Energies of one saved state of the persistent kernel (land-on-save mode: the
// state itself), by one CTA through L2, for every pending save index.
__device__ void persist_energies(const D8Args& a, const DevPlan& P, const D8Dev& s, const double2* Y,
                                 double* red) {
  const int Ns = P.pb.Ns;
  double* e0 = a.energies + (size_t)s.save_lo * (2 + Ns);
  save_energies(P, a.masses, [&](size_t e) { return __ldcg(Y + e); }, e0, red);
  if (threadIdx.x == 0) {
    for (int idx = s.save_lo + 1; idx < s.save_hi; ++idx)
      for (int q = 0; q < 2 + Ns; ++q) a.energies[(size_t)idx * (2 + Ns) + q] = e0[q];
    a.st->saved = s.save_hi;
  }
}

__global__ void __launch_bounds__(NTHREADS, 2) k_d8_persist(D8Args a, int natt) {
  __shared__ DevPlan P;
  __shared__ D8Dev s;
  __shared__ Attempt at;
  __shared__ double red[NTHREADS / 32];
  __shared__ EpiTerms terms;
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ unsigned int saves_seen;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, a.plan, a.tab);
  // uniform values live in shared memory (P, s, at): registers stay with the stage body
  if (threadIdx.x == 0) {
    load_state_l2(s, a.st);
    saves_seen = s.save_seq;
  }
  __syncthreads();
  for (int q = 0; q < natt; ++q) {
    if (threadIdx.x == 0) {
      load_state_l2(s, a.st);
      at = attempt_params(s, a.save_ts);
    }
    __syncthreads();
    if (!at.go) {
      if (blockIdx.x == 0 && threadIdx.x == 0 && s.status == SPX_ST_RUNNING)
        a.st->status = (s.accepted + s.rejected >= s.max_steps) ? SPX_ST_MAX_STEPS : SPX_ST_DT_UNDERFLOW;
      return;
    }
    for (int stage = 0; stage < rk::S; ++stage) {
      // the producers of this stage's inputs have finished stage - 1
      const int nblk = P.pb.Ns * P.ntiles;
      bool ok = true;
      const int polls = s.wait_polls < 0 ? -s.wait_polls : s.wait_polls;
      // time-out test: a target no CTA ever publishes
      const unsigned int never = s.wait_polls < 0 ? 0x40000000u : 0u;
      if (stage > 0) {
        const unsigned int need = s.att * rk::S + stage + never;
        const int b = blockIdx.x;
        if (b < nblk) {
          const int tl = b % P.ntiles;
          if (threadIdx.x == 0 && tl > 0) ok = wait_counter(a.done + b - 1, need, polls);
          if (threadIdx.x == 1 && tl + 1 < P.ntiles) ok = wait_counter(a.done + b + 1, need, polls);
          if (threadIdx.x == 2) ok = wait_counter(a.done + nblk, need, polls);
        } else {
          // the field CTA reads the tiles holding planes 0 and 1; the others must be
          // past stage - 2 before this stage overwrites their stage - 2 input buffer
          const int t01 = 1 / P.tile;
          for (int c = threadIdx.x; c < nblk && ok; c += blockDim.x)
            ok = wait_counter(a.done + c, (c % P.ntiles) <= t01 ? need : need - 1, polls);
        }
      }
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(&a.st->status, SPX_ST_WAIT_TIMEOUT);
        return;
      }
      if (threadIdx.x < 32) fill_terms(terms, stage, at.h);
      __syncthreads();
      const long long len = a.len;
      const double2* Y = s.cur ? a.Y[1] : a.Y[0];
      double2* Ki = a.K + (size_t)stage * len;
      auto ring = [&](int i) { return i == 0 ? a.S[0] : (i == 1 ? a.S[1] : a.S3); };
      if (stage == 0 && s.k1_valid) {
        // rejected attempt: K_0 = f(y) is kept; rebuild the next input y + h a(1,0) K_0
        double2* Sn = ring(1);
        for_each_owned_1v(P, blockIdx.x, [&](size_t e) { Sn[e] = crfma(terms.cself, Ki[e], Y[e]); });
      } else {
        StageIO io;
        io.in = (stage == 0) ? Y : ring(stage % 3);
        io.Y = Y;
        io.K = a.K;
        io.len = len;
        io.Ki = Ki;
        io.out = (stage == rk::S - 1) ? (s.cur ? a.Y[0] : a.Y[1]) : ring((stage + 1) % 3);
        io.npf = a.npf;
        io.herm = s.herm != 0;
        io.rtol = s.rtol;
        io.atol = s.atol;
        io.adaptive = s.adaptive;
        io.timeout_status = &a.st->status;
        io.persistent = true;
        const bool ok_stage =
            (stage < rk::S - 1)
                ? staged_stage_1v<false, 2, 0>(P, stab, io, terms, bars, [](auto&) {})
                : staged_stage_1v<true, 2, 0>(P, stab, io, terms, bars, [&](auto& el) { last_stage_tail(a, at, el, red); });
        if (!ok_stage) return;   // status already says WAIT_TIMEOUT; the CTAs waiting on this one time out too
      }
      // this stage's writes (generic proxy) are read by later bulk copies (async proxy)
      fence_proxy_async();
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        st_release_u32(a.done + blockIdx.x, s.att * rk::S + stage + 1);
      }
    }
    // attempt barrier: the controller of this attempt has run
    bool ok = true;
    if (threadIdx.x == 0) {
      const int polls = s.wait_polls < 0 ? -s.wait_polls : s.wait_polls;
      ok = wait_counter(&a.st->att, s.att + 1 + (s.wait_polls < 0 ? 0x40000000u : 0u), polls);
    }
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicExch(&a.st->status, SPX_ST_WAIT_TIMEOUT);
      return;
    }
    if (threadIdx.x == 0) load_state_l2(s, a.st);
    __syncthreads();
    if (s.save_seq != saves_seen) {
      const double2* Yc = s.cur ? a.Y[1] : a.Y[0];
      if (a.saved)
        for (int idx = s.save_lo; idx < s.save_hi; ++idx) {
          double2* dst = a.saved + (size_t)idx * a.len;
          for_each_owned_1v(P, blockIdx.x, [&](size_t e) { dst[e] = __ldcg(Yc + e); });
        }
      if ((int)blockIdx.x == P.pb.Ns * P.ntiles) persist_energies(a, P, s, Yc, red);
      __syncthreads();
      if (threadIdx.x == 0) saves_seen = s.save_seq;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(GEN_THREADS, 1) k_d8_real(D8Args a, int stage) {
  __shared__ DevPlan P;
  __shared__ D8Dev s;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  __shared__ Attempt sat;
  load_plan(P, stab, a.plan, a.tab);
  pdl_wait_and_release();
  if (threadIdx.x == 0) {
    s = *a.st;
    sat = attempt_params(s, a.save_ts);
  }
  __syncthreads();
  const Attempt at = sat;
  if (!at.go || (stage == 0 && s.k1_valid)) return;
  const double2* in = (stage == 0) ? pick(a.Y, s.cur) : pick(a.S, stage & 1);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  general_to_real(P, stab, in, blockIdx.x, a.ws + (size_t)blockIdx.x * P.plane, sA, sB);
}

template <bool LAST>
__global__ void __launch_bounds__(GEN_THREADS, 1) k_d8_stage_gen(D8Args a, int stage) {
  __shared__ DevPlan P;
  __shared__ D8Dev s;
  __shared__ double red[GEN_THREADS / 32];
  __shared__ Attempt sat;
  __shared__ double hcs[2][16];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, a.plan, a.tab);
  pdl_wait_and_release();
  if (threadIdx.x == 0) {
    s = *a.st;
    sat = attempt_params(s, a.save_ts);
    if (stage == 0 && blockIdx.x == 0) a.st->save_pending = 0;
  }
  __syncthreads();
  const Attempt at = sat;
  if (!at.go) {
    if (stage == rk::S - 1 && blockIdx.x == 0 && threadIdx.x == 0 && s.status == SPX_ST_RUNNING) {
      a.st->status = (s.accepted + s.rejected >= s.max_steps) ? SPX_ST_MAX_STEPS : SPX_ST_DT_UNDERFLOW;
    }
    return;
  }
  // stage coefficients times h, one lane each
  if (threadIdx.x < rk::S) {
    const int j = threadIdx.x;
    hcs[0][j] = at.h * cCoef[LAST ? 12 : stage][j];
    hcs[1][j] = LAST ? at.h * cCoef[13][j] : 0.0;
  }
  __syncthreads();
  const double2* Y = pick(a.Y, s.cur);
  const double2* in = (stage == 0) ? Y : pick(a.S, stage & 1);
  const int nplanes = P.pb.Ns * P.nh;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int b = blockIdx.x;
  const double2* GB = a.ws + (size_t)nplanes * P.plane;
  if constexpr (!LAST) {
    EpiStage epi{Y, a.K, pick(a.S, (stage + 1) & 1), a.len, stage, hcs[0]};
    if (stage == 0 && s.k1_valid) {
      for_each_owned_gen(P, b, [&](size_t e) { epi(e, a.K[e]); });
    } else if (b == nplanes) {
      maxwell_range(P, stab, in, 0, P.plane, epi);
    } else {
      general_nl_plane(P, stab, in, a.ws, GB, b, sA, sB, epi);
    }
  } else {
    EpiLast el{Y, a.K, pick(a.Y, s.cur ^ 1), a.K + (size_t)(rk::S - 1) * a.len, a.len, hcs[0], hcs[1],
               s.rtol, s.atol, s.adaptive, 0.0, 0};
    if (b == nplanes) maxwell_range(P, stab, in, 0, P.plane, el);
    else general_nl_plane(P, stab, in, a.ws, GB, b, sA, sB, el);
    last_stage_tail(a, at, el, red);
  }
}

// Copy the current state (Y[st->cur], chosen on the device) to dst: device
// memory or page-locked host memory (written through the mapped address), so
// reading the state out needs no host round trip for the buffer index.
__global__ void __launch_bounds__(NTHREADS) k_d8_export(D8Args a, double2* __restrict__ dst) {
  const double2* Y = pick(a.Y, a.st->cur);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.len; i += (long long)gridDim.x * blockDim.x)
    dst[i] = Y[i];
}

// Exact Hermitian test of a fused-1D1V state (odd Nx): every line of Nx entries
// (Hermite planes and field components) must satisfy y(N-1-c) == conj y(c).
// Any violation clears *flag (set to 1 by the caller).
__global__ void __launch_bounds__(NTHREADS) k_d8_herm_check(const double2* __restrict__ y, long long nlines,
                                                           int N, int* flag) {
  const long long total = nlines * N;
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / N;
    const int c = (int)(i - l * N);
    const double2 a = y[i], b = y[l * N + (N - 1 - c)];
    if (!(a.x == b.x && a.y == -b.y)) bad = 1;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicAnd(flag, 0);
}

// Save: for every pending save index, the state at that save time -- the current
// state when the time is the end of the accepted step (or in land-on-save mode),
// otherwise the dense output y_old + sum_j h b_j(theta) K_j of the step just
// accepted -- copied out if states are kept, and its energies.
__global__ void __launch_bounds__(NTHREADS) k_d8_save(D8Args a) {
  __shared__ D8Dev s;
  __shared__ double red[NTHREADS / 32];
  __shared__ double w[rk::S];
  pdl_wait_and_release();
  if (threadIdx.x == 0) s = *a.st;
  __syncthreads();
  if (!s.save_pending) return;
  const double2* Yn = pick(a.Y, s.cur);
  const double2* Yo = pick(a.Y, s.cur ^ 1);
  const long long len = a.len;
  const DevPlan& P = *a.plan;
  for (int idx = s.save_lo; idx < s.save_hi; ++idx) {
    const double tsv = a.save_ts[idx];
    const bool exact = !s.interp || s.save_h == 0.0 || tsv == s.t;
    if (threadIdx.x < rk::S)
      w[threadIdx.x] = exact ? 0.0 : s.save_h * rk::dense_weight(threadIdx.x, (tsv - s.save_t0) / s.save_h);
    __syncthreads();
    auto val = [&](size_t e) -> double2 {
      if (exact) return Yn[e];
      double2 v = Yo[e];
#pragma unroll 1
      for (int j = 0; j < rk::S; ++j)
        if (w[j] != 0.0) v = crfma(w[j], a.K[(size_t)j * len + e], v);
      return v;
    };
    if (a.saved) {
      double2* dst = a.saved + (size_t)idx * len;
      for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len;
           i += (long long)gridDim.x * blockDim.x)
        dst[i] = val((size_t)i);
    }
    if (blockIdx.x == 0) save_energies(P, a.masses, val, a.energies + (size_t)idx * (2 + P.pb.Ns), red);
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.st->saved = s.save_hi;
}

}  // namespace spx

// ------------------------------------------------------------------ host side
using namespace spx;

struct spx_dopri8 {
  const spx_plan* plan = nullptr;
  D8Args args{};
  D8Dev init{};
  void* block = nullptr;
  int nsave = 0;
  int grid_stage = 0, grid_real = 0;
  size_t smem_stage = 0;      // dynamic shared memory of the stage kernels
  int attempts_per_graph = 8;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr, graph1 = nullptr;
  cudaGraphExec_t exec = nullptr, exec1 = nullptr;   // `attempts_per_graph` attempts / one attempt
  int* h_status = nullptr;   // pinned
  std::vector<double> ts;
  bool herm_allowed = false;  // requested, fused 1D1V path, odd Nx, antisymmetric k table
  bool persistent = false;    // attempts run by k_d8_persist (one cooperative launch per replay)
  D8Dev* d_init = nullptr;    // the reset record, in device memory (reset copies it without a host wait)
};

static bool g_d8_consts = false;
constexpr int kDefaultWaitPolls = 1 << 22;   // ~0.3-1 s of polling with short sleeps

static int upload_consts() {
  if (g_d8_consts) return SPX_OK;
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
  int tn[13], tj[13][MAX_TERMS];
  std::memset(tj, 0, sizeof(tj));
  for (int i = 0; i < 13; ++i) {
    tn[i] = 0;
    for (int j = 0; j < i; ++j) {
      const bool use = (i < 12) ? (c[i][j] != 0.0) : (c[12][j] != 0.0 || c[13][j] != 0.0);
      if (!use) continue;
      if (tn[i] == MAX_TERMS) { set_error("tableau has more stage terms than supported"); return SPX_E_UNSUPPORTED; }
      tj[i][tn[i]++] = j;
    }
  }
  SPX_CUDA(cudaMemcpyToSymbol(cCoef, c, sizeof(c)));
  SPX_CUDA(cudaMemcpyToSymbol(cMask, m, sizeof(m)));
  SPX_CUDA(cudaMemcpyToSymbol(cEpiN, tn, sizeof(tn)));
  SPX_CUDA(cudaMemcpyToSymbol(cEpiJ, tj, sizeof(tj)));
  g_d8_consts = true;
  return SPX_OK;
}

static int d8_attrs() {
  static bool done = false;
  if (done) return SPX_OK;
  const int optin = smem_optin();
  cudaFuncAttributes fa;
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_stage_1v<false, false>));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_stage_1v<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_stage_1v<true, false>));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_stage_1v<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_stage_1v<false, true>));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_stage_1v<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_stage_1v<true, true>));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_stage_1v<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_persist));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_real));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_real, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_stage_gen<false>));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_stage_gen<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  SPX_CUDA(cudaFuncGetAttributes(&fa, k_d8_stage_gen<true>));
  SPX_CUDA(cudaFuncSetAttribute(k_d8_stage_gen<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  done = true;
  return SPX_OK;
}


// The reset record (device copy of the controller state at t0): a save time at
// (or before) t0 is taken from y0.
static cudaError_t write_reset_record(spx_dopri8* s) {
  D8Dev R = s->init;
  R.cur = 0;
  int hi = 0;
  while (hi < s->nsave && s->ts[hi] <= R.t0) ++hi;
  if (hi > 0) { R.save_pending = 1; R.save_lo = 0; R.save_hi = hi; R.isave = hi; }
  if (R.t0 >= R.t1) R.status = SPX_ST_DONE;
  R.herm = s->herm_allowed ? 1 : 0;
  return cudaMemcpy(s->d_init, &R, sizeof(R), cudaMemcpyHostToDevice);
}

// All `natt` attempts in one cooperative launch (every CTA co-resident).
static void enqueue_persistent(spx_dopri8* s, cudaStream_t st, int natt) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(s->grid_stage, 1, 1);
  cfg.blockDim = dim3(s->plan->threads, 1, 1);
  cfg.dynamicSmemBytes = s->smem_stage;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_d8_persist, s->args, natt);
}

static void enqueue_attempt(spx_dopri8* s, cudaStream_t st) {
  const DevPlan& P = s->plan->host;
  for (int stage = 0; stage < rk::S; ++stage) {
    if (P.path == 0) {
      const bool mg = P.axm.n != P.ax[1].n;
      auto k = stage < rk::S - 1 ? (mg ? k_d8_stage_1v<false, true> : k_d8_stage_1v<false, false>)
                                 : (mg ? k_d8_stage_1v<true, true> : k_d8_stage_1v<true, false>);
      launch_pdl(k, s->grid_stage, s->plan->threads, s->smem_stage, st, s->args, stage);
    } else {
      launch_pdl(k_d8_real, s->grid_real, GEN_THREADS, s->plan->smem_gen, st, s->args, stage);
      if (stage < rk::S - 1)
        launch_pdl(k_d8_stage_gen<false>, s->grid_stage, GEN_THREADS, s->smem_stage, st, s->args, stage);
      else
        launch_pdl(k_d8_stage_gen<true>, s->grid_stage, GEN_THREADS, s->smem_stage, st, s->args, stage);
    }
  }
  launch_pdl(k_d8_save, s->plan->nsm, (int)NTHREADS, (size_t)0, st, s->args);
}

static int d8_free(spx_dopri8* s) {
  if (!s) return SPX_OK;
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  if (s->exec1) cudaGraphExecDestroy(s->exec1);
  if (s->graph1) cudaGraphDestroy(s->graph1);
  if (s->cap) cudaStreamDestroy(s->cap);
  if (s->block) cudaFree(s->block);
  if (s->h_status) cudaFreeHost(s->h_status);
  delete s;
  return SPX_OK;
}

extern "C" {

int spx_dopri8_create(const spx_plan* plan, const spx_dopri8_opts* o, spx_dopri8** out) {
  if (!plan || !o || !out) { set_error("spx_dopri8_create: null argument"); return SPX_E_ARG; }
  *out = nullptr;
  if (int rd = check_plan_device(plan, "spx_dopri8_create")) return rd;
  if (!(o->t1 >= o->t0) || !(o->dt0 > 0.0) || o->nsave < 0 || (o->nsave > 0 && !o->save_ts) ||
      o->max_steps <= 0 || o->saveat < 0 || o->saveat > 1) {
    set_error("spx_dopri8_create: bad options"); return SPX_E_ARG;
  }
  if (o->adaptive && !(o->rtol >= 0.0 && o->atol >= 0.0 && o->rtol + o->atol > 0.0)) {
    set_error("spx_dopri8_create: tolerances must be non-negative and not both zero"); return SPX_E_ARG;
  }
  for (int i = 1; i < o->nsave; ++i)
    if (!(o->save_ts[i] >= o->save_ts[i - 1])) { set_error("save times must be non-decreasing"); return SPX_E_ARG; }
  if (plan->big) {
    set_error("spx_dopri8_create: a Fourier plane of this size does not fit in shared memory "
              "(drive spx_rhs from the host instead)");
    return SPX_E_UNSUPPORTED;
  }
  int rc;
  if ((rc = upload_consts()) != SPX_OK) return rc;
  if ((rc = d8_attrs()) != SPX_OK) return rc;
  spx_dopri8* s = new spx_dopri8();
  s->plan = plan;
  const DevPlan& P = plan->host;
  const long long len = (long long)P.nc + 6LL * P.plane;
  const int Ns = P.pb.Ns;
  s->nsave = o->nsave;
  s->grid_stage = (P.path == 0) ? P.pb.Ns * P.ntiles + 1 : P.pb.Ns * P.nh + 1;
  s->grid_real = (P.path == 0) ? 0 : P.pb.Ns * P.nh + 3 * Ns + 3;
  const int nparts = s->grid_stage;
  int npf = 0;
  if (P.path == 0) {
    // stage kernel shared memory: table + line buffers + coefficients + staged
    // epilogue operands (as many as keep two CTAs per SM resident, at least y)
    cudaFuncAttributes fa;
    cudaError_t ea = cudaFuncGetAttributes(&fa, k_d8_stage_1v<true, false>);
    if (ea != cudaSuccess) { delete s; return cuda_fail(ea, "cudaFuncGetAttributes"); }
    s->smem_stage = stage_smem_1v(plan, fa.sharedSizeBytes, &npf);
    if (npf < 1) { delete s; set_error("Nx / tile too large for the Dopri8 stage kernel"); return SPX_E_UNSUPPORTED; }
    if (o->persistent && o->saveat == 1 && P.axm.n == P.ax[1].n) {
      // the persistent kernel needs every CTA resident at once (a cooperative launch);
      // it is compiled for the Nx-point product grid only (its register budget)
      int coop = 0, per_sm = 0;
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, plan->device);
      cudaFuncAttributes fp;
      if (cudaFuncGetAttributes(&fp, k_d8_persist) == cudaSuccess &&
          fp.sharedSizeBytes + s->smem_stage <= (size_t)smem_optin() &&
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_d8_persist, plan->threads, s->smem_stage) ==
              cudaSuccess)
        s->persistent = coop && (long long)per_sm * plan->nsm >= s->grid_stage;
      cudaGetLastError();
    }
  } else {
    s->smem_stage = plan->smem_gen;
  }
  // one allocation: st | part | save_ts | masses | energies | Y0 Y1 S0 S1 S3 | done | K[13] | ws | saved
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t vec = al((size_t)len * sizeof(double2));
  size_t off = 0;
  const size_t o_st = off; off += al(sizeof(D8Dev));
  const size_t o_init = off; off += al(sizeof(D8Dev));
  const size_t o_part = off; off += al(2 * (size_t)nparts * sizeof(double));
  const size_t o_ts = off; off += al(std::max(1, o->nsave) * sizeof(double));
  const size_t o_m = off; off += al(SPX_MAX_SPECIES * sizeof(double));
  const size_t o_en = off; off += al(std::max(1, o->nsave) * (size_t)(2 + Ns) * sizeof(double));
  const size_t o_y = off; off += 5 * vec;      // Y0 Y1 S0 S1 S3
  const size_t o_done = off; off += al(sizeof(unsigned int) * (size_t)s->grid_stage);
  const size_t o_k = off; off += 13 * vec;
  const size_t o_ws = off; off += al(plan->ws_bytes);
  const size_t o_sv = off; off += o->save_states ? (size_t)std::max(1, o->nsave) * vec : 0;
  cudaError_t e = cudaMalloc(&s->block, off);
  if (e != cudaSuccess) { d8_free(s); return cuda_fail(e, "cudaMalloc(dopri8)"); }
  char* b = static_cast<char*>(s->block);
  D8Args& A = s->args;
  A.plan = plan->d_plan;
  A.tab = plan->d_tab;
  A.st = reinterpret_cast<D8Dev*>(b + o_st);
  s->d_init = reinterpret_cast<D8Dev*>(b + o_init);
  A.part = reinterpret_cast<double*>(b + o_part);
  A.save_ts = reinterpret_cast<const double*>(b + o_ts);
  A.masses = reinterpret_cast<const double*>(b + o_m);
  A.energies = reinterpret_cast<double*>(b + o_en);
  for (int i = 0; i < 2; ++i) {
    A.Y[i] = reinterpret_cast<double2*>(b + o_y + i * vec);
    A.S[i] = reinterpret_cast<double2*>(b + o_y + (2 + i) * vec);
  }
  A.S3 = reinterpret_cast<double2*>(b + o_y + 4 * vec);
  A.done = reinterpret_cast<unsigned int*>(b + o_done);
  A.K = reinterpret_cast<double2*>(b + o_k);   // stage j at K + j*len
  A.ws = reinterpret_cast<double2*>(b + o_ws);
  A.saved = o->save_states ? reinterpret_cast<double2*>(b + o_sv) : nullptr;
  A.len = len;
  A.npf = npf;
  s->ts.assign(o->save_ts, o->save_ts + o->nsave);
  double masses[SPX_MAX_SPECIES];
  for (int i = 0; i < SPX_MAX_SPECIES; ++i) masses[i] = 1.0;
  if (o->masses)
    for (int i = 0; i < Ns; ++i) masses[i] = o->masses[i];
  D8Dev& I = s->init;
  std::memset(&I, 0, sizeof(I));
  I.t = o->t0; I.t0 = o->t0; I.t1 = o->t1; I.dt = o->dt0;
  I.rtol = o->rtol; I.atol = o->atol; I.adaptive = o->adaptive ? 1 : 0;
  I.max_steps = o->max_steps; I.nsave = o->nsave; I.status = SPX_ST_RUNNING;
  I.interp = o->saveat == 0 ? 1 : 0;
  I.wait_polls = kDefaultWaitPolls;
  if (o->hermitian && P.path == 0 && (P.ax[1].n & 1)) {
    // the streaming and Maxwell terms keep the symmetry only if k(N-1-c) == -k(c) exactly
    const int N = P.ax[1].n;
    bool anti = true;
    for (int c = 0; c < N; ++c)
      if (!(plan->tab[P.ax[1].kofs + c].x == -plan->tab[P.ax[1].kofs + N - 1 - c].x)) anti = false;
    s->herm_allowed = anti;
  }
  e = write_reset_record(s);
  if (e != cudaSuccess) { d8_free(s); return cuda_fail(e, "dopri8 reset record"); }
  e = cudaMallocHost(&s->h_status, sizeof(int) * 4);
  if (e == cudaSuccess && o->nsave > 0)
    e = cudaMemcpy(b + o_ts, o->save_ts, o->nsave * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b + o_m, masses, sizeof(masses), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(b + o_en, 0, std::max(1, o->nsave) * (size_t)(2 + Ns) * sizeof(double));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) { d8_free(s); return cuda_fail(e, "dopri8 set-up"); }
  // capture `attempts_per_graph` step attempts into one graph
  e = cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) { d8_free(s); return cuda_fail(e, "cudaStreamBeginCapture"); }
  if (s->persistent) enqueue_persistent(s, s->cap, s->attempts_per_graph);
  else
    for (int i = 0; i < s->attempts_per_graph; ++i) enqueue_attempt(s, s->cap);
  e = cudaStreamEndCapture(s->cap, &s->graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s->exec, s->graph, 0);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    if (s->persistent) enqueue_persistent(s, s->cap, 1);
    else enqueue_attempt(s, s->cap);
    e = cudaStreamEndCapture(s->cap, &s->graph1);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s->exec1, s->graph1, 0);
  if (e != cudaSuccess) { d8_free(s); return cuda_fail(e, "dopri8 graph"); }
  *out = s;
  return SPX_OK;
}

int spx_dopri8_destroy(spx_dopri8* s) { return d8_free(s); }

int spx_dopri8_set_wait_test(spx_dopri8* s, int32_t polls, int32_t unreachable) {
  if (!s || polls < 0) { set_error("spx_dopri8_set_wait_test: bad argument"); return SPX_E_ARG; }
  const int p = polls == 0 ? kDefaultWaitPolls : polls;
  s->init.wait_polls = unreachable ? -p : p;
  SPX_CUDA(write_reset_record(s));
  return SPX_OK;
}

int spx_dopri8_reset(spx_dopri8* s, const void* y0, void* stream) {
  if (!s || !y0) { set_error("spx_dopri8_reset: null argument"); return SPX_E_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  int hi = 0;
  while (hi < s->nsave && s->ts[hi] <= s->init.t0) ++hi;
  // everything stream-ordered, no host wait: the reset record lives on the device,
  // y0 may be device memory or page-locked host memory
  SPX_CUDA(cudaMemcpyAsync(s->args.st, s->d_init, sizeof(D8Dev), cudaMemcpyDeviceToDevice, st));
  SPX_CUDA(cudaMemcpyAsync(s->args.Y[0], y0, (size_t)s->args.len * sizeof(double2), cudaMemcpyDefault, st));
  SPX_CUDA(cudaMemsetAsync(s->args.done, 0, sizeof(unsigned int) * (size_t)s->grid_stage, st));
  if (s->herm_allowed) {
    const int N = s->plan->host.ax[1].n;
    const long long nlines = s->args.len / N;
    const int grid = (int)std::min<long long>(4LL * s->plan->nsm, (s->args.len + NTHREADS - 1) / NTHREADS);
    k_d8_herm_check<<<grid, NTHREADS, 0, st>>>(s->args.Y[0], nlines, N, &s->args.st->herm);
  }
  if (hi > 0) k_d8_save<<<s->plan->nsm, NTHREADS, 0, st>>>(s->args);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_dopri8_advance(spx_dopri8* s, int64_t max_attempts, void* stream, int32_t* status_out) {
  if (!s) { set_error("spx_dopri8_advance: null solver"); return SPX_E_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  int status = SPX_ST_RUNNING;
  int64_t left = max_attempts;
  while (left > 0) {
    // replay whole graphs of `attempts_per_graph` attempts, then single attempts
    if (left >= s->attempts_per_graph) {
      SPX_CUDA(cudaGraphLaunch(s->exec, st));
      left -= s->attempts_per_graph;
    } else {
      SPX_CUDA(cudaGraphLaunch(s->exec1, st));
      left -= 1;
      if (left > 0) continue;
    }
    SPX_CUDA(cudaMemcpyAsync(s->h_status, &s->args.st->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPX_CUDA(cudaStreamSynchronize(st));
    status = *s->h_status;
    if (status != SPX_ST_RUNNING) break;
  }
  if (status_out) *status_out = status;
  return SPX_OK;
}

int spx_dopri8_enqueue(spx_dopri8* s, int64_t attempts, void* stream) {
  if (!s || attempts < 0) { set_error("spx_dopri8_enqueue: bad argument"); return SPX_E_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  for (int64_t i = 0; i + s->attempts_per_graph <= attempts; i += s->attempts_per_graph)
    SPX_CUDA(cudaGraphLaunch(s->exec, st));
  for (int64_t i = 0; i < attempts % s->attempts_per_graph; ++i) SPX_CUDA(cudaGraphLaunch(s->exec1, st));
  return SPX_OK;
}

int spx_dopri8_run(spx_dopri8* s, void* stream, int32_t* status_out) {
  if (!s) { set_error("spx_dopri8_run: null solver"); return SPX_E_ARG; }
  int32_t status = SPX_ST_RUNNING;
  while (status == SPX_ST_RUNNING) {
    int rc = spx_dopri8_advance(s, 64LL * s->attempts_per_graph, stream, &status);
    if (rc != SPX_OK) return rc;
  }
  if (status_out) *status_out = status;
  return SPX_OK;
}

int spx_dopri8_stats_get(spx_dopri8* s, spx_dopri8_stats* out, void* stream) {
  if (!s || !out) { set_error("spx_dopri8_stats_get: null argument"); return SPX_E_ARG; }
  D8Dev d;
  SPX_CUDA(cudaMemcpyAsync(&d, s->args.st, sizeof(d), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  SPX_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  out->t = d.t; out->dt = d.dt;
  out->accepted = d.accepted; out->rejected = d.rejected; out->rhs_evals = d.evals;
  out->status = d.status; out->saved = d.saved;
  out->hermitian = d.herm; out->persistent = s->persistent ? 1 : 0;
  return SPX_OK;
}

const void* spx_dopri8_state(spx_dopri8* s) {
  if (!s) return nullptr;
  D8Dev d;
  if (cudaMemcpy(&d, s->args.st, sizeof(d), cudaMemcpyDeviceToHost) != cudaSuccess) return nullptr;
  return s->args.Y[d.cur];
}

const void* spx_dopri8_saved_states(spx_dopri8* s) { return s ? s->args.saved : nullptr; }

const double* spx_dopri8_saved_energies(spx_dopri8* s) { return s ? s->args.energies : nullptr; }

int spx_dopri8_copy(spx_dopri8* s, int32_t what, void* dst, size_t bytes, void* stream) {
  if (!s || !dst) { set_error("spx_dopri8_copy: null argument"); return SPX_E_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t vec = (size_t)s->args.len * sizeof(double2);
  const void* src = nullptr;
  size_t want = 0;
  if (what == 0) {
    if (bytes != vec) { set_error("spx_dopri8_copy: size mismatch"); return SPX_E_ARG; }
    // the address this device dereferences for dst (device memory, or page-locked
    // host memory mapped into the device's address space); NULL otherwise
    cudaPointerAttributes pa;
    void* target = nullptr;
    if (cudaPointerGetAttributes(&pa, dst) == cudaSuccess &&
        (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeHost || pa.type == cudaMemoryTypeManaged))
      target = pa.devicePointer;
    cudaGetLastError();
    if (!target) {
      // pageable host memory: read the buffer index first, then copy
      D8Dev d;
      SPX_CUDA(cudaMemcpyAsync(&d, s->args.st, sizeof(d), cudaMemcpyDeviceToHost, st));
      SPX_CUDA(cudaStreamSynchronize(st));
      SPX_CUDA(cudaMemcpyAsync(dst, s->args.Y[d.cur], vec, cudaMemcpyDefault, st));
      return SPX_OK;
    }
    const int grid = (int)std::min<long long>(4LL * s->plan->nsm, (s->args.len + NTHREADS - 1) / NTHREADS);
    k_d8_export<<<grid, NTHREADS, 0, st>>>(s->args, static_cast<double2*>(target));
    SPX_CUDA(cudaGetLastError());
    return SPX_OK;
  } else if (what == 1) {
    if (!s->args.saved) { set_error("spx_dopri8_copy: states were not kept (save_states = 0)"); return SPX_E_ARG; }
    src = s->args.saved;
    want = (size_t)s->nsave * vec;
  } else if (what == 2) {
    src = s->args.energies;
    want = (size_t)s->nsave * (2 + s->plan->host.pb.Ns) * sizeof(double);
  } else {
    set_error("spx_dopri8_copy: unknown item"); return SPX_E_ARG;
  }
  if (bytes != want) { set_error("spx_dopri8_copy: size mismatch"); return SPX_E_ARG; }
  if (want) SPX_CUDA(cudaMemcpyAsync(dst, src, want, cudaMemcpyDefault, st));
  return SPX_OK;
}

}  // extern "C"
