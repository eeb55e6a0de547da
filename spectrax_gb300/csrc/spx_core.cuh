// spx_core.cuh — device-side core of the GB300 Hermite-Fourier right-hand side.
//
// FP64 everywhere.  On GB300 the FP64 pipe (about 2 lane-ops per clock per SM) is
// the binding resource, far below HBM bandwidth, so the code is organised to
// spend as few FP64 instructions as possible and to keep whole warps busy:
//  * FFTs are mixed-radix Stockham transforms in shared memory.  Radix 2/4/8
//    butterflies run in registers; odd radices use a two-phase symmetric direct
//    DFT (pair x_q, x_{R-q} -> a_q = sum, b_q = difference, then
//    X_k = x_0 + sum a_q cos - i sum b_q sin) that needs ~R^2 FP64 ops instead
//    of 4 R^2.
//  * The 1/N of norm="forward", q*Omega_c and the Hermite ladder factors are
//    folded into the final fused multiply-adds of each mode.
//  * Per-plane coefficients are uniform per CTA, so Hermite-boundary cases are
//    uniform branches (no lane divergence).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "../../include/spectrax_gb300.h"

namespace spx {

constexpr int MAXST = 12;      // FFT stages per axis
constexpr int NTHREADS = 256;  // threads per CTA of the 1D1V and helper kernels
// CTA width of the general-path (2-D/3-D plane) kernels: one plane per CTA fills
// most of the shared memory, so one CTA per SM runs and 16 warps hide latency
constexpr int GEN_THREADS = 512;

struct AxisPlan {
  int n;                 // length along the axis (1 = nothing to transform)
  int nst;               // number of Stockham stages
  int cut;               // 2/3 mask: largest |k| kept (-1 = nothing kept)
  int koff;              // k-grid: k_c = 2*pi*(c + koff)   (spectrax/_initialization.py:114-116)
  int radix[MAXST];
  int span[MAXST];       // product of the radices of the earlier stages
  int tw[MAXST];         // offset of the stage twiddles (span*(R-1) entries), -1 when span == 1
  int cs[MAXST];         // offset of the odd-radix table (cos, sin)(2 pi j / R), j < R; -1 if even
  int kofs;              // offset of the per-axis k table: (k_c / L, k_c) pairs, n entries
};

// Programmatic dependent launch: wait until the previous launch in the stream
// has completed and its writes are visible, then let the next launch start its
// own prologue.  Both are no-ops when the launch has no programmatic dependency.
__device__ __forceinline__ void pdl_wait_and_release() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Shared-memory lines (of N double2) after the table on the fused 1D1V path:
// two JVP line buffers of 2T+2 lines, or the gathered field CTA's 2*Ns+6 lines.
__host__ __device__ __forceinline__ int lines_1v(int T, int Ns) {
  return (4 * (T + 1) > 2 * Ns + 6) ? 4 * (T + 1) : 2 * Ns + 6;
}

// Shared memory (double2 entries, after the table) of the staged 1D1V stage
// kernel for tiles of T planes, Nx = N and product grid M: transform lines sA,
// sB ((T+1)*M each), staged planes U ((T+2)*N), field lines F3 (3*N); the field
// CTA reuses the area for its (2*Ns+12)*N gather and output lines.
__host__ __device__ __forceinline__ int stage_area_1v(int T, int Ns, int N, int M) {
  const int a = 2 * (T + 1) * M + (T + 2) * N + 3 * N, b = (2 * Ns + 12) * N;
  return a > b ? a : b;
}

// Everything a kernel needs about one problem; lives in device memory next to
// the double2 table it indexes.
struct DevPlan {
  spx_problem pb;
  AxisPlan ax[3];        // 0: y, 1: x, 2: z (the axis order of the data)
  int plane;             // Ny*Nx*Nz
  int nh;                // Nn*Nm*Np
  long long nc;          // N_C = Ns*nh*plane
  int tab_len;           // double2 entries in the table
  int path;              // 0: fused 1D1V path; 1: general path
  int tile;              // Hermite planes per CTA on the fused path
  int ntiles;            // tiles per species on the fused path
  int prow;              // general path: shared-memory row length (Nx*Nz, odd when Ny > 1)
  int pplane;            // general path: shared-memory plane length Ny*prow
  // fused 1D1V path: per (species, plane) coefficients, COEF_1V doubles each
  // (coef_1v), in device memory; computed once on the host because every
  // square root or division costs ~10 FP64 instructions per thread on the GPU
  const double* coef;
  double ua[SPX_MAX_SPECIES];   // u_x / alpha_x per species
  double iO0;                   // 1 / Omega_c of species 0
  const void* gen;              // general path: per-plane constants (GenPlane[Ns * nh]), device memory
  // Fused 1D1V stepper: the grid of the real-space products G * C_{n-1}.  Both
  // factors are masked to |k| <= K (K = ax[1].cut), so on any grid of M >= 3K+1
  // points the kept output modes come out without wrap-around.  axm is such a
  // grid when one is cheaper to transform than Nx (a copy of ax[1] otherwise);
  // rnm = Nx / M rescales the 1/Nx of coef_1v; alias = 1 when M != Nx and
  // Nx == 3K: the reference's Nx-point products then fold the k = +-2K term
  // C_{+-K} G_{+-K} onto -+K, which the stepper adds back.
  AxisPlan axm;
  double rnm;
  int alias;
};

// Coefficients of Hermite plane n of species s on the fused 1D1V path:
//   [0] sqrt((n+1)/2), [1] sqrt(n/2)          (streaming ladder, spectrax/_model.py:193-204)
//   [2] q Omega_c sqrt(2n) / alpha_x / Nx     (nonlinear term with the 1/N of the forward FFT)
//   [3] nu col(Nn, n), [4] col(Nn, n)         (hypercollisions, spectrax/_initialization.py:121-130)
constexpr int COEF_1V = 5;

// ------------------------------------------------------------------ complex helpers
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
// acc + a*b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
// acc + s*a (s real)
__device__ __forceinline__ double2 crfma(double s, double2 a, double2 acc) {
  return make_double2(fma(s, a.x, acc.x), fma(s, a.y, acc.y));
}
template <bool INV>
__device__ __forceinline__ double2 twiddle(double2 v, double2 w) {
  return INV ? cmulc(v, w) : cmul(v, w);
}
// complex conjugate by flipping the sign bit with an integer instruction (the
// result of -x, bit for bit, without spending an FP64 issue slot)
__device__ __forceinline__ double2 conj_bits(double2 a) {
  return make_double2(a.x, __longlong_as_double(__double_as_longlong(a.y) ^ (long long)0x8000000000000000ULL));
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ double2 rot90(double2 a) {
  return INV ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

// centered (fftshift) index <-> standard FFT index along an axis of length n
__device__ __forceinline__ int std_index(int c, int n) { int k = c - n / 2; return k < 0 ? k + n : k; }

// ------------------------------------------------------------------ line addressing
// nl lines of length n inside one shared buffer: element e of line l sits at
// base(l) + e*es with base(l) = (l / div)*shi + (l % div)*slo.
// Optional: lines l > rk are taken as l + rg (skips a block of rg lines, e.g.
// rows that are all zero or not needed beyond a 2/3 cut); lf = 1 puts the line
// index fastest across threads in the register-radix stages (consecutive
// threads on neighbouring lines: conflict-free shared-memory access when the
// lines are strided or padded rows).  Zero-initialised members change nothing.
struct Lines {
  int nl, es, div, shi, slo;
  int rk, rg, lf;
  __device__ __forceinline__ int base(int l) const {
    if (l > rk) l += rg;
    return (l / div) * shi + (l % div) * slo;
  }
};

// ------------------------------------------------------------------ register butterflies
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
  __device__ __forceinline__ static void run(double2* v) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  }
};
// X1,2 = x0 - (x1+x2)/2 -+ i (sqrt3/2)(x1-x2) (forward; the inverse swaps the signs)
template <bool INV> struct Dft<3, INV> {
  __device__ __forceinline__ static void run(double2* v) {
    const double c = INV ? -0.86602540378443864676 : 0.86602540378443864676;
    const double2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
    const double2 m = make_double2(fma(-0.5, t1.x, v[0].x), fma(-0.5, t1.y, v[0].y));
    v[0] = cadd(v[0], t1);
    v[1] = make_double2(fma(c, t2.y, m.x), fma(-c, t2.x, m.y));
    v[2] = make_double2(fma(-c, t2.y, m.x), fma(c, t2.x, m.y));
  }
};
template <bool INV> struct Dft<4, INV> {
  __device__ __forceinline__ static void run(double2* v) {
    double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    double2 s13 = cadd(v[1], v[3]), d13 = rot90<INV>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13); v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13); v[3] = csub(d02, d13);
  }
};
template <bool INV> struct Dft<8, INV> {
  __device__ __forceinline__ static void run(double2* v) {
    const double h = 0.70710678118654752440;   // 1/sqrt(2)
    double2 e[4] = {v[0], v[2], v[4], v[6]};
    double2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    // o[k] *= w8^k,  w8 = exp(-+ i pi/4)
    double2 o1, o3;
    if (!INV) {
      o1 = make_double2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
      o3 = make_double2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
    } else {
      o1 = make_double2(h * (o[1].x - o[1].y), h * (o[1].x + o[1].y));
      o3 = make_double2(-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y));
    }
    double2 o2 = rot90<INV>(o[2]);
    v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);   v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);   v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);   v[7] = csub(e[3], o3);
  }
};

// Largest pair index q of butterfly j whose inputs (first decimation-in-time
// stage) or outputs (last decimation-in-frequency stage) can be non-zero /
// are needed, when only standard indices <= cut or >= n - cut matter.
__device__ __forceinline__ int pair_limit(int j, int M, int h, int cut) {
  const int q = (cut + j) / M;
  return q < h ? q : h;
}

// ---- decimation in time (Stockham): gather stride M, twiddle, DFT, scatter
// to (j/Ns)*Ns*R + k + r*Ns.
template <int R, bool INV>
__device__ __forceinline__ void stage_reg_dit(const double2* __restrict__ in, double2* __restrict__ out,
                                              int n, int Ns, const double2* __restrict__ tw, const Lines& L) {
  const int M = n / R;
  const int ntask = L.nl * M;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int l = L.lf ? t % L.nl : t / M;
    const int j = L.lf ? t / L.nl : t - l * M;
    const int b = L.base(l);
    const int k = j % Ns;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[b + (j + r * M) * L.es];
    if (Ns > 1 && k > 0) {
      const double2* w = tw + k * (R - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = twiddle<INV>(v[r], w[r - 1]);
    }
    Dft<R, INV>::run(v);
    const int idx = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[b + (idx + r * Ns) * L.es] = v[r];
  }
}

// ---- decimation in frequency: the transpose of the stage above (gather from
// the DIT output positions, DFT, twiddle the outputs, scatter with stride M).
template <int R, bool INV>
__device__ __forceinline__ void stage_reg_dif(const double2* __restrict__ in, double2* __restrict__ out,
                                              int n, int Ns, const double2* __restrict__ tw, const Lines& L) {
  const int M = n / R;
  const int ntask = L.nl * M;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int l = L.lf ? t % L.nl : t / M;
    const int j = L.lf ? t / L.nl : t - l * M;
    const int b = L.base(l);
    const int k = j % Ns;
    const int idx = (j / Ns) * Ns * R + k;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[b + (idx + r * Ns) * L.es];
    Dft<R, INV>::run(v);
    if (Ns > 1 && k > 0) {
      const double2* w = tw + k * (R - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = twiddle<INV>(v[r], w[r - 1]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) out[b + (j + r * M) * L.es] = v[r];
  }
}

// Odd radix R (any R >= 3), two phases.  Phase 1, in place on `in`: replace
// each pair (x_q, x_{R-q}) by (x_q + x_{R-q}, x_q - x_{R-q}) (with the
// decimation-in-time twiddles applied first).  Phase 2: one task per output
// pair (kk, R-kk): X = x_0 + sum_q a_q cos -+ i sum_q b_q sin.
// DIF = false: gather stride M, scatter to the DIT positions; `pcut` >= 0 on
//              the first stage skips input pairs that are zero.
// DIF = true : gather from the DIT positions, twiddle the outputs, scatter
//              with stride M; `pcut` >= 0 on the last stage skips output pairs
//              that are not needed.
template <bool INV, bool DIF>
__device__ __forceinline__ void stage_odd(double2* __restrict__ in, double2* __restrict__ out, int n,
                                          int R, int Ns, const double2* __restrict__ tw,
                                          const double2* __restrict__ cs, const Lines& L, int pcut) {
  const int M = n / R;
  const int h = (R - 1) >> 1;
  {
    const int ntask = L.nl * M * h;
    for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
      const int q = t % h + 1;
      const int lj = t / h;
      const int l = lj / M, j = lj - l * M;
      if (!DIF && pcut >= 0 && q > pair_limit(j, M, h, pcut)) continue;
      const int b = L.base(l);
      const int k = j % Ns;
      int i1, i2;
      if (!DIF) {
        i1 = b + (j + q * M) * L.es;
        i2 = b + (j + (R - q) * M) * L.es;
      } else {
        const int idx = (j / Ns) * Ns * R + k;
        i1 = b + (idx + q * Ns) * L.es;
        i2 = b + (idx + (R - q) * Ns) * L.es;
      }
      double2 x1 = in[i1], x2 = in[i2];
      if (!DIF && Ns > 1 && k > 0) {
        const double2* w = tw + k * (R - 1);
        x1 = twiddle<INV>(x1, w[q - 1]);
        x2 = twiddle<INV>(x2, w[R - q - 1]);
      }
      in[i1] = cadd(x1, x2);
      in[i2] = csub(x1, x2);
    }
  }
  __syncthreads();
  {
    // task list: per butterfly j the output pairs kk = 0 .. kmax(j), two pairs
    // (kk, kk + 1) per task so that a_q / b_q loads are shared and each thread
    // runs eight independent FMA chains.
    const bool prune_out = DIF && pcut >= 0;
    int per_line = M * ((h + 2) >> 1);
    if (prune_out) {
      per_line = 0;
      for (int j = 0; j < M; ++j) per_line += (pair_limit(j, M, h, pcut) + 2) >> 1;
    }
    const int ntask = L.nl * per_line;
    // Work goes out per warp: full warps take 32 tasks, one lane each; the
    // remainder (rem < 32 tasks) shares one warp, each task's sum over q split
    // over G lanes (G a power of two, G * rem <= 32) and reduced by shuffles, so
    // that a nearly empty warp does not cost a full task loop.  FP64 issue is
    // per warp instruction, whatever the number of active lanes.
    // Alternatively, when the task list fits the CTA at least twice over, every
    // task is split over GA lanes (the largest power of two <= 8 that still
    // fits): a warp issues at most one FP64 instruction per ~68 cycles, so
    // shorter loops on more warps shorten the phase.  Chosen by measurement
    // over the tile shapes the autotuner tries.
    const int nfw = ntask >> 5;
    const int rem = ntask - (nfw << 5);
    int G = 1;
    if (rem > 0 && rem <= 16) {
      G = 32 / rem;
      while (G & (G - 1)) G &= G - 1;
    }
    int GA = 1;
    while (GA < 8 && ntask * GA * 2 <= (int)blockDim.x) GA *= 2;
    const int units = GA > 1 ? (ntask * GA + 31) >> 5 : nfw + (rem > 0 ? 1 : 0);
    const int lane = threadIdx.x & 31;
    for (int u = threadIdx.x >> 5; u < units; u += blockDim.x >> 5) {
      const bool split = GA == 1 && u == nfw;          // the remainder warp (G lanes per task)
      const int Gu = GA > 1 ? GA : (split ? G : 1);
      const int t = GA > 1 ? ((u << 5) + lane) / GA : (split ? (nfw << 5) + lane / Gu : (u << 5) + lane);
      const int g = GA > 1 ? lane % GA : (split ? lane % Gu : 0);
      const bool active = GA > 1 ? t < ntask : (split ? (lane / Gu) < rem : true);
      double2 A0 = make_double2(0.0, 0.0), A1 = A0, B0 = A0, B1 = A0;
      int l = 0, j = 0, kk0 = 0, kk1 = 0;
      bool two = false;
      if (active) {
        l = t / per_line;
        int r = t - l * per_line;
        int kmax;
        if (!prune_out) {
          const int pj = (h + 2) >> 1;
          j = r / pj;
          r -= j * pj;
          kmax = h;
        } else {
          j = 0;
          kmax = pair_limit(0, M, h, pcut);
          int c = (kmax + 2) >> 1;
          while (r >= c) { r -= c; ++j; kmax = pair_limit(j, M, h, pcut); c = (kmax + 2) >> 1; }
        }
        kk0 = 2 * r;
        two = kk0 + 1 <= kmax;
        kk1 = two ? kk0 + 1 : kk0;
        const int b = L.base(l);
        const int k = j % Ns;
        const int idx = (j / Ns) * Ns * R + k;
        const int qmax = (!DIF && pcut >= 0) ? pair_limit(j, M, h, pcut) : h;
        const int s0 = DIF ? Ns : M;                    // input stride between q's
        const int i0 = DIF ? idx : j;                   // input position of q = 0
        int q0 = 1, q1 = qmax;
        if (Gu > 1) {
          const int seg = (qmax + Gu - 1) / Gu;
          q0 = 1 + g * seg;
          q1 = min(qmax, (g + 1) * seg);
        }
        if (g == 0) { A0 = in[b + i0 * L.es]; A1 = A0; }
        int ang0 = ((q0 - 1) * kk0) % R, ang1 = ((q0 - 1) * kk1) % R;   // (q * kk) mod R
        for (int q = q0; q <= q1; ++q) {
          ang0 += kk0;
          if (ang0 >= R) ang0 -= R;
          ang1 += kk1;
          if (ang1 >= R) ang1 -= R;
          const double2 aq = in[b + (i0 + q * s0) * L.es];
          const double2 bq = in[b + (i0 + (R - q) * s0) * L.es];
          const double2 c0 = cs[ang0], c1 = cs[ang1];
          A0 = crfma(c0.x, aq, A0);
          B0 = crfma(c0.y, bq, B0);
          A1 = crfma(c1.x, aq, A1);
          B1 = crfma(c1.y, bq, B1);
        }
      }
      if (Gu > 1) {
        for (int off = Gu >> 1; off > 0; off >>= 1) {
          A0.x += __shfl_down_sync(0xffffffffu, A0.x, off);
          A0.y += __shfl_down_sync(0xffffffffu, A0.y, off);
          B0.x += __shfl_down_sync(0xffffffffu, B0.x, off);
          B0.y += __shfl_down_sync(0xffffffffu, B0.y, off);
          A1.x += __shfl_down_sync(0xffffffffu, A1.x, off);
          A1.y += __shfl_down_sync(0xffffffffu, A1.y, off);
          B1.x += __shfl_down_sync(0xffffffffu, B1.x, off);
          B1.y += __shfl_down_sync(0xffffffffu, B1.y, off);
        }
      }
      if (!active || g != 0) continue;
      const int b = L.base(l);
      const int k = j % Ns;
      const int idx = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int uu = 0; uu < 2; ++uu) {
        if (uu == 1 && !two) break;
        const int kk = uu ? kk1 : kk0;
        const double2 A = uu ? A1 : A0, B = uu ? B1 : B0;
        // forward: X_kk = A - iB, X_{R-kk} = A + iB ; inverse: signs swapped
        const double2 iB = INV ? make_double2(-B.y, B.x) : make_double2(B.y, -B.x);
        double2 X1 = cadd(A, iB), X2 = csub(A, iB);
        if (!DIF) {
          out[b + (idx + kk * Ns) * L.es] = X1;
          if (kk > 0) out[b + (idx + (R - kk) * Ns) * L.es] = X2;
        } else {
          if (Ns > 1 && k > 0 && kk > 0) {
            const double2* w = tw + k * (R - 1);
            X1 = twiddle<INV>(X1, w[kk - 1]);
            X2 = twiddle<INV>(X2, w[R - kk - 1]);
          }
          out[b + (j + kk * M) * L.es] = X1;
          if (kk > 0) out[b + (j + (R - kk) * M) * L.es] = X2;
        }
      }
    }
  }
}

// Transform all lines along one axis.  DIF = false runs the stages in order
// (decimation in time), DIF = true runs their transposes in reverse order
// (decimation in frequency).  pcut >= 0 prunes the first DIT stage's zero
// inputs or the last DIF stage's unneeded outputs (standard indices beyond
// +-pcut).  Returns the buffer holding the result (a or b).
template <bool INV, bool DIF>
__device__ double2* fft_axis_t(double2* a, double2* b, const AxisPlan& ap, const double2* tab,
                               const Lines& L, int pcut) {
  for (int i = 0; i < ap.nst; ++i) {
    const int st = DIF ? ap.nst - 1 - i : i;
    const int R = ap.radix[st], Ns = ap.span[st];
    const double2* tw = ap.tw[st] >= 0 ? tab + ap.tw[st] : nullptr;
    const int pc = (st == 0) ? pcut : -1;
    switch (R) {
      case 2: DIF ? stage_reg_dif<2, INV>(a, b, ap.n, Ns, tw, L) : stage_reg_dit<2, INV>(a, b, ap.n, Ns, tw, L); break;
      case 3: DIF ? stage_reg_dif<3, INV>(a, b, ap.n, Ns, tw, L) : stage_reg_dit<3, INV>(a, b, ap.n, Ns, tw, L); break;
      case 4: DIF ? stage_reg_dif<4, INV>(a, b, ap.n, Ns, tw, L) : stage_reg_dit<4, INV>(a, b, ap.n, Ns, tw, L); break;
      case 8: DIF ? stage_reg_dif<8, INV>(a, b, ap.n, Ns, tw, L) : stage_reg_dit<8, INV>(a, b, ap.n, Ns, tw, L); break;
      default: stage_odd<INV, DIF>(a, b, ap.n, R, Ns, tw, tab + ap.cs[st], L, pc); break;
    }
    __syncthreads();
    double2* t = a; a = b; b = t;
  }
  return a;
}

// Unpruned decimation-in-time transform (kept for callers without a mask).
template <bool INV>
__device__ __forceinline__ double2* fft_axis(double2* a, double2* b, const AxisPlan& ap, const double2* tab,
                                             const Lines& L) {
  return fft_axis_t<INV, false>(a, b, ap, tab, L, -1);
}

// 3-D transform of one plane of shape (Ny, Nx, Nz) held in buffer a with rows
// of P.prow entries (element (y, x, z) at y*prow + x*Nz + z; prow is Nx*Nz
// rounded up to an odd count when Ny > 1, so neighbouring rows fall in different
// shared-memory banks); b is the ping-pong partner.  DIF = false: masked input
// (zero beyond each axis' cut), DIF = true: only the masked outputs are needed.
// On 2-D planes (Nz = 1) the inverse skips the x-lines of rows beyond the y cut
// (all zero) and the forward skips the y-lines of columns beyond the x cut (never
// read).  Returns the result buffer.
__device__ __forceinline__ bool prunable(const AxisPlan& ap) { return ap.cut >= 0 && 2 * ap.cut + 1 < ap.n; }

template <bool INV, bool DIF>
__device__ double2* fft_planes_t(double2* a, double2* b, const DevPlan& P, const double2* tab) {
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const int R = P.prow;
  if (Nz > 1) {   // z-lines, l = y*Nx + x, base = y*prow + x*Nz
    Lines L{Ny * Nx, 1, Nx, R, Nz};
    double2* r = fft_axis_t<INV, DIF>(a, b, P.ax[2], tab, L, P.ax[2].cut);
    if (r != a) { b = a; a = r; }
  }
  if (Nx > 1) {   // x-lines, l = y*Nz + z, base = y*prow + z
    Lines L{Ny * Nz, Nz, Nz, R, 1};
    L.lf = 1;
    if (!DIF && Nz == 1 && Ny > 1 && prunable(P.ax[0])) {
      const int cy = P.ax[0].cut;
      L.nl = 2 * cy + 1;
      L.rk = cy;
      L.rg = Ny - L.nl;
      if (P.ax[1].nst & 1) {
        // the result lands in b: its skipped rows must read as zero
        for (int i = threadIdx.x; i < L.rg * Nx; i += blockDim.x) {
          const int y = cy + 1 + i / Nx;
          b[y * R + i % Nx] = make_double2(0.0, 0.0);
        }
      }
    }
    double2* r = fft_axis_t<INV, DIF>(a, b, P.ax[1], tab, L, P.ax[1].cut);
    if (r != a) { b = a; a = r; }
  }
  if (Ny > 1) {   // y-lines, l = x*Nz + z, base = l, stride prow
    Lines L{Nx * Nz, R, Nx * Nz, 0, 1};
    L.lf = 1;
    if (DIF && Nz == 1 && Nx > 1 && prunable(P.ax[1])) {
      const int cx = P.ax[1].cut;
      L.nl = 2 * cx + 1;
      L.rk = cx;
      L.rg = Nx - L.nl;
    }
    double2* r = fft_axis_t<INV, DIF>(a, b, P.ax[0], tab, L, P.ax[0].cut);
    if (r != a) { b = a; a = r; }
  }
  return a;
}

// Shared-memory position of plane entry pt = (y*Nx + x)*Nz + z (padded rows).
__device__ __forceinline__ int padded(const DevPlan& P, int pt) {
  const int row = P.ax[1].n * P.ax[2].n;
  return (pt / row) * P.prow + pt % row;
}

// k-table entry (k_c / L, k_c) of axis `ax` at centered index c.
__device__ __forceinline__ double2 ktab(const DevPlan& P, const double2* tab, int ax, int c) {
  return tab[P.ax[ax].kofs + c];
}

__device__ __forceinline__ bool kept(int c, int n, int cut) {
  int k = c - n / 2;
  k = k < 0 ? -k : k;
  return k <= cut;
}

// hypercollision coefficient c(N, i); spectrax/_initialization.py:125-129
__host__ __device__ __forceinline__ double colc(int N, int i) {
  if (N <= 3) return 0.0;
  return (double)i * (double)(i - 1) * (double)(i - 2) / ((double)(N - 1) * (double)(N - 2) * (double)(N - 3));
}

__host__ inline void coef_1v(const spx_problem& pb, int s, int n, double* c) {
  const double qOc = pb.qs[s] * pb.Omega_cs[s];
  const double a0 = pb.alpha_s[3 * s];
  c[0] = sqrt((double)(n + 1) * 0.5);
  c[1] = sqrt((double)n * 0.5);
  c[2] = qOc * sqrt(2.0 * (double)n) / a0 / (double)pb.Nx;
  c[3] = pb.nu * colc(pb.Nn, n);
  c[4] = colc(pb.Nn, n);
}

}  // namespace spx
