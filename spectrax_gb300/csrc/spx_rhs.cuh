// spx_rhs.cuh — the fused right-hand-side tile routines (device), shared by the
// plain RHS entry point, the Dopri8 stage kernels and the batched solver.
//
// Each routine computes the derivative of a block of Hermite planes and hands
// every output value to an epilogue functor `epi(flat_index, value)`, so a
// caller can store it (plain RHS), or turn it into a Runge-Kutta stage vector
// plus the next stage input (Dopri8) without another pass over memory.
#pragma once
#include "spx_core.cuh"

namespace spx {

// Global-load policies.  Kernels that only read data written by earlier
// launches use plain loads; a persistent kernel that reads what other CTAs of
// the same launch wrote uses L2-coherent loads (ld.global.cg, no L1/texture).
struct LdPlain {
  __device__ __forceinline__ static double2 ld(const double2* p) { return *p; }
};
struct LdCG {
  __device__ __forceinline__ static double2 ld(const double2* p) { return __ldcg(p); }
};

// Load the plan header and the table into shared memory (whole CTA).
__device__ __forceinline__ void load_plan(DevPlan& sP, double2* stab, const DevPlan* __restrict__ gP,
                                          const double2* __restrict__ gtab) {
  const int* src = reinterpret_cast<const int*>(gP);
  int* dst = reinterpret_cast<int*>(&sP);
  for (int i = threadIdx.x; i < (int)(sizeof(DevPlan) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  for (int i = threadIdx.x; i < sP.tab_len; i += blockDim.x) stab[i] = gtab[i];
  __syncthreads();
}

// ------------------------------------------------------------------------
// Fused 1D1V tile (Ny = Nz = 1, Nm = Np = 1): species s, Hermite planes
// n0 .. n0+nt-1.  With one velocity dimension the nonlinear bracket of
// spectrax/_model.py:168-184,205-209 reduces to
//     sqrt(2n)/a0 * (E_x + u_y B_z - u_z B_y)(x) * C_{n-1}(x),
// so one inverse FFT per plane (C_{n-1}), one for the species field
// combination G, one product and one forward FFT per plane suffice.
//
// JVP = false: the right-hand side at y (yl is ignored).
// JVP = true : the linearisation at y applied to v = yl:
//     L v + N(F_y, C_v) + N(F_v, C_y)   (the bracket is bilinear in (F, C)).
// sA, sB: 2*L*Nx double2 of shared memory with L = nt+1 (RHS) or 2*nt+2 (JVP).
// ------------------------------------------------------------------------
template <bool JVP, class Epi, class LD = LdPlain>
__device__ void rhs1v_tile_t(const DevPlan& P, const double2* __restrict__ tab,
                             const double2* y, const double2* yl,
                             int s, int n0, int nt, double2* sA, double2* sB, double* scoef, Epi& epi) {
  const int N = P.ax[1].n, cut = P.ax[1].cut, Nn = P.pb.Nn;
  const double2* lin = JVP ? yl : y;              // source of the linear terms
  const double2* Cs = y + (size_t)s * Nn * N;
  const double2* Ls = lin + (size_t)s * Nn * N;
  const double2* Fk = y + P.nc;
  const double a0 = P.pb.alpha_s[3 * s];
  const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
  // lines: RHS  [G_y | C_{n-1}(y) x nt]
  //        JVP  [G_y | G_v | C_{n-1}(v) x nt | C_{n-1}(y) x nt]
  const int ng = JVP ? 2 : 1;
  const int nl = JVP ? 2 * nt + 2 : nt + 1;

  if (threadIdx.x < nt) {
    const int n = n0 + threadIdx.x;
    double* c = scoef + 4 * threadIdx.x;
    const double* t = P.coef + ((size_t)s * Nn + n) * COEF_1V;
    c[0] = t[0]; c[1] = t[1]; c[2] = t[2]; c[3] = t[3];
  }
  for (int i = threadIdx.x; i < nl * N; i += blockDim.x) {
    const int l = i / N, c = i - l * N;
    double2 v = make_double2(0.0, 0.0);
    if (kept(c, N, cut)) {
      if (l < ng) {
        const double2* F = (l == 0 ? y : yl) + P.nc;
        v = LD::ld(F + c);
        v = crfma(u1, LD::ld(F + 5 * N + c), v);
        v = crfma(-u2, LD::ld(F + 4 * N + c), v);
      } else {
        const int q = l - ng;                      // 0 .. nt-1 (first set), nt .. 2nt-1 (second)
        const bool second = JVP && q >= nt;
        const int nm1 = n0 + (second ? q - nt : q) - 1;
        const double2* src = (JVP && !second) ? (yl + (size_t)s * Nn * N) : Cs;
        if (nm1 >= 0) v = LD::ld(src + (size_t)nm1 * N + c);
      }
    }
    sA[l * N + std_index(c, N)] = v;
  }
  __syncthreads();
  double2* r = fft_axis_t<true, false>(sA, sB, P.ax[1], tab, Lines{nl, 1, 1, N, 0}, cut);
  double2* o = (r == sA) ? sB : sA;
  // real-space products into the lines right after the G lines
  for (int i = threadIdx.x; i < nt * N; i += blockDim.x) {
    const int x = i % N;
    double2 pr = cmul(r[x], r[ng * N + i]);
    if (JVP) pr = cfma(r[N + x], r[(ng + nt) * N + i], pr);
    r[ng * N + i] = pr;
  }
  __syncthreads();
  double2* f = fft_axis_t<false, true>(r + ng * N, o + ng * N, P.ax[1], tab, Lines{nt, 1, 1, N, 0}, cut);
  const double ua = P.ua[s];
  const double Dd = P.pb.D;
  for (int i = threadIdx.x; i < nt * N; i += blockDim.x) {
    const int l = i / N, c = i - l * N;
    const int n = n0 + l;
    const double* cf = scoef + 4 * l;
    const double2 kt = ktab(P, tab, 1, c);
    const double w = kt.x * a0;
    const double2 C0 = LD::ld(Ls + (size_t)n * N + c);
    const double2 Cp = (n + 1 < Nn) ? LD::ld(Ls + (size_t)(n + 1) * N + c) : make_double2(0.0, 0.0);
    const double2 Cm = (n >= 1) ? LD::ld(Ls + (size_t)(n - 1) * N + c) : make_double2(0.0, 0.0);
    double2 t = cscale(ua, C0);
    t = crfma(cf[0], Cp, t);
    t = crfma(cf[1], Cm, t);
    double d = cf[3];
    if (Dd != 0.0) d = fma(Dd, kt.y * kt.y, d);
    double re = fma(w, t.y, -d * C0.x);
    double im = fma(-w, t.x, -d * C0.y);
    if (n >= 1 && kept(c, N, cut)) {
      const double2 nl2 = f[l * N + std_index(c, N)];
      re = fma(cf[2], nl2.x, re);
      im = fma(cf[2], nl2.y, im);
    }
    epi((size_t)(s * Nn + n) * N + c, make_double2(re, im));
  }
}

template <class Epi>
__device__ __forceinline__ void rhs1v_tile(const DevPlan& P, const double2* __restrict__ tab,
                                           const double2* __restrict__ y, int s, int n0, int nt,
                                           double2* sA, double2* sB, double* scoef, Epi& epi) {
  rhs1v_tile_t<false>(P, tab, y, y, s, n0, nt, sA, sB, scoef, epi);
}

// ------------------------------------------------------------------------
// Fused 1D1V tile over a stage input already staged in shared memory:
//   U  : planes n0-1 .. n0+nt of species s ((nt+2)*N, zero outside [0, Nn))
//   F3 : the field lines E_x, B_z, B_y (3*N), centred order.
// The epilogue functor gets (global index, index within the tile's own planes,
// value); its prepare() runs on every thread before the first call and may
// wait for staged operands (returning false abandons the epilogue).  HERM = false: complex transforms of G and the nt lines C_{n-1}.
// HERM = true (exactly Hermitian state, odd Nx): C(-k) = conj C(k) on every
// line, so G(x) and C_{n-1}(x) are real and two real lines share one complex
// transform: the inverse FFT of X_a + i X_b gives x_a + i x_b, and the forward
// FFT W of p_a + i p_b gives P_a(k) = (W(k) + conj W(-k)) / 2 and
// P_b(k) = -i (W(k) - conj W(-k)) / 2 -- half the transforms.  Only the k <= 0
// half of each output plane is evaluated: the epilogue's
// pair(e, il, e2, il2, v, two) stores v at e and, when two, conj(v) at the
// mirrored entry e2 (its own operands being exactly Hermitian, everything it
// derives from them is too), so the property holds along a Runge-Kutta
// trajectory.
// sA / sB: (nt+1)*N double2 each; scoef: 4*nt doubles.
// ------------------------------------------------------------------------
template <bool HERM, bool MG, class Epi>
__device__ void rhs1v_tile_u(const DevPlan& P, const double2* __restrict__ tab, int s, int n0, int nt,
                             const double2* U, const double2* F3, double2* sA, double2* sB,
                             double* scoef, Epi& epi) {
  const int N = P.ax[1].n, cut = P.ax[1].cut, Nn = P.pb.Nn;
  // MG: products on the grid axm of Lm points (mode k at position k mod Lm);
  // otherwise on the Nx-point grid (positions std_index(c, N)), compiled apart
  const AxisPlan& am = MG ? P.axm : P.ax[1];
  const int Lm = MG ? am.n : N, half = N / 2;
  const size_t sbase = (size_t)s * Nn * N;
  const double a0 = P.pb.alpha_s[3 * s];
  const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
  if (threadIdx.x < nt) {
    const int n = n0 + threadIdx.x;
    double* c = scoef + 4 * threadIdx.x;
    const double* t = P.coef + ((size_t)s * Nn + n) * COEF_1V;
    // HERM: the 1/2 of the packed-spectrum split is folded into the coefficient (exact)
    // rnm = N / Lm turns the 1/N of the table into the product grid's 1/Lm
    c[0] = t[0]; c[1] = t[1]; c[2] = (HERM ? 0.5 * t[2] : t[2]) * (MG ? P.rnm : 1.0); c[3] = t[3];
  }
  // G = E_x + u_y B_z - u_z B_y at centred index c (masked)
  auto G = [&](int c) {
    double2 v = F3[c];
    v = crfma(u1, F3[N + c], v);
    return crfma(-u2, F3[2 * N + c], v);
  };
  const double2 zero = make_double2(0.0, 0.0);
  double2* f;                           // forward transforms of the products
  if (!HERM) {
    // FFT lines: 0 = G, l + 1 = C_{n0+l-1} = U line l (masked, transform order)
    for (int i = threadIdx.x; i < (nt + 1) * Lm; i += blockDim.x) {
      const int l = i / Lm, x = i - l * Lm;
      const int k = x < (Lm + 1) / 2 ? x : x - Lm;
      double2 v = zero;
      if (k >= -cut && k <= cut) v = (l == 0) ? G(k + half) : U[(l - 1) * N + k + half];
      sA[i] = v;
    }
    __syncthreads();
    double2* r = fft_axis_t<true, false>(sA, sB, am, tab, Lines{nt + 1, 1, 1, Lm, 0}, cut);
    double2* o = (r == sA) ? sB : sA;
    for (int i = threadIdx.x; i < nt * Lm; i += blockDim.x) {
      const int x = i % Lm;
      r[Lm + i] = cmul(r[x], r[Lm + i]);
    }
    __syncthreads();
    f = fft_axis_t<false, true>(r + Lm, o + Lm, am, tab, Lines{nt, 1, 1, Lm, 0}, cut);
  } else {
    const int nreal = nt + 1;             // real lines: 0 = G, q + 1 = C_{n0+q-1} = U line q
    const int nin = (nreal + 1) / 2;      // packed inverse transforms
    const int nout = (nt + 1) / 2;        // packed forward transforms
    for (int i = threadIdx.x; i < nin * Lm; i += blockDim.x) {
      const int j = i / Lm, x = i - j * Lm;
      const int k = x < (Lm + 1) / 2 ? x : x - Lm;
      double2 z = zero;
      if (k >= -cut && k <= cut) {
        const int c = k + half;
        const int la = 2 * j, lb = 2 * j + 1;
        const double2 xa = la == 0 ? G(c) : U[(la - 1) * N + c];
        const double2 xb = lb < nreal ? U[(lb - 1) * N + c] : zero;
        z = make_double2(xa.x - xb.y, xa.y + xb.x);
      }
      sA[i] = z;
    }
    __syncthreads();
    double2* r = fft_axis_t<true, false>(sA, sB, am, tab, Lines{nin, 1, 1, Lm, 0}, cut);
    double2* o = (r == sA) ? sB : sA;
    // real-space products p_q = G * C_{n0+q-1}, packed in pairs into o
    for (int i = threadIdx.x; i < nout * Lm; i += blockDim.x) {
      const int j = i / Lm, x = i - j * Lm;
      const double g = r[x].x;
      const int qa = 2 * j, qb = 2 * j + 1;      // real lines qa + 1, qb + 1
      const double2 za = r[((qa + 1) >> 1) * Lm + x];
      const double ca = ((qa + 1) & 1) ? za.y : za.x;
      double cb = 0.0;
      if (qb < nt) {
        const double2 zb = r[((qb + 1) >> 1) * Lm + x];
        cb = ((qb + 1) & 1) ? zb.y : zb.x;
      }
      o[j * Lm + x] = make_double2(g * ca, g * cb);
    }
    __syncthreads();
    f = fft_axis_t<false, true>(o, r, am, tab, Lines{nout, 1, 1, Lm, 0}, cut);
  }
  // the epilogue's own staged operands (called by every thread; false: give up)
  if (!epi.prepare()) return;
  const double ua = P.ua[s];
  const double Dd = P.pb.D;
  // HERM: only the k <= 0 half (c <= centre) is evaluated; the epilogue's
  // pair() also writes the conjugates at the mirrored entries
  const int Nc = HERM ? (N + 1) / 2 : N;
  for (int i = threadIdx.x; i < nt * Nc; i += blockDim.x) {
    const int l = i / Nc, c = i - l * Nc;
    const int n = n0 + l;
    const double* cf = scoef + 4 * l;
    const double2 kt = ktab(P, tab, 1, c);
    const double w = kt.x * a0;
    const double2 Cm = U[l * N + c], C0 = U[(l + 1) * N + c], Cp = U[(l + 2) * N + c];
    double2 t = cscale(ua, C0);
    t = crfma(cf[0], Cp, t);
    t = crfma(cf[1], Cm, t);
    double d = cf[3];
    if (Dd != 0.0) d = fma(Dd, kt.y * kt.y, d);
    double re = fma(w, t.y, -d * C0.x);
    double im = fma(-w, t.x, -d * C0.y);
    if (n >= 1 && kept(c, N, cut)) {
      double2 nl2;
      const int kk = c - half;
      const int px = kk < 0 ? kk + Lm : kk;       // grid position of mode kk
      if (!HERM) {
        nl2 = f[l * Lm + px];
      } else {
        const double2* fl = f + (l >> 1) * Lm;
        const double2 W = fl[px], Wm = fl[kk > 0 ? Lm - kk : -kk];
        if ((l & 1) == 0) nl2 = make_double2(W.x + Wm.x, W.y - Wm.y);
        else nl2 = make_double2(W.y + Wm.y, Wm.x - W.x);
      }
      if (MG && P.alias && (kk == cut || kk == -cut)) {
        // the Nx-point products fold k1 = k2 = -kk (sum -2kk = kk -+ Nx) onto kk:
        // add G_{-kk} C_{-kk}, in the units of the transform output (x Lm, x 2 packed)
        const int cc = half - kk;
        nl2 = cfma(cscale(HERM ? 2.0 * Lm : (double)Lm, G(cc)), U[l * N + cc], nl2);
      }
      re = fma(cf[2], nl2.x, re);
      im = fma(cf[2], nl2.y, im);
    }
    const size_t e = sbase + (size_t)n * N + c;
    if constexpr (!HERM) {
      epi(e, l * N + c, make_double2(re, im));
    } else {
      const int c2 = N - 1 - c;
      epi.pair(e, l * N + c, sbase + (size_t)n * N + c2, l * N + c2, make_double2(re, im), c2 != c);
    }
  }
}

struct SrcPlain {
  const double2* y;
  __device__ __forceinline__ double2 operator()(size_t e) const { return y[e]; }
};

// Field CTA of the staged 1D1V path: C_{s,0}, C_{s,1} and the six field lines
// are gathered through `src` into shared memory F ((2*Ns + 12)*N double2, one
// source read in flight per thread), Maxwell + current as in maxwell_range
// with Ny = Nz = Nm = Np = 1 go to the last 6*N entries of F, and one loop
// hands them to the epilogue (global index, index within the six field lines,
// value), so a heavy epilogue is instantiated once.
template <class Src, class Epi>
__device__ void maxwell1v_g(const DevPlan& P, const double2* __restrict__ tab, const Src& src,
                            double2* F, Epi& epi) {
  const spx_problem& pb = P.pb;
  const int N = P.ax[1].n, Ns = pb.Ns, Nn = pb.Nn;
  const int nent = 2 * Ns + 6;
#pragma unroll 1
  for (int i = threadIdx.x; i < nent * N; i += blockDim.x) {
    const int q = i / N, c = i - q * N;
    double2 v = make_double2(0.0, 0.0);
    if (q < 2 * Ns) {
      const int sp = q >> 1, n = q & 1;
      if (n < Nn) v = src(((size_t)sp * Nn + n) * N + c);
    } else {
      v = src((size_t)P.nc + (size_t)(q - 2 * Ns) * N + c);
    }
    F[i] = v;
  }
  __syncthreads();
  const double2* Fl = F + 2 * Ns * N;
  double2* Fo = F + (2 * Ns + 6) * N;
  const double rs2 = 0.70710678118654752440;
  const double iO = P.iO0;
  const double2 zero = make_double2(0.0, 0.0);
  const double Ky = ktab(P, tab, 0, 0).x, Kz = ktab(P, tab, 2, 0).x;
  for (int pt = threadIdx.x; pt < N; pt += blockDim.x) {
    const double Kx = ktab(P, tab, 1, pt).x;
    double2 J0 = zero, J1 = zero, J2 = zero;
    for (int sp = 0; sp < Ns; ++sp) {
      const double a0 = pb.alpha_s[3 * sp], a1 = pb.alpha_s[3 * sp + 1], a2 = pb.alpha_s[3 * sp + 2];
      const double pre = pb.qs[sp] * a0 * a1 * a2;
      const double2 C000 = F[2 * sp * N + pt], C100 = F[(2 * sp + 1) * N + pt];
      J0 = crfma(pre, crfma(pb.u_s[3 * sp], C000, cscale(a0 * rs2, C100)), J0);
      J1 = crfma(pre, crfma(pb.u_s[3 * sp + 1], C000, cscale(a1 * rs2, zero)), J1);
      J2 = crfma(pre, crfma(pb.u_s[3 * sp + 2], C000, cscale(a2 * rs2, zero)), J2);
    }
    const double2 Ex = Fl[pt], Ey = Fl[N + pt], Ez = Fl[2 * N + pt];
    const double2 Bx = Fl[3 * N + pt], By = Fl[4 * N + pt], Bz = Fl[5 * N + pt];
    const double2 kbx = csub(cscale(Ky, Bz), cscale(Kz, By));
    const double2 kby = csub(cscale(Kz, Bx), cscale(Kx, Bz));
    const double2 kbz = csub(cscale(Kx, By), cscale(Ky, Bx));
    const double2 kex = csub(cscale(Ky, Ez), cscale(Kz, Ey));
    const double2 key = csub(cscale(Kz, Ex), cscale(Kx, Ez));
    const double2 kez = csub(cscale(Kx, Ey), cscale(Ky, Ex));
    Fo[pt] = make_double2(fma(-J0.x, iO, -kbx.y), fma(-J0.y, iO, kbx.x));
    Fo[N + pt] = make_double2(fma(-J1.x, iO, -kby.y), fma(-J1.y, iO, kby.x));
    Fo[2 * N + pt] = make_double2(fma(-J2.x, iO, -kbz.y), fma(-J2.y, iO, kbz.x));
    Fo[3 * N + pt] = make_double2(kex.y, -kex.x);
    Fo[4 * N + pt] = make_double2(key.y, -key.x);
    Fo[5 * N + pt] = make_double2(kez.y, -kez.x);
  }
  __syncthreads();
#pragma unroll 1
  for (int i = threadIdx.x; i < 6 * N; i += blockDim.x) epi((size_t)P.nc + i, i, Fo[i]);
}

// ------------------------------------------------------------------------
// Maxwell + current for Fourier points [p0, p1) of the field planes.
// ------------------------------------------------------------------------
template <class Epi, class LD = LdPlain>
__device__ void maxwell_range(const DevPlan& P, const double2* __restrict__ tab,
                              const double2* y, int p0, int p1, Epi& epi) {
  const spx_problem& pb = P.pb;
  const int Nx = P.ax[1].n, Nz = P.ax[2].n;
  const size_t pl = (size_t)P.plane;
  const double2* F = y + P.nc;
  const double rs2 = 0.70710678118654752440;
  const double iO = P.iO0;
  for (int pt = p0 + threadIdx.x; pt < p1; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    const double Kx = ktab(P, tab, 1, cx).x, Ky = ktab(P, tab, 0, cy).x, Kz = ktab(P, tab, 2, cz).x;
    double2 J0 = make_double2(0, 0), J1 = make_double2(0, 0), J2 = make_double2(0, 0);
    for (int s = 0; s < pb.Ns; ++s) {
      const double a0 = pb.alpha_s[3 * s], a1 = pb.alpha_s[3 * s + 1], a2 = pb.alpha_s[3 * s + 2];
      const double pre = pb.qs[s] * a0 * a1 * a2;
      const size_t b0 = (size_t)s * P.nh * pl + pt;
      const double2 C000 = LD::ld(y + b0);
      const double2 C100 = pb.Nn > 1 ? LD::ld(y + b0 + pl) : make_double2(0, 0);
      const double2 C010 = pb.Nm > 1 ? LD::ld(y + b0 + (size_t)pb.Nn * pl) : make_double2(0, 0);
      const double2 C001 = pb.Np > 1 ? LD::ld(y + b0 + (size_t)pb.Nn * pb.Nm * pl) : make_double2(0, 0);
      J0 = crfma(pre, crfma(pb.u_s[3 * s], C000, cscale(a0 * rs2, C100)), J0);
      J1 = crfma(pre, crfma(pb.u_s[3 * s + 1], C000, cscale(a1 * rs2, C010)), J1);
      J2 = crfma(pre, crfma(pb.u_s[3 * s + 2], C000, cscale(a2 * rs2, C001)), J2);
    }
    const double2 Ex = LD::ld(F + pt), Ey = LD::ld(F + pl + pt), Ez = LD::ld(F + 2 * pl + pt);
    const double2 Bx = LD::ld(F + 3 * pl + pt), By = LD::ld(F + 4 * pl + pt), Bz = LD::ld(F + 5 * pl + pt);
    const double2 kbx = csub(cscale(Ky, Bz), cscale(Kz, By));
    const double2 kby = csub(cscale(Kz, Bx), cscale(Kx, Bz));
    const double2 kbz = csub(cscale(Kx, By), cscale(Ky, Bx));
    const double2 kex = csub(cscale(Ky, Ez), cscale(Kz, Ey));
    const double2 key = csub(cscale(Kz, Ex), cscale(Kx, Ez));
    const double2 kez = csub(cscale(Kx, Ey), cscale(Ky, Ex));
    const size_t f0 = (size_t)P.nc + pt;
    // dE = i K x B - J / Omega_0 ; dB = -i K x E   (spectrax/_simulation.py:103-106)
    epi(f0, make_double2(fma(-J0.x, iO, -kbx.y), fma(-J0.y, iO, kbx.x)));
    epi(f0 + pl, make_double2(fma(-J1.x, iO, -kby.y), fma(-J1.y, iO, kby.x)));
    epi(f0 + 2 * pl, make_double2(fma(-J2.x, iO, -kbz.y), fma(-J2.y, iO, kbz.x)));
    epi(f0 + 3 * pl, make_double2(kex.y, -kex.x));
    epi(f0 + 4 * pl, make_double2(key.y, -key.x));
    epi(f0 + 5 * pl, make_double2(kez.y, -kez.x));
  }
}

// ------------------------------------------------------------------------
// General path, pass 1: masked inverse 3-D FFT of one plane into `out`
// (natural real-space order).  Plane ids: [0, Ns*nh) are Hermite planes of y;
// then 3*Ns species field combinations G_s = E + u_s x B, then B (3 planes).
// ------------------------------------------------------------------------
__device__ __forceinline__ double2 field_combo_point(const DevPlan& P, const double2* __restrict__ F,
                                                     int id, size_t pt) {
  const size_t pl = (size_t)P.plane;
  const int Ns = P.pb.Ns;
  if (id >= 3 * Ns) return F[(size_t)(3 + id - 3 * Ns) * pl + pt];
  const int s = id / 3, comp = id % 3;
  const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
  const double2 Bx = F[3 * pl + pt], By = F[4 * pl + pt], Bz = F[5 * pl + pt];
  double2 v = F[(size_t)comp * pl + pt];
  if (comp == 0) { v = crfma(u1, Bz, v); v = crfma(-u2, By, v); }        // E_x + u_y B_z - u_z B_y
  else if (comp == 1) { v = crfma(u2, Bx, v); v = crfma(-u0, Bz, v); }   // E_y + u_z B_x - u_x B_z
  else { v = crfma(u0, By, v); v = crfma(-u1, Bx, v); }                  // E_z + u_x B_y - u_y B_x
  return v;
}

__device__ inline void general_to_real(const DevPlan& P, const double2* __restrict__ tab,
                                const double2* __restrict__ y, int id, double2* __restrict__ out,
                                double2* sA, double2* sB) {
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const int pl = P.plane;
  const int nplanes = P.pb.Ns * P.nh;
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    double2 v = make_double2(0.0, 0.0);
    if (kept(cy, Ny, P.ax[0].cut) && kept(cx, Nx, P.ax[1].cut) && kept(cz, Nz, P.ax[2].cut)) {
      v = (id < nplanes) ? y[(size_t)id * pl + pt] : field_combo_point(P, y + P.nc, id - nplanes, pt);
    }
    const int d = std_index(cy, Ny) * P.prow + std_index(cx, Nx) * Nz + std_index(cz, Nz);
    sA[d] = v;
  }
  __syncthreads();
  double2* r = fft_planes_t<true, false>(sA, sB, P, tab);
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) out[pt] = r[padded(P, pt)];
}

// Per-plane coefficients of the general nonlinear bracket (spectrax/_model.py:168-184).
struct NlCoef {
  double gx, gy, gz;           // sqrt(2n)/a0, sqrt(2m)/a1, sqrt(2p)/a2 on C_{n-1}, C_{m-1}, C_{p-1}
  double bx[3], by[3], bz[3];  // B-bracket weights (0 when the neighbour is outside the box)
  int ix[3], iy[3], iz[3];     // neighbour plane ids (-1 when absent)
  int in_, im_, ip_;           // plane ids of C_{n-1}, C_{m-1}, C_{p-1} (-1 when absent)
};

__host__ __device__ inline NlCoef nl_coef(const DevPlan& P, int s, int n, int m, int p) {
  const spx_problem& pb = P.pb;
  const int Nn = pb.Nn, Nm = pb.Nm, Np = pb.Np;
  const double a0 = pb.alpha_s[3 * s], a1 = pb.alpha_s[3 * s + 1], a2 = pb.alpha_s[3 * s + 2];
  const double sn = sqrt((double)n), sm = sqrt((double)m), sp = sqrt((double)p);
  const double sn1 = sqrt((double)(n + 1)), sm1 = sqrt((double)(m + 1)), sp1 = sqrt((double)(p + 1));
  const double r2 = 1.41421356237309504880;
  const int base = s * P.nh;
  auto id = [&](int nn, int mm, int pp) -> int {
    if (nn < 0 || nn >= Nn || mm < 0 || mm >= Nm || pp < 0 || pp >= Np) return -1;
    return base + (pp * Nm + mm) * Nn + nn;
  };
  NlCoef c;
  c.gx = r2 * sn / a0; c.gy = r2 * sm / a1; c.gz = r2 * sp / a2;
  c.in_ = n >= 1 ? id(n - 1, m, p) : -1;
  c.im_ = m >= 1 ? id(n, m - 1, p) : -1;
  c.ip_ = p >= 1 ? id(n, m, p - 1) : -1;
  // B_x: C_{m-1,p-1}, C_{m-1,p+1}, C_{m+1,p-1}
  c.bx[0] = sm * sp * (a2 / a1 - a1 / a2); c.ix[0] = (m >= 1 && p >= 1) ? id(n, m - 1, p - 1) : -1;
  c.bx[1] = sm * sp1 * (a2 / a1);          c.ix[1] = (m >= 1) ? id(n, m - 1, p + 1) : -1;
  c.bx[2] = -sm1 * sp * (a1 / a2);         c.ix[2] = (p >= 1) ? id(n, m + 1, p - 1) : -1;
  // B_y: C_{n-1,p-1}, C_{n+1,p-1}, C_{n-1,p+1}
  c.by[0] = sn * sp * (a0 / a2 - a2 / a0); c.iy[0] = (n >= 1 && p >= 1) ? id(n - 1, m, p - 1) : -1;
  c.by[1] = sn1 * sp * (a0 / a2);          c.iy[1] = (p >= 1) ? id(n + 1, m, p - 1) : -1;
  c.by[2] = -sn * sp1 * (a2 / a0);         c.iy[2] = (n >= 1) ? id(n - 1, m, p + 1) : -1;
  // B_z: C_{n-1,m-1}, C_{n-1,m+1}, C_{n+1,m-1}
  c.bz[0] = sn * sm * (a1 / a0 - a0 / a1); c.iz[0] = (n >= 1 && m >= 1) ? id(n - 1, m - 1, p) : -1;
  c.bz[1] = sn * sm1 * (a1 / a0);          c.iz[1] = (n >= 1) ? id(n - 1, m + 1, p) : -1;
  c.bz[2] = -sn1 * sm * (a0 / a1);         c.iz[2] = (m >= 1) ? id(n + 1, m - 1, p) : -1;
  for (int k = 0; k < 3; ++k) {
    if (c.ix[k] < 0) c.bx[k] = 0.0;
    if (c.iy[k] < 0) c.by[k] = 0.0;
    if (c.iz[k] < 0) c.bz[k] = 0.0;
  }
  return c;
}

// General path: every constant of one Hermite plane's bracket and linear terms,
// built once on the host (one table entry per (species, mode)) so that no CTA
// spends serial FP64 work on square roots and divisions.
struct GenPlane {
  NlCoef cf;
  // q Omega / N, nu col, sqrt((n+1)/2), sqrt(n/2), sqrt((m+1)/2), sqrt(m/2),
  // sqrt((p+1)/2), sqrt(p/2), u_x/a_x, u_y/a_y, u_z/a_z
  double lin[11];
};

__host__ inline GenPlane gen_plane(const DevPlan& P, int id) {
  const spx_problem& pb = P.pb;
  const int Nn = pb.Nn, Nm = pb.Nm, Np = pb.Np;
  const int s = id / P.nh, h = id % P.nh;
  const int n = h % Nn, m = (h / Nn) % Nm, p = h / (Nn * Nm);
  GenPlane g;
  g.cf = nl_coef(P, s, n, m, p);
  const double rh = 0.5;
  g.lin[0] = pb.qs[s] * pb.Omega_cs[s] / (double)P.plane;
  g.lin[1] = pb.nu * (colc(Nn, n) + colc(Nm, m) + colc(Np, p));
  g.lin[2] = sqrt((n + 1) * rh); g.lin[3] = sqrt(n * rh);
  g.lin[4] = sqrt((m + 1) * rh); g.lin[5] = sqrt(m * rh);
  g.lin[6] = sqrt((p + 1) * rh); g.lin[7] = sqrt(p * rh);
  g.lin[8] = pb.u_s[3 * s] / pb.alpha_s[3 * s];
  g.lin[9] = pb.u_s[3 * s + 1] / pb.alpha_s[3 * s + 1];
  g.lin[10] = pb.u_s[3 * s + 2] / pb.alpha_s[3 * s + 2];
  return g;
}

// Transposed bracket of one Hermite plane q: the (output plane r, field j,
// weight c) of every bracket term of r that reads C_q (field j: 0..2 = the
// species combinations G_x, G_y, G_z, 3..5 = B_x, B_y, B_z).  At most 3 + 9
// entries (one per E term, three per B term).  Stored after the GenPlane table.
constexpr int GENT_MAX = 12;
struct GenPlaneT {
  int cnt;
  int r[GENT_MAX];
  int j[GENT_MAX];
  double c[GENT_MAX];
};

static_assert(sizeof(GenPlane) % alignof(GenPlaneT) == 0, "GenPlaneT entries follow the GenPlane table");

__host__ __device__ inline const GenPlaneT* gen_t(const DevPlan& P) {
  return reinterpret_cast<const GenPlaneT*>(static_cast<const char*>(P.gen) +
                                            (size_t)P.pb.Ns * P.nh * sizeof(GenPlane));
}

// Builds the transposed table from the forward entries (r ascending, so the
// device sums run in a fixed order).  Returns false if a plane has more than
// GENT_MAX entries (cannot happen for the bracket of spectrax/_model.py:168-184).
__host__ inline bool gen_plane_t(const GenPlane* fwd, int nplanes, GenPlaneT* T) {
  for (int q = 0; q < nplanes; ++q) T[q] = GenPlaneT{};
  auto add = [&](int q, int r, int j, double c) {
    if (q < 0) return true;
    GenPlaneT& t = T[q];
    if (t.cnt >= GENT_MAX) return false;
    t.r[t.cnt] = r; t.j[t.cnt] = j; t.c[t.cnt] = c; ++t.cnt;
    return true;
  };
  for (int r = 0; r < nplanes; ++r) {
    const NlCoef& cf = fwd[r].cf;
    bool ok = add(cf.in_, r, 0, cf.gx) && add(cf.im_, r, 1, cf.gy) && add(cf.ip_, r, 2, cf.gz);
    for (int k = 0; k < 3; ++k)
      ok = ok && add(cf.ix[k], r, 3, cf.bx[k]) && add(cf.iy[k], r, 4, cf.by[k]) && add(cf.iz[k], r, 5, cf.bz[k]);
    if (!ok) return false;
  }
  return true;
}

// sum_k w[k] * R[ids[k]][pt] over the present neighbours
__device__ __forceinline__ double2 combo3(const double2* __restrict__ R, size_t pl, const int* ids,
                                          const double* w, size_t pt) {
  double2 t = make_double2(0.0, 0.0);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (ids[k] >= 0) t = crfma(w[k], R[(size_t)ids[k] * pl + pt], t);
  return t;
}

// Real-space bracket at one point for plane coefficients `cf`:
// Gx*gx*C_{n-1} + Gy*gy*C_{m-1} + Gz*gz*C_{p-1} + Bx*(..) + By*(..) + Bz*(..).
struct FieldPlanes {
  const double2 *Gx, *Gy, *Gz, *Bx, *By, *Bz;
};

__device__ __forceinline__ FieldPlanes field_planes(const double2* GB, int s, int Ns, size_t pl) {
  FieldPlanes f;
  f.Gx = GB + (size_t)(3 * s) * pl;
  f.Gy = f.Gx + pl;
  f.Gz = f.Gy + pl;
  f.Bx = GB + (size_t)(3 * Ns) * pl;
  f.By = f.Bx + pl;
  f.Bz = f.By + pl;
  return f;
}

__device__ __forceinline__ double2 bracket_point(const NlCoef& cf, const double2* __restrict__ Cr,
                                                 const FieldPlanes& F, size_t pl, size_t pt,
                                                 bool anyx, bool anyy, bool anyz, double2 acc) {
  if (cf.in_ >= 0) acc = cfma(F.Gx[pt], cscale(cf.gx, Cr[(size_t)cf.in_ * pl + pt]), acc);
  if (cf.im_ >= 0) acc = cfma(F.Gy[pt], cscale(cf.gy, Cr[(size_t)cf.im_ * pl + pt]), acc);
  if (cf.ip_ >= 0) acc = cfma(F.Gz[pt], cscale(cf.gz, Cr[(size_t)cf.ip_ * pl + pt]), acc);
  if (anyx) acc = cfma(F.Bx[pt], combo3(Cr, pl, cf.ix, cf.bx, pt), acc);
  if (anyy) acc = cfma(F.By[pt], combo3(Cr, pl, cf.iy, cf.by, pt), acc);
  if (anyz) acc = cfma(F.Bz[pt], combo3(Cr, pl, cf.iz, cf.bz, pt), acc);
  return acc;
}

// ------------------------------------------------------------------------
// General path, pass 2: real-space bracket of plane `id`, forward FFT, mask,
// plus streaming, collisions and diffusion of `lin`.
//   RHS: bracket(C_y, G_y),           lin = y
//   JVP: bracket(C_v, G_y) + bracket(C_y, G_v), lin = v
// RA/GA: real-space Hermite planes and field combinations of the first
// operand; RB/GB2 of the second (JVP only).
// MODE 0: RHS; 1: JVP (two brackets); 2: linearised JVP, where RB holds the
// six precomputed bracket sums of y for this plane (lin_bracket_sums), so the
// second bracket is six complex products with v's fields GB2.
// MODE 3: VJP (plain transpose J^T w) of Hermite plane `id`: lin = w, RA = the
// planes W_r = (q Omega / N)_r FFT(P_i M w_r) (general_w_real), GA = y's field
// combinations.  The transposed bracket sum_e c_e F_{j_e}(x) W_{r_e}(x) goes
// through the inverse transform (the transpose of the forward one, the DFT
// matrix being symmetric), is masked, and the streaming/collision/diffusion
// terms are the forward formula applied to w (the Hermite streaming matrix is
// symmetric, the rest diagonal); the current's transpose adds the -J/Omega_0
// weights of w_E to the (0,0,0), (1,0,0), (0,1,0), (0,0,1) planes.
// ------------------------------------------------------------------------
template <int MODE, class Epi>
__device__ void general_nl_plane_t(const DevPlan& P, const double2* __restrict__ tab,
                                   const double2* __restrict__ lin,
                                   const double2* __restrict__ RA, const double2* __restrict__ GA,
                                   const double2* __restrict__ RB, const double2* __restrict__ GB2,
                                   int id, double2* sA, double2* sB, Epi& epi) {
  const spx_problem& pb = P.pb;
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const size_t pl = (size_t)P.plane;
  const int Nn = pb.Nn, Nm = pb.Nm, Np = pb.Np, Ns = pb.Ns;
  const int s = id / P.nh, h = id % P.nh;
  const int n = h % Nn, m = (h / Nn) % Nm, p = h / (Nn * Nm);
  // per-plane constants from the host-built table (no square roots or divisions here)
  const GenPlane* gp = static_cast<const GenPlane*>(P.gen) + id;
  const NlCoef cf = gp->cf;
  const double* s_lin = gp->lin;
  const bool anyx = cf.ix[0] >= 0 || cf.ix[1] >= 0 || cf.ix[2] >= 0;
  const bool anyy = cf.iy[0] >= 0 || cf.iy[1] >= 0 || cf.iy[2] >= 0;
  const bool anyz = cf.iz[0] >= 0 || cf.iz[1] >= 0 || cf.iz[2] >= 0;
  // RHS: (RA = C_y, GA = G_y).  JVP: RA = C_v, GA = G_y, RB = C_y (MODE 2: the
  // bracket sums of y), GB2 = G_v.
  const FieldPlanes FA = field_planes(GA, s, Ns, pl);
  FieldPlanes FB;
  if (MODE == 1 || MODE == 2) FB = field_planes(GB2, s, Ns, pl);
  const double2* Sy = (MODE == 2) ? RB + (size_t)id * 6 * pl : nullptr;
  if (MODE == 3) {
    const GenPlaneT* tq = gen_t(P) + id;
    const int ne = tq->cnt;
    for (size_t pt = threadIdx.x; pt < pl; pt += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      for (int e = 0; e < ne; ++e) {
        const int j = tq->j[e];
        const double2* Fj = j < 3 ? FA.Gx + (size_t)j * pl : FA.Bx + (size_t)(j - 3) * pl;
        acc = cfma(Fj[pt], cscale(tq->c[e], RA[(size_t)tq->r[e] * pl + pt]), acc);
      }
      sA[padded(P, (int)pt)] = acc;
    }
  }
  for (size_t pt = threadIdx.x; MODE != 3 && pt < pl; pt += blockDim.x) {
    double2 acc = bracket_point(cf, RA, FA, pl, pt, anyx, anyy, anyz, make_double2(0.0, 0.0));
    if (MODE == 1) acc = bracket_point(cf, RB, FB, pl, pt, anyx, anyy, anyz, acc);
    if (MODE == 2) {
      if (cf.in_ >= 0) acc = cfma(FB.Gx[pt], Sy[pt], acc);
      if (cf.im_ >= 0) acc = cfma(FB.Gy[pt], Sy[pl + pt], acc);
      if (cf.ip_ >= 0) acc = cfma(FB.Gz[pt], Sy[2 * pl + pt], acc);
      if (anyx) acc = cfma(FB.Bx[pt], Sy[3 * pl + pt], acc);
      if (anyy) acc = cfma(FB.By[pt], Sy[4 * pl + pt], acc);
      if (anyz) acc = cfma(FB.Bz[pt], Sy[5 * pl + pt], acc);
    }
    sA[padded(P, (int)pt)] = acc;
  }
  __syncthreads();
  double2* f = fft_planes_t<MODE == 3, true>(sA, sB, P, tab);

  const double a0 = pb.alpha_s[3 * s], a1 = pb.alpha_s[3 * s + 1], a2 = pb.alpha_s[3 * s + 2];
  const double sc = MODE == 3 ? 1.0 : s_lin[0], dcol = s_lin[1];
  // MODE 3: transposed current weights on w_E (spectrax/_model.py:15-72 and
  // dE = -J / Omega_0 of spectrax/_simulation.py:103-106)
  double cjx = 0.0, cjy = 0.0, cjz = 0.0;
  if (MODE == 3) {
    const double w0 = -P.iO0 * pb.qs[s] * a0 * a1 * a2;
    const double rs2 = 0.70710678118654752440;
    if (n == 0 && m == 0 && p == 0) {
      cjx = w0 * pb.u_s[3 * s]; cjy = w0 * pb.u_s[3 * s + 1]; cjz = w0 * pb.u_s[3 * s + 2];
    } else if (n == 1 && m == 0 && p == 0) {
      cjx = w0 * a0 * rs2;
    } else if (n == 0 && m == 1 && p == 0) {
      cjy = w0 * a1 * rs2;
    } else if (n == 0 && m == 0 && p == 1) {
      cjz = w0 * a2 * rs2;
    }
  }
  const bool hasJ = MODE == 3 && (cjx != 0.0 || cjy != 0.0 || cjz != 0.0);
  const double snp = s_lin[2], snm = s_lin[3], smp = s_lin[4], smm = s_lin[5], spp = s_lin[6], spm = s_lin[7];
  const double ux = s_lin[8], uy = s_lin[9], uz = s_lin[10];
  const double2* Cp = lin + (size_t)id * pl;
  const size_t sn_ = pl, sm_ = (size_t)Nn * pl, sp_ = (size_t)Nn * Nm * pl;
  for (size_t pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    const double2 C0 = Cp[pt];
    double re = 0.0, im = 0.0;
    double k2 = 0.0;
    if (Nx > 1) {
      const double2 kt = ktab(P, tab, 1, cx);
      double2 t = cscale(ux, C0);
      if (n + 1 < Nn) t = crfma(snp, Cp[pt + sn_], t);
      if (n >= 1) t = crfma(snm, Cp[pt - sn_], t);
      const double w = kt.x * a0;
      re = fma(w, t.y, re); im = fma(-w, t.x, im);
      k2 = fma(kt.y, kt.y, k2);
    }
    if (Ny > 1) {
      const double2 kt = ktab(P, tab, 0, cy);
      double2 t = cscale(uy, C0);
      if (m + 1 < Nm) t = crfma(smp, Cp[pt + sm_], t);
      if (m >= 1) t = crfma(smm, Cp[pt - sm_], t);
      const double w = kt.x * a1;
      re = fma(w, t.y, re); im = fma(-w, t.x, im);
      k2 = fma(kt.y, kt.y, k2);
    }
    if (Nz > 1) {
      const double2 kt = ktab(P, tab, 2, cz);
      double2 t = cscale(uz, C0);
      if (p + 1 < Np) t = crfma(spp, Cp[pt + sp_], t);
      if (p >= 1) t = crfma(spm, Cp[pt - sp_], t);
      const double w = kt.x * a2;
      re = fma(w, t.y, re); im = fma(-w, t.x, im);
      k2 = fma(kt.y, kt.y, k2);
    }
    const double d = fma(pb.D, k2, dcol);
    re = fma(-d, C0.x, re);
    im = fma(-d, C0.y, im);
    if (kept(cy, Ny, P.ax[0].cut) && kept(cx, Nx, P.ax[1].cut) && kept(cz, Nz, P.ax[2].cut)) {
      const int sidx = std_index(cy, Ny) * P.prow + std_index(cx, Nx) * Nz + std_index(cz, Nz);
      const double2 v = f[sidx];
      re = fma(sc, v.x, re);
      im = fma(sc, v.y, im);
    }
    if (hasJ) {
      const double2* wE = lin + P.nc;
      const double2 ex = wE[pt], ey = wE[pl + pt], ez = wE[2 * pl + pt];
      re = fma(cjx, ex.x, fma(cjy, ey.x, fma(cjz, ez.x, re)));
      im = fma(cjx, ex.y, fma(cjy, ey.y, fma(cjz, ez.y, im)));
    }
    epi((size_t)id * pl + pt, make_double2(re, im));
  }
}

template <class Epi>
__device__ __forceinline__ void general_nl_plane(const DevPlan& P, const double2* __restrict__ tab,
                                                 const double2* __restrict__ y,
                                                 const double2* __restrict__ Creal,
                                                 const double2* __restrict__ GB, int id,
                                                 double2* sA, double2* sB, Epi& epi) {
  general_nl_plane_t<0>(P, tab, y, Creal, GB, nullptr, nullptr, id, sA, sB, epi);
}

// Multi-pass general path (planes larger than one CTA's shared memory): the
// value of output entry pt (centred order) of Hermite plane `id` as in the
// epilogue of general_nl_plane_t (MODE 0), with the forward-transformed bracket
// read from plane `id` of F (global, natural order, standard index per axis).
__device__ inline double2 big_epi_point(const DevPlan& P, const double2* __restrict__ tab,
                                        const double2* __restrict__ y, const double2* __restrict__ F,
                                        int id, size_t pt) {
  const spx_problem& pb = P.pb;
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const size_t pl = (size_t)P.plane;
  const int Nn = pb.Nn, Nm = pb.Nm, Np = pb.Np;
  const int s = id / P.nh, h = id % P.nh;
  const int n = h % Nn, m = (h / Nn) % Nm, p = h / (Nn * Nm);
  const double* L = (static_cast<const GenPlane*>(P.gen) + id)->lin;
  const double a0 = pb.alpha_s[3 * s], a1 = pb.alpha_s[3 * s + 1], a2 = pb.alpha_s[3 * s + 2];
  const double2* Cp = y + (size_t)id * pl;
  const size_t sn_ = pl, sm_ = (size_t)Nn * pl, sp_ = (size_t)Nn * Nm * pl;
  const int cz = (int)(pt % Nz), cx = (int)((pt / Nz) % Nx), cy = (int)(pt / ((size_t)Nz * Nx));
  const double2 C0 = Cp[pt];
  double re = 0.0, im = 0.0, k2 = 0.0;
  if (Nx > 1) {
    const double2 kt = ktab(P, tab, 1, cx);
    double2 t = cscale(L[8], C0);
    if (n + 1 < Nn) t = crfma(L[2], Cp[pt + sn_], t);
    if (n >= 1) t = crfma(L[3], Cp[pt - sn_], t);
    const double w = kt.x * a0;
    re = fma(w, t.y, re); im = fma(-w, t.x, im);
    k2 = fma(kt.y, kt.y, k2);
  }
  if (Ny > 1) {
    const double2 kt = ktab(P, tab, 0, cy);
    double2 t = cscale(L[9], C0);
    if (m + 1 < Nm) t = crfma(L[4], Cp[pt + sm_], t);
    if (m >= 1) t = crfma(L[5], Cp[pt - sm_], t);
    const double w = kt.x * a1;
    re = fma(w, t.y, re); im = fma(-w, t.x, im);
    k2 = fma(kt.y, kt.y, k2);
  }
  if (Nz > 1) {
    const double2 kt = ktab(P, tab, 2, cz);
    double2 t = cscale(L[10], C0);
    if (p + 1 < Np) t = crfma(L[6], Cp[pt + sp_], t);
    if (p >= 1) t = crfma(L[7], Cp[pt - sp_], t);
    const double w = kt.x * a2;
    re = fma(w, t.y, re); im = fma(-w, t.x, im);
    k2 = fma(kt.y, kt.y, k2);
  }
  const double d = fma(pb.D, k2, L[1]);
  re = fma(-d, C0.x, re);
  im = fma(-d, C0.y, im);
  if (kept(cy, Ny, P.ax[0].cut) && kept(cx, Nx, P.ax[1].cut) && kept(cz, Nz, P.ax[2].cut)) {
    const size_t sidx = ((size_t)std_index(cy, Ny) * Nx + std_index(cx, Nx)) * Nz + std_index(cz, Nz);
    const double2 v = F[(size_t)id * pl + sidx];
    re = fma(L[0], v.x, re);
    im = fma(L[0], v.y, im);
  }
  return make_double2(re, im);
}

// The six bracket sums of plane `id` for the real-space planes R of a state y
// (the part of N(F_v, C_y) that does not depend on v): S_0..2 = g_x C_{n-1},
// g_y C_{m-1}, g_z C_{p-1}; S_3..5 = the B_x, B_y, B_z neighbour combinations;
// absent terms are zero.  Written to S (6 planes).
__device__ inline void lin_bracket_sums(const DevPlan& P, const double2* __restrict__ R, int id,
                                        double2* __restrict__ S) {
  const spx_problem& pb = P.pb;
  const size_t pl = (size_t)P.plane;
  const int s = id / P.nh, h = id % P.nh;
  const int n = h % pb.Nn, m = (h / pb.Nn) % pb.Nm, p = h / (pb.Nn * pb.Nm);
  const NlCoef cf = (static_cast<const GenPlane*>(P.gen) + id)->cf;
  const double2 zero = make_double2(0.0, 0.0);
  for (size_t pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    S[pt] = cf.in_ >= 0 ? cscale(cf.gx, R[(size_t)cf.in_ * pl + pt]) : zero;
    S[pl + pt] = cf.im_ >= 0 ? cscale(cf.gy, R[(size_t)cf.im_ * pl + pt]) : zero;
    S[2 * pl + pt] = cf.ip_ >= 0 ? cscale(cf.gz, R[(size_t)cf.ip_ * pl + pt]) : zero;
    S[3 * pl + pt] = combo3(R, pl, cf.ix, cf.bx, pt);
    S[4 * pl + pt] = combo3(R, pl, cf.iy, cf.by, pt);
    S[5 * pl + pt] = combo3(R, pl, cf.iz, cf.bz, pt);
  }
}

// ------------------------------------------------------------------------
// General-path VJP.  The nonlinear term of output plane r is
//   sc_r M P_f FFT( sum_j F_j(x) S_{r,j}(x) ),  S_{r,j} = sum_q c_{r,j,q} IFFT(P_i M C_q),
// F_j the real-space field combinations (G_s = E + u_s x B, then B), so its
// transpose needs, per plane r, W_r = sc_r FFT(P_i M w_r) (the forward DFT
// matrix is symmetric, so the transpose of "mask, shift, forward" applied to
// w_r is "mask, shift, forward" of w_r): general_w_real.
// ------------------------------------------------------------------------
__device__ inline void general_w_real(const DevPlan& P, const double2* __restrict__ tab,
                                      const double2* __restrict__ w, int id, double2* __restrict__ out,
                                      double2* sA, double2* sB) {
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const int pl = P.plane;
  const double sc = (static_cast<const GenPlane*>(P.gen) + id)->lin[0];
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    double2 v = make_double2(0.0, 0.0);
    if (kept(cy, Ny, P.ax[0].cut) && kept(cx, Nx, P.ax[1].cut) && kept(cz, Nz, P.ax[2].cut))
      v = w[(size_t)id * pl + pt];
    sA[std_index(cy, Ny) * P.prow + std_index(cx, Nx) * Nz + std_index(cz, Nz)] = v;
  }
  __syncthreads();
  double2* r = fft_planes_t<false, false>(sA, sB, P, tab);
  for (int pt = threadIdx.x; pt < pl; pt += blockDim.x) out[pt] = cscale(sc, r[padded(P, pt)]);
}

// Field part of the transpose, per species s and bracket component j at
// real-space point pt: R_{s,j} = sum_{r in s} W_r S_{r,j} (j = 0..2: the G_s
// terms; j = 3..5: the species' share of the B terms), here the partial sum
// over the species' planes h in [h0, h1), in plane order.
constexpr int VJP_HCHUNK = 64;   // Hermite planes per partial field sum
__host__ __device__ __forceinline__ int vjp_nchunk(int nh) { return (nh + VJP_HCHUNK - 1) / VJP_HCHUNK; }

__device__ inline double2 vjp_field_sum(const DevPlan& P, const double2* __restrict__ Cr,
                                        const double2* __restrict__ W, size_t pt, int s, int j,
                                        int h0, int h1) {
  const size_t pl = (size_t)P.plane;
  const GenPlane* gp = static_cast<const GenPlane*>(P.gen);
  double2 R = make_double2(0.0, 0.0);
  for (int h = h0; h < h1; ++h) {
    const int r = s * P.nh + h;
    const NlCoef& cf = gp[r].cf;
    double2 t;
    if (j < 3) {
      const int q = j == 0 ? cf.in_ : j == 1 ? cf.im_ : cf.ip_;
      if (q < 0) continue;
      t = cscale(j == 0 ? cf.gx : j == 1 ? cf.gy : cf.gz, Cr[(size_t)q * pl + pt]);
    } else {
      t = j == 3 ? combo3(Cr, pl, cf.ix, cf.bx, pt) : j == 4 ? combo3(Cr, pl, cf.iy, cf.by, pt)
                                                     : combo3(Cr, pl, cf.iz, cf.bz, pt);
    }
    R = cfma(W[(size_t)r * pl + pt], t, R);
  }
  return R;
}

// Real-space gradient of field component c (0..5 = Ex..Bz) at pt from the
// partial sums S (plane (chunk * Ns + s) * 6 + j), chunks added in order:
// g_E = sum_s R_{s,0..2}, g_B = sum_s (R_{s,3..5} + the chain through
// G_s = E + u_s x B).
__device__ __forceinline__ double2 vjp_field_grad(const DevPlan& P, const double2* __restrict__ S, int c,
                                                  size_t pt) {
  const size_t pl = (size_t)P.plane;
  const int Ns = P.pb.Ns, nch = vjp_nchunk(P.nh);
  auto R = [&](int s, int j) {
    double2 v = make_double2(0.0, 0.0);
    for (int k = 0; k < nch; ++k) v = cadd(v, S[((size_t)(k * Ns + s) * 6 + j) * pl + pt]);
    return v;
  };
  double2 g = make_double2(0.0, 0.0);
  for (int s = 0; s < Ns; ++s) {
    g = cadd(g, R(s, c));
    if (c < 3) continue;
    const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
    // G_x = E_x + u_y B_z - u_z B_y, G_y = E_y + u_z B_x - u_x B_z, G_z = E_z + u_x B_y - u_y B_x
    if (c == 3) { g = crfma(u2, R(s, 1), g); g = crfma(-u1, R(s, 2), g); }
    else if (c == 4) { g = crfma(-u2, R(s, 0), g); g = crfma(u0, R(s, 2), g); }
    else { g = crfma(u1, R(s, 0), g); g = crfma(-u0, R(s, 1), g); }
  }
  return g;
}

// Field component c (0..5 = Ex..Bz) of the transpose: the masked inverse
// transform of its real-space gradient (vjp_field_grad of the per-species sums
// S), plus the curl's transpose (dE = i K x B, dB = -i K x E give
// g_E += i K x w_B, g_B += -i K x w_E).
template <class Epi>
__device__ inline void vjp_field_plane(const DevPlan& P, const double2* __restrict__ tab,
                                       const double2* __restrict__ wF, const double2* __restrict__ S,
                                       int c, double2* sA, double2* sB, Epi& epi) {
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const size_t pl = (size_t)P.plane;
  for (size_t pt = threadIdx.x; pt < pl; pt += blockDim.x) sA[padded(P, (int)pt)] = vjp_field_grad(P, S, c, pt);
  __syncthreads();
  double2* f = fft_planes_t<true, true>(sA, sB, P, tab);
  const double2* wO = wF + (size_t)(c < 3 ? 3 : 0) * pl;   // w_B for E, w_E for B
  for (size_t pt = threadIdx.x; pt < pl; pt += blockDim.x) {
    const int cz = pt % Nz, cx = (pt / Nz) % Nx, cy = pt / (Nz * Nx);
    const double Kx = ktab(P, tab, 1, cx).x, Ky = ktab(P, tab, 0, cy).x, Kz = ktab(P, tab, 2, cz).x;
    const double2 o0 = wO[pt], o1 = wO[pl + pt], o2 = wO[2 * pl + pt];
    const int k = c % 3;
    const double2 kx = k == 0 ? csub(cscale(Ky, o2), cscale(Kz, o1))
                     : k == 1 ? csub(cscale(Kz, o0), cscale(Kx, o2))
                              : csub(cscale(Kx, o1), cscale(Ky, o0));
    double2 v = c < 3 ? make_double2(-kx.y, kx.x) : make_double2(kx.y, -kx.x);
    if (kept(cy, Ny, P.ax[0].cut) && kept(cx, Nx, P.ax[1].cut) && kept(cz, Nz, P.ax[2].cut)) {
      const int sidx = std_index(cy, Ny) * P.prow + std_index(cx, Nx) * Nz + std_index(cz, Nz);
      v = cadd(v, f[sidx]);
    }
    epi((size_t)P.nc + (size_t)c * pl + pt, v);
  }
}

// ------------------------------------------------------------------------
// VJP of the fused 1D1V path, pass 1 (planes).  g = J(y)^T w (plain
// transpose).  For output planes m in [m0, m0+nt) of species s:
//   * streaming + damping: the Hermite streaming matrix is symmetric, so its
//     transpose applied to w is the forward formula with C := w;
//   * nonlinear term: NL_n = k_n M P_f FFT(G . IFFT(P_i M C_{n-1})) with
//     k_n = q Omega sqrt(2n) / a0 / N, so its transpose gives
//     g_{n-1} += k_n M P_f IFFT(G . FFT(P_i M w_n))   (FFT directions swapped)
//     and, for the field combination G, the per-species real-space sum
//     R_s(x) = sum_n k_n c_{n-1}(x) W_n(x), written per tile to `part`;
//   * Maxwell: the current J depends on C_{s,0} and C_{s,1}; its transpose adds
//     -(q a0 a1 a2 / Omega_0)(u . w_E) to g_{s,0} and -(q a0^2 a1 a2/(sqrt2 Omega_0)) w_Ex
//     to g_{s,1}.
// sA/sB: 2*(2 nt + 1)*N double2.
// ------------------------------------------------------------------------
__device__ inline void vjp1v_tile(const DevPlan& P, const double2* __restrict__ tab,
                                  const double2* __restrict__ y, const double2* __restrict__ w,
                                  double2* __restrict__ g, double2* __restrict__ part,
                                  int s, int tile, int m0, int nt, double2* sA, double2* sB,
                                  double* scoef, double* pacc = nullptr) {
  const int N = P.ax[1].n, cut = P.ax[1].cut, Nn = P.pb.Nn;
  const double2* __restrict__ Cs = y + (size_t)s * Nn * N;
  const double2* __restrict__ Ws = w + (size_t)s * Nn * N;
  const double2* __restrict__ Fk = y + P.nc;
  const double2* __restrict__ Wf = w + P.nc;
  const double a0 = P.pb.alpha_s[3 * s], a1 = P.pb.alpha_s[3 * s + 1], a2 = P.pb.alpha_s[3 * s + 2];
  const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
  // lines: [G_y | c_m (nt) | W_{m+1} (nt)]
  const int nl = 2 * nt + 1;
  if (threadIdx.x < nt) {
    const int m = m0 + threadIdx.x;
    double* c = scoef + 4 * threadIdx.x;
    const double* t = P.coef + ((size_t)s * Nn + m) * COEF_1V;
    c[0] = t[0]; c[1] = t[1];
    c[2] = (m + 1 < Nn) ? t[COEF_1V + 2] : 0.0;   // k_{m+1}
    c[3] = t[4];
  }
  for (int i = threadIdx.x; i < nl * N; i += blockDim.x) {
    const int l = i / N, c = i - l * N;
    double2 v = make_double2(0.0, 0.0);
    if (kept(c, N, cut)) {
      if (l == 0) {
        v = Fk[c];
        v = crfma(u1, Fk[5 * N + c], v);
        v = crfma(-u2, Fk[4 * N + c], v);
      } else if (l <= nt) {
        v = Cs[(size_t)(m0 + l - 1) * N + c];
      } else {
        const int n = m0 + (l - 1 - nt) + 1;
        if (n < Nn) v = Ws[(size_t)n * N + c];
      }
    }
    sA[l * N + std_index(c, N)] = v;
  }
  __syncthreads();
  // both transforms have the same number of stages, so both results land in `r`
  double2* r = fft_axis_t<true, false>(sA, sB, P.ax[1], tab, Lines{nt + 1, 1, 1, N, 0}, cut);
  double2* o = (r == sA) ? sB : sA;
  {
    double2* r2 = fft_axis_t<false, false>(sA + (nt + 1) * N, sB + (nt + 1) * N, P.ax[1], tab,
                                           Lines{nt, 1, 1, N, 0}, cut);
    (void)r2;
  }
  // partial field sum R_s(x) for this tile (fixed order over planes), then Q = G . W in place
  double2* Rp = part + ((size_t)s * P.ntiles + tile) * N;
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int l = 0; l < nt; ++l) {
      const double k = scoef[4 * l + 2];
      acc = cfma(cscale(k, r[(1 + l) * N + x]), r[(1 + nt + l) * N + x], acc);
    }
    Rp[x] = acc;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nt * N; i += blockDim.x) {
    const int x = i % N;
    r[(1 + nt) * N + i] = cmul(r[x], r[(1 + nt) * N + i]);
  }
  __syncthreads();
  double2* q = fft_axis_t<true, true>(r + (1 + nt) * N, o + (1 + nt) * N, P.ax[1], tab, Lines{nt, 1, 1, N, 0}, cut);
  const double ua = P.ua[s];
  const double Dd = P.pb.D;
  const double iO = P.iO0;
  const double pre = P.pb.qs[s] * a0 * a1 * a2;
  double p_nu = 0.0, p_k = 0.0, p_u = 0.0;     // parameter terms of the own planes (pacc)
  for (int i = threadIdx.x; i < nt * N; i += blockDim.x) {
    const int l = i / N, c = i - l * N;
    const int m = m0 + l;
    const double* cf = scoef + 4 * l;
    const double2 kt = ktab(P, tab, 1, c);
    const double wk = kt.x * a0;
    const double2 W0 = Ws[(size_t)m * N + c];
    const double2 Wp = (m + 1 < Nn) ? Ws[(size_t)(m + 1) * N + c] : make_double2(0.0, 0.0);
    const double2 Wm = (m >= 1) ? Ws[(size_t)(m - 1) * N + c] : make_double2(0.0, 0.0);
    if (pacc) {
      // Re w . df/dtheta at this entry: nu (-col C), k d/dk (streaming), u_x,s (-i K C)
      const double2 C0 = Cs[(size_t)m * N + c];
      const double2 Cp = (m + 1 < Nn) ? Cs[(size_t)(m + 1) * N + c] : make_double2(0.0, 0.0);
      const double2 Cm = (m >= 1) ? Cs[(size_t)(m - 1) * N + c] : make_double2(0.0, 0.0);
      p_nu += -cf[3] * (W0.x * C0.x - W0.y * C0.y);
      double2 tc = cscale(ua, C0);
      tc = crfma(cf[0], Cp, tc);
      tc = crfma(cf[1], Cm, tc);
      p_k += W0.x * (wk * tc.y) - W0.y * (-wk * tc.x);
      p_u += W0.x * (kt.x * C0.y) - W0.y * (-kt.x * C0.x);
    }
    double2 t = cscale(ua, W0);
    t = crfma(cf[0], Wp, t);
    t = crfma(cf[1], Wm, t);
    double d = P.pb.nu * cf[3];
    if (Dd != 0.0) d = fma(Dd, kt.y * kt.y, d);
    double re = fma(wk, t.y, -d * W0.x);
    double im = fma(-wk, t.x, -d * W0.y);
    if (m + 1 < Nn && kept(c, N, cut)) {
      const double2 v = q[l * N + std_index(c, N)];
      re = fma(cf[2], v.x, re);
      im = fma(cf[2], v.y, im);
    }
    if (m == 0) {
      const double2 ex = Wf[c], ey = Wf[N + c], ez = Wf[2 * N + c];
      const double co = -pre * iO;
      re = fma(co, fma(u0, ex.x, fma(u1, ey.x, u2 * ez.x)), re);
      im = fma(co, fma(u0, ex.y, fma(u1, ey.y, u2 * ez.y)), im);
    } else if (m == 1) {
      const double co = -pre * iO * a0 * 0.70710678118654752440;
      re = fma(co, Wf[c].x, re);
      im = fma(co, Wf[c].y, im);
    }
    g[(size_t)(s * Nn + m) * N + c] = make_double2(re, im);
  }
  if (pacc) { pacc[0] += p_nu; pacc[1] += p_k; pacc[2] += p_u; }
}

// VJP tile over operands staged in shared memory (same arithmetic as
// vjp1v_tile):  Uy / Uw: planes m0-1 .. m0+nt of y and w for species s
// ((nt+2)*N each, zero outside [0, Nn)); yF3: y's E_x, B_z, B_y lines; wE: w's
// E_x, E_y, E_z lines (3*N each).  pacc (3 doubles) accumulates the parameter
// terms of the own planes: Re w . (-col C), Re w . f_K, Re w . (-i K C).
// MG: the transposed products on the plan's product grid axm (Lm points, mode k
// at position k mod Lm; sA / sB hold lines of Lm): every factor is masked, so the
// kept modes are the Nx-grid ones times Lm / Nx, undone by rnm = Nx / Lm.  Only
// for plans without the folded term (alias == 0).
template <bool HERM, bool MG = false>
__device__ inline void vjp1v_tile_u(const DevPlan& P, const double2* __restrict__ tab,
                                    const double2* Uy, const double2* Uw, const double2* yF3,
                                    const double2* wE, double2* __restrict__ g,
                                    double2* __restrict__ part, int s, int tile, int m0, int nt,
                                    double2* sA, double2* sB, double* scoef, double* pacc) {
  const int N = P.ax[1].n, cut = P.ax[1].cut, Nn = P.pb.Nn;
  const AxisPlan& am = MG ? P.axm : P.ax[1];
  const int Lm = MG ? am.n : N, half = N / 2;
  const double rn = MG ? P.rnm : 1.0;
  // grid position of the mode at centred index c (std_index(c, N) when Lm == N)
  auto pos = [&](int c) { const int k = c - half; return k < 0 ? k + Lm : k; };
  const double a0 = P.pb.alpha_s[3 * s], a1 = P.pb.alpha_s[3 * s + 1], a2 = P.pb.alpha_s[3 * s + 2];
  const double u0 = P.pb.u_s[3 * s], u1 = P.pb.u_s[3 * s + 1], u2 = P.pb.u_s[3 * s + 2];
  if (threadIdx.x < nt) {
    const int m = m0 + threadIdx.x;
    double* c = scoef + 4 * threadIdx.x;
    const double* t = P.coef + ((size_t)s * Nn + m) * COEF_1V;
    c[0] = t[0]; c[1] = t[1];
    c[2] = (m + 1 < Nn) ? t[COEF_1V + 2] * rn : 0.0;   // k_{m+1} (x rn on the product grid)
    c[3] = t[4];
  }
  // spectrum (masked, centred index c) of line q of [G_y | c_m (nt) | conj W_{m+1} (nt)]
  // (U line l = plane m0-1+l); the inverse transform of conj W is conj(FFT W), so
  // every line goes through one inverse pass
  auto spec = [&](int q, int c) -> double2 {
    if (q == 0) {
      double2 v = yF3[c];
      v = crfma(u1, yF3[N + c], v);
      return crfma(-u2, yF3[2 * N + c], v);
    }
    if (q <= nt) return Uy[(size_t)q * N + c];                     // plane m0 + q - 1
    const double2 wv = Uw[(size_t)(q - nt + 1) * N + c];           // plane m0 + (q - 1 - nt) + 1
    return make_double2(wv.x, -wv.y);
  };
  const double2* q;                     // inverse transforms of the products (and R) by line
  double2* Rp = part + ((size_t)s * P.ntiles + tile) * N;
  if constexpr (!HERM) {
    const int nl = 2 * nt + 1;
    // masked spectra at their grid positions (every position of the Lm-point lines)
    for (int i = threadIdx.x; i < nl * Lm; i += blockDim.x) {
      const int l = i / Lm, x = i - l * Lm;
      const int k = x < (Lm + 1) / 2 ? x : x - Lm;
      sA[i] = (k >= -cut && k <= cut) ? spec(l, k + half) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    double2* r = fft_axis_t<true, false>(sA, sB, am, tab, Lines{nl, 1, 1, Lm, 0}, cut);
    double2* o = (r == sA) ? sB : sA;
    // this tile's share of the field sum R_s(x) = sum_n k_n c_{n-1}(x) W_n(x), as an
    // extra line after the nt product lines: its inverse transform (masked) goes
    // through the same pass, and the tile stores the kept modes as its partial
    for (int x = threadIdx.x; x < Lm; x += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      for (int l = 0; l < nt; ++l) {
        const double k = scoef[4 * l + 2];
        const double2 wt = r[(1 + nt + l) * Lm + x];
        acc = cfma(cscale(k, r[(1 + l) * Lm + x]), make_double2(wt.x, -wt.y), acc);
      }
      r[(1 + 2 * nt) * Lm + x] = acc;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nt * Lm; i += blockDim.x) {
      const int x = i % Lm;
      const double2 wt = r[(1 + nt) * Lm + i];
      r[(1 + nt) * Lm + i] = cmul(r[x], make_double2(wt.x, -wt.y));
    }
    __syncthreads();
    q = fft_axis_t<true, true>(r + (1 + nt) * Lm, o + (1 + nt) * Lm, am, tab, Lines{nt + 1, 1, 1, Lm, 0}, cut);
    for (int c = threadIdx.x; c < N; c += blockDim.x)
      Rp[c] = kept(c, N, cut) ? q[nt * Lm + pos(c)] : make_double2(0.0, 0.0);
  } else {
    // Exactly Hermitian y and w: every real-space line is real, so two lines share
    // one complex transform (inverse of X_a + i X_b is x_a + i x_b).
    const int nreal = 2 * nt + 1, nin = nt + 1;
    for (int i = threadIdx.x; i < nin * Lm; i += blockDim.x) {
      const int j = i / Lm, x = i - j * Lm;
      const int k = x < (Lm + 1) / 2 ? x : x - Lm;
      double2 z = make_double2(0.0, 0.0);
      if (k >= -cut && k <= cut) {
        const int c = k + half;
        const double2 xa = spec(2 * j, c);
        const double2 xb = (2 * j + 1 < nreal) ? spec(2 * j + 1, c) : make_double2(0.0, 0.0);
        z = make_double2(xa.x - xb.y, xa.y + xb.x);
      }
      sA[i] = z;
    }
    __syncthreads();
    double2* r = fft_axis_t<true, false>(sA, sB, am, tab, Lines{nin, 1, 1, Lm, 0}, cut);
    double2* o = (r == sA) ? sB : sA;
    auto rl = [&](int ql, int x) -> double {
      const double2 z = r[(ql >> 1) * Lm + x];
      return (ql & 1) ? z.y : z.x;
    };
    // real lines p_l = G W_l (l < nt) and R = sum_l k_{m0+l+1} c_l W_l, in pairs
    const int nprod = nt + 1, nout = (nprod + 1) / 2;
    for (int i = threadIdx.x; i < nout * Lm; i += blockDim.x) {
      const int j = i / Lm, x = i - j * Lm;
      double pv[2];
#pragma unroll
      for (int h2 = 0; h2 < 2; ++h2) {
        const int l = 2 * j + h2;
        double v = 0.0;
        if (l < nt) {
          v = rl(0, x) * rl(1 + nt + l, x);
        } else if (l == nt) {
          for (int ll = 0; ll < nt; ++ll) v = fma(scoef[4 * ll + 2] * rl(1 + ll, x), rl(1 + nt + ll, x), v);
        }
        pv[h2] = v;
      }
      o[j * Lm + x] = make_double2(pv[0], pv[1]);
    }
    __syncthreads();
    double2* qq = fft_axis_t<true, true>(o, r, am, tab, Lines{nout, 1, 1, Lm, 0}, cut);
    q = qq;
    // R's spectrum: P_b of a pair (nt odd) or P_a (nt even), at every kept mode
    for (int c = threadIdx.x; c < N; c += blockDim.x) {
      double2 v = make_double2(0.0, 0.0);
      if (kept(c, N, cut)) {
        const double2* fl = qq + (nt >> 1) * Lm;
        const double2 W = fl[pos(c)], Wm = fl[pos(N - 1 - c)];
        v = (nt & 1) ? make_double2(0.5 * (W.y + Wm.y), 0.5 * (Wm.x - W.x))
                     : make_double2(0.5 * (W.x + Wm.x), 0.5 * (W.y - Wm.y));
      }
      Rp[c] = v;
    }
  }
  const double ua = P.ua[s];
  const double Dd = P.pb.D;
  const double iO = P.iO0;
  const double pre = P.pb.qs[s] * a0 * a1 * a2;
  double p_nu = 0.0, p_k = 0.0, p_u = 0.0;
  // HERM: only the k <= 0 half; the mirrored entry gets the conjugate and the
  // same parameter contributions
  const int Nc = HERM ? (N + 1) / 2 : N;
  for (int i = threadIdx.x; i < nt * Nc; i += blockDim.x) {
    const int l = i / Nc, c = i - l * Nc;
    const int m = m0 + l;
    const double* cf = scoef + 4 * l;
    const double2 kt = ktab(P, tab, 1, c);
    const double wk = kt.x * a0;
    const double2 Wm = Uw[(size_t)l * N + c], W0 = Uw[(size_t)(l + 1) * N + c], Wp = Uw[(size_t)(l + 2) * N + c];
    const double2 Cm = Uy[(size_t)l * N + c], C0 = Uy[(size_t)(l + 1) * N + c], Cp = Uy[(size_t)(l + 2) * N + c];
    const int c2 = N - 1 - c;
    const double mult = (HERM && c2 != c) ? 2.0 : 1.0;
    double2 tc = cscale(ua, C0);
    tc = crfma(cf[0], Cp, tc);
    tc = crfma(cf[1], Cm, tc);
    p_nu = fma(mult, -cf[3] * (W0.x * C0.x - W0.y * C0.y), p_nu);
    p_k = fma(mult, W0.x * (wk * tc.y) - W0.y * (-wk * tc.x), p_k);
    p_u = fma(mult, W0.x * (kt.x * C0.y) - W0.y * (-kt.x * C0.x), p_u);
    double2 t = cscale(ua, W0);
    t = crfma(cf[0], Wp, t);
    t = crfma(cf[1], Wm, t);
    double d = P.pb.nu * cf[3];
    if (Dd != 0.0) d = fma(Dd, kt.y * kt.y, d);
    double re = fma(wk, t.y, -d * W0.x);
    double im = fma(-wk, t.x, -d * W0.y);
    if (m + 1 < Nn && kept(c, N, cut)) {
      double2 v;
      if constexpr (!HERM) {
        v = q[l * Lm + pos(c)];
      } else {
        const double2* fl = q + (l >> 1) * Lm;
        const double2 W = fl[pos(c)], Wn = fl[pos(c2)];
        v = (l & 1) ? make_double2(0.5 * (W.y + Wn.y), 0.5 * (Wn.x - W.x))
                    : make_double2(0.5 * (W.x + Wn.x), 0.5 * (W.y - Wn.y));
      }
      re = fma(cf[2], v.x, re);
      im = fma(cf[2], v.y, im);
    }
    if (m == 0) {
      const double2 ex = wE[c], ey = wE[N + c], ez = wE[2 * N + c];
      const double co = -pre * iO;
      re = fma(co, fma(u0, ex.x, fma(u1, ey.x, u2 * ez.x)), re);
      im = fma(co, fma(u0, ex.y, fma(u1, ey.y, u2 * ez.y)), im);
    } else if (m == 1) {
      const double co = -pre * iO * a0 * 0.70710678118654752440;
      re = fma(co, wE[c].x, re);
      im = fma(co, wE[c].y, im);
    }
    g[(size_t)(s * Nn + m) * N + c] = make_double2(re, im);
    if (HERM && c2 != c) g[(size_t)(s * Nn + m) * N + c2] = conj_bits(make_double2(re, im));
  }
  pacc[0] += p_nu; pacc[1] += p_k; pacc[2] += p_u;
}

// VJP of the fused 1D1V path, pass 2 (fields): one CTA.
//   g_E = i K x w_B + sum_s gG_s e_x,  g_B = -i K x w_E + sum_s gG_s (0, -u_z, u_y)
// with gG_s = M P_f IFFT(sum_tiles R_s).
__device__ inline void vjp1v_fields(const DevPlan& P, const double2* __restrict__ tab,
                                    const double2* __restrict__ w, double2* __restrict__ g,
                                    const double2* __restrict__ part, double2* sA, double2* sB) {
  const int N = P.ax[1].n, cut = P.ax[1].cut, Ns = P.pb.Ns;
  for (int i = threadIdx.x; i < Ns * N; i += blockDim.x) {
    const int s = i / N, x = i - s * N;
    // eight interleaved partial sums (tiles t = 8q + r, eight loads in flight),
    // combined in a fixed order
    const double2* pt = part + (size_t)s * P.ntiles * N + x;
    double2 a[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) a[r] = make_double2(0.0, 0.0);
    int t = 0;
    for (; t + 8 <= P.ntiles; t += 8) {
      double2 v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = __ldcg(pt + (size_t)(t + r) * N);
#pragma unroll
      for (int r = 0; r < 8; ++r) a[r] = cadd(a[r], v[r]);
    }
    for (int r = 0; t < P.ntiles; ++t, ++r) a[r] = cadd(a[r], __ldcg(pt + (size_t)t * N));
    sA[s * N + x] = cadd(cadd(cadd(a[0], a[1]), cadd(a[2], a[3])), cadd(cadd(a[4], a[5]), cadd(a[6], a[7])));
  }
  __syncthreads();
  double2* r = fft_axis_t<true, true>(sA, sB, P.ax[1], tab, Lines{Ns, 1, 1, N, 0}, cut);
  const double2* Wf = w + P.nc;
  double2* gF = g + P.nc;
  for (int c = threadIdx.x; c < N; c += blockDim.x) {
    double2 gx = make_double2(0, 0), gy = make_double2(0, 0), gz = make_double2(0, 0);
    if (kept(c, N, cut)) {
      for (int s = 0; s < Ns; ++s) {
        const double2 v = r[s * N + std_index(c, N)];
        gx = cadd(gx, v);
        gy = crfma(-P.pb.u_s[3 * s + 2], v, gy);   // d G / d B_y = -u_z
        gz = crfma(P.pb.u_s[3 * s + 1], v, gz);    // d G / d B_z = +u_y
      }
    }
    const double Kx = ktab(P, tab, 1, c).x;   // Ky = Kz = 0 on this path
    const double2 wEy = Wf[N + c], wEz = Wf[2 * N + c];
    const double2 wBy = Wf[4 * N + c], wBz = Wf[5 * N + c];
    // i K x w_B with K = (Kx, 0, 0): (0, -Kx wBz, Kx wBy) * i
    const double2 kbx = make_double2(0, 0);
    const double2 kby = cscale(-Kx, wBz), kbz = cscale(Kx, wBy);
    const double2 kex = make_double2(0, 0);
    const double2 key = cscale(-Kx, wEz), kez = cscale(Kx, wEy);
    gF[c] = make_double2(-kbx.y + gx.x, kbx.x + gx.y);
    gF[N + c] = make_double2(-kby.y, kby.x);
    gF[2 * N + c] = make_double2(-kbz.y, kbz.x);
    gF[3 * N + c] = make_double2(kex.y, -kex.x);
    gF[4 * N + c] = make_double2(key.y + gy.x, -key.x + gy.y);
    gF[5 * N + c] = make_double2(kez.y + gz.x, -kez.x + gz.y);
  }
}

// Field pass of the staged VJP (one CTA): like vjp1v_fields, with partials the
// tiles already transformed (kept modes, centred order) and summed per group of
// 8 tiles, so only the sum over groups is left here.
// Sum of `cnt` partial lines spaced `stride` entries apart, at entry c (eight
// loads in flight, a fixed order).
__device__ __forceinline__ double2 sum_lines8(const double2* __restrict__ p, int cnt, size_t stride) {
  double2 a[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) a[r] = make_double2(0.0, 0.0);
  int t = 0;
  for (; t + 8 <= cnt; t += 8) {
    double2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = __ldcg(p + (size_t)(t + r) * stride);
#pragma unroll
    for (int r = 0; r < 8; ++r) a[r] = cadd(a[r], v[r]);
  }
  for (int r = 0; t < cnt; ++t, ++r) a[r] = cadd(a[r], __ldcg(p + (size_t)t * stride));
  return cadd(cadd(cadd(a[0], a[1]), cadd(a[2], a[3])), cadd(cadd(a[4], a[5]), cadd(a[6], a[7])));
}

__device__ inline void vjp1v_fields_spectral(const DevPlan& P, const double2* __restrict__ tab,
                                             const double2* __restrict__ Wf, double2* __restrict__ gF,
                                             const double2* __restrict__ gpart, int ngroups, double2* sA) {
  const int N = P.ax[1].n, cut = P.ax[1].cut, Ns = P.pb.Ns;
  for (int i = threadIdx.x; i < Ns * N; i += blockDim.x) {
    const int s = i / N, c = i - s * N;
    sA[i] = kept(c, N, cut) ? sum_lines8(gpart + (size_t)s * ngroups * N + c, ngroups, N) : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < N; c += blockDim.x) {
    double2 gx = make_double2(0, 0), gy = make_double2(0, 0), gz = make_double2(0, 0);
    if (kept(c, N, cut)) {
      for (int s = 0; s < Ns; ++s) {
        const double2 v = sA[s * N + c];
        gx = cadd(gx, v);
        gy = crfma(-P.pb.u_s[3 * s + 2], v, gy);   // d G / d B_y = -u_z
        gz = crfma(P.pb.u_s[3 * s + 1], v, gz);    // d G / d B_z = +u_y
      }
    }
    const double Kx = ktab(P, tab, 1, c).x;   // Ky = Kz = 0 on this path
    const double2 wEy = Wf[N + c], wEz = Wf[2 * N + c];
    const double2 wBy = Wf[4 * N + c], wBz = Wf[5 * N + c];
    const double2 kbx = make_double2(0, 0);
    const double2 kby = cscale(-Kx, wBz), kbz = cscale(Kx, wBy);
    const double2 kex = make_double2(0, 0);
    const double2 key = cscale(-Kx, wEz), kez = cscale(Kx, wEy);
    gF[c] = make_double2(-kbx.y + gx.x, kbx.x + gx.y);
    gF[N + c] = make_double2(-kby.y, kby.x);
    gF[2 * N + c] = make_double2(-kbz.y, kbz.x);
    gF[3 * N + c] = make_double2(kex.y, -kex.x);
    gF[4 * N + c] = make_double2(key.y + gy.x, -key.x + gy.y);
    gF[5 * N + c] = make_double2(kez.y + gz.x, -kez.x + gz.y);
  }
}

struct EpiStore {
  double2* __restrict__ dy;
  __device__ __forceinline__ void operator()(size_t e, double2 v) const { dy[e] = v; }
};

}  // namespace spx
