// spx_rhs.cu — plan construction, right-hand-side kernels and their C ABI:
//  * plans: FFT tables, the 1D1V coefficient table and product grid, the
//    general layout's per-plane tables (GenPlane, GenPlaneT);
//  * spx_rhs / spx_jvp / spx_linearize / spx_jvp_lin on the fused 1D1V path
//    (one launch) and the general path (plane transforms in shared memory, or
//    the multi-pass kernels k_big_* for planes larger than a CTA's shared memory);
//  * spx_vjp: the transposes of both paths (k_vjp1v*, k_vjp_real/_fsum/_gen).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "spx_plan.h"
#include "spx_rhs.cuh"

namespace spx {

static thread_local std::string g_last_error = "no error";

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return SPX_E_CUDA;
}

// cos/sin(2*pi*p/q) with the angle reduced to |angle| <= pi/4 by exact quarter turns.
static void sincos2pi(long long p, long long q, double* c, double* s) {
  p %= q;
  if (p < 0) p += q;
  const long long m = (4 * p + q / 2) / q;         // nearest quarter turn
  const long long num = 4 * p - m * q;             // remainder in units of 1/(4q) turns
  const double ang = (2.0 * M_PI) * ((double)num / (double)(4 * q));
  double cc = std::cos(ang), ss = std::sin(ang);
  switch (m & 3) {
    case 0: *c = cc; *s = ss; break;
    case 1: *c = -ss; *s = cc; break;
    case 2: *c = -cc; *s = -ss; break;
    default: *c = ss; *s = -cc; break;
  }
}

static std::vector<int> factorize(int n) {
  std::vector<int> r;
  int m = n;
  while (m % 8 == 0) { r.push_back(8); m /= 8; }
  while (m % 4 == 0) { r.push_back(4); m /= 4; }
  while (m % 2 == 0) { r.push_back(2); m /= 2; }
  for (int p = 3; m > 1; p += 2)
    while (m % p == 0) { r.push_back(p); m /= p; }
  std::sort(r.begin(), r.end(), [](int a, int b) { return a > b; });
  return r;
}

// rads: the Stockham radices in stage order (default: factorize(n)); ktable:
// append the axis' k table (not needed by a transform-only axis).
static int build_axis(int n, int cut, double L, std::vector<double2>& tab, AxisPlan& ap,
                      const std::vector<int>* rads = nullptr, bool ktable = true) {
  std::memset(&ap, 0, sizeof(ap));
  ap.n = n;
  ap.cut = cut;
  const int fl = -((n + 1) / 2);     // floor(-n/2)
  ap.koff = fl + 1;
  ap.kofs = (int)tab.size();
  for (int c = 0; ktable && c < n; ++c) {
    const double k = (double)(2 * (c + ap.koff)) * M_PI;
    tab.push_back(make_double2(k / L, k));
  }
  if (n == 1) { ap.nst = 0; return SPX_OK; }
  std::vector<int> rad = rads ? *rads : factorize(n);
  if ((int)rad.size() > MAXST) { set_error("FFT length has too many factors"); return SPX_E_UNSUPPORTED; }
  ap.nst = (int)rad.size();
  std::map<int, int> cs_of;
  int Ns = 1;
  for (int st = 0; st < ap.nst; ++st) {
    const int R = rad[st];
    ap.radix[st] = R;
    ap.span[st] = Ns;
    ap.tw[st] = -1;
    ap.cs[st] = -1;
    if (Ns > 1) {
      ap.tw[st] = (int)tab.size();
      for (int k = 0; k < Ns; ++k)
        for (int r = 1; r < R; ++r) {
          double c, s;
          sincos2pi(-(long long)r * k, (long long)Ns * R, &c, &s);   // exp(-2 pi i r k / (Ns R))
          tab.push_back(make_double2(c, s));
        }
    }
    if (R % 2 == 1) {
      auto it = cs_of.find(R);
      if (it == cs_of.end()) {
        cs_of[R] = (int)tab.size();
        for (int j = 0; j < R; ++j) {
          double c, s;
          sincos2pi(j, R, &c, &s);
          tab.push_back(make_double2(c, s));
        }
      }
      ap.cs[st] = cs_of[R];
    }
    Ns *= R;
  }
  return SPX_OK;
}

// FP64 instructions of one masked inverse (input-pruned) plus one forward
// (output-pruned) transform of a line of length n with radices `rads`: the
// count the Stockham stages of spx_core.cuh issue (twiddles, register
// butterflies for 2/3/4/8, the two-phase symmetric DFT for other odd radices,
// pruned at the stage next to the masked side).
static double line_pair_cost(int n, const std::vector<int>& rads, int cut) {
  double total = 0.0;
  for (int dif = 0; dif < 2; ++dif) {
    int Ns = 1;
    for (size_t si = 0; si < rads.size(); ++si) {
      const int R = rads[si], M = n / R;
      const double tw_tasks = Ns > 1 ? (double)(M - M / Ns) : 0.0;
      if (R == 2 || R == 3 || R == 4 || R == 8) {
        total += tw_tasks * 4.0 * (R - 1);
        total += (double)M * (R == 2 ? 4 : R == 3 ? 12 : R == 4 ? 16 : 56);
      } else {
        const int h = (R - 1) / 2;
        total += tw_tasks * h * 8.0;
        double pairs = 0.0, outs = 0.0;
        for (int j = 0; j < M; ++j) {
          const int q = si == 0 ? std::min(h, (cut + j) / M) : h;
          if (!dif) { pairs += q; outs += (4.0 * q + 4.0) * (h + 1); }
          else { pairs += h; outs += (4.0 * h + 4.0) * (q + 1); }
        }
        total += 4.0 * pairs + outs;
      }
      Ns *= R;
    }
  }
  return total;
}

// Radix orders tried for a product-grid length m: the default factorisation,
// and with two factors 3 merged into one odd radix 9 placed first (fewer
// stages; the first stage is the one the mask prunes).
static std::vector<std::vector<int>> radix_orders(int m) {
  std::vector<std::vector<int>> out{factorize(m)};
  std::vector<int> f = factorize(m);
  int threes = (int)std::count(f.begin(), f.end(), 3);
  if (threes >= 2) {
    std::vector<int> g{9};
    int skip = 2;
    for (int r : f) {
      if (r == 3 && skip > 0) { --skip; continue; }
      g.push_back(r);
    }
    out.push_back(g);
  }
  if (m == 16) out.push_back({4, 4});
  return out;
}

// 0: a register-radix grid where Nx needs odd two-phase stages; 1: always Nx;
// 2: the cheapest grid by FP64 count at <= 0.8x without an extra stage
static int g_product_grid = 0;

// Modeled cost of one transform of m points through register butterflies of
// radices 4, 3, 2 in the order `rads`: FP64 instructions per point of each stage
// (radix 4: 16 per butterfly + 12 for twiddles, radix 3: 12 + 8, radix 2: 4 + 4;
// the first stage has no twiddles) plus kStageCost per Stockham stage (a barrier
// and a pass through shared memory).  Fitted to the two-stream stage kernel
// (Nx = 129 planes, tiles of 6 planes): 144 = 4*4*3*3 ran 0.311 ms per Dopri8
// attempt, 192 = 4*4*4*3 0.337, 162 = 3^4*2 0.344, 256 = 4^4 0.375, against
// 0.382 for 43*3 (two-phase radix 43); per-stage cost about 480 FP64
// instructions, chains with radix 8 or a leading 2 slower than the count.
static double register_chain_cost(int m, const std::vector<int>& rads) {
  constexpr double kStageCost = 480.0;
  double c = 0.0;
  for (size_t i = 0; i < rads.size(); ++i) {
    const int R = rads[i];
    const double bf = (R == 4 ? 16.0 : R == 3 ? 12.0 : 4.0) + (i > 0 ? (R == 4 ? 12.0 : R == 3 ? 8.0 : 4.0) : 0.0);
    c += (double)m / R * bf + kStageCost;
  }
  return c;
}

// Radices 4 (as many as fit), then 3, then a lone 2 for m = 2^a 3^b; empty if m
// has another prime factor.
static std::vector<int> register_chain(int m) {
  std::vector<int> r;
  int a = 0, b = 0;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  if (m != 1) return r;
  for (int i = 0; i < a / 2; ++i) r.push_back(4);
  for (int i = 0; i < b; ++i) r.push_back(3);
  if (a & 1) r.push_back(2);
  return r;
}

// Product grid of the fused 1D1V stepper for an axis of n points and mask cut
// K (both factors of the product are masked to |k| <= K, so any m >= 3K+1 gives
// the kept modes exactly; m <= n when max_n).  Mode 0: an n with a prime factor
// >= 5 (whose transform needs the two-phase odd-radix stages, measured slower than
// their FP64 count) takes the 2^a 3^b length of least register_chain_cost;
// n = 2^a 3^b keeps n.  Mode 2: the cheapest length by line_pair_cost (radices 2,
// 4, 8 or odd up to 31) at <= 0.8x of n's, with no more stages than n.  Returns
// m == n (and rads empty) otherwise.
static int choose_product_grid(int n, int cut, bool max_n, std::vector<int>& rads, int mode = -1) {
  rads.clear();
  if (mode < 0) mode = g_product_grid;
  // M != n is exact only where the n-point product folds at most the single
  // pair k1 = k2 = +-cut (3 cut == n); with 3 cut > n more terms alias on the
  // n-point grid than the stepper adds back, so such plans keep n
  if (mode == 1 || cut < 1 || n < 8 || 3 * cut > n) return n;
  if (mode == 0) {
    if (!register_chain(n).empty()) return n;
    double best = 0.0;
    int bm = n;
    for (int m = 3 * cut + 1; m <= 2 * n; ++m) {
      if (max_n && m > n) break;
      const std::vector<int> r = register_chain(m);
      if (r.empty() || (int)r.size() > MAXST) continue;
      const double c = register_chain_cost(m, r);
      if (bm == n || c < best) { best = c; bm = m; rads = r; }
    }
    return bm;
  }
  const std::vector<int> fn = factorize(n);
  const double base = line_pair_cost(n, fn, cut);
  double best = 0.8 * base;
  int bm = n;
  for (int m = 3 * cut + 1; m <= 2 * n; ++m) {
    if (m == n || (max_n && m > n)) continue;
    const std::vector<int> f = factorize(m);
    bool small = (int)f.size() <= MAXST;
    for (int r : f) small = small && (r <= 8 || ((r & 1) && r <= 31));
    if (!small) continue;
    for (const auto& o : radix_orders(m)) {
      const double c = line_pair_cost(m, o, cut);
      if ((int)o.size() > (int)fn.size() && c > 0.5 * base) continue;
      if (c < best) { best = c; bm = m; rads = o; }
    }
  }
  return bm;
}

int build_plan_host(const spx_problem* pb, int nsm, spx_plan* pl, int tile, int mgrid) {
  if (!pb) { set_error("null problem"); return SPX_E_ARG; }
  const spx_problem& p = *pb;
  if (p.Nx < 1 || p.Ny < 1 || p.Nz < 1 || p.Nn < 1 || p.Nm < 1 || p.Np < 1 || p.Ns < 1) {
    set_error("all sizes must be >= 1"); return SPX_E_ARG;
  }
  if (p.Ns > SPX_MAX_SPECIES) { set_error("too many species"); return SPX_E_ARG; }
  if (p.Nx > SPX_MAX_AXIS || p.Ny > SPX_MAX_AXIS || p.Nz > SPX_MAX_AXIS) {
    set_error("an axis is longer than SPX_MAX_AXIS"); return SPX_E_UNSUPPORTED;
  }
  for (int s = 0; s < p.Ns; ++s)
    for (int d = 0; d < 3; ++d)
      if (!(p.alpha_s[3 * s + d] != 0.0)) { set_error("alpha_s must be non-zero"); return SPX_E_ARG; }
  if (!(p.Omega_cs[0] != 0.0)) { set_error("Omega_cs[0] must be non-zero"); return SPX_E_ARG; }
  if (!(p.Lx != 0.0) || !(p.Ly != 0.0) || !(p.Lz != 0.0)) { set_error("L must be non-zero"); return SPX_E_ARG; }

  DevPlan& P = pl->host;
  std::memset(&P, 0, sizeof(P));
  P.pb = p;
  pl->tab.clear();
  int rc;
  if ((rc = build_axis(p.Ny, p.cut_y, p.Ly, pl->tab, P.ax[0])) != SPX_OK) return rc;
  if ((rc = build_axis(p.Nx, p.cut_x, p.Lx, pl->tab, P.ax[1])) != SPX_OK) return rc;
  if ((rc = build_axis(p.Nz, p.cut_z, p.Lz, pl->tab, P.ax[2])) != SPX_OK) return rc;
  P.plane = p.Ny * p.Nx * p.Nz;
  P.nh = p.Nn * p.Nm * p.Np;
  P.nc = (long long)p.Ns * P.nh * P.plane;
  P.tab_len = (int)pl->tab.size();
  P.prow = p.Nx * p.Nz;
  P.pplane = P.plane;
  pl->nsm = nsm > 0 ? nsm : 152;
  pl->smem_tab = ((size_t)P.tab_len * sizeof(double2) + 255) / 256 * 256;
  const size_t smem_max = 227 * 1024 - 4096;
  const bool onev = (p.Ny == 1 && p.Nz == 1 && p.Nm == 1 && p.Np == 1);
  for (int sp = 0; sp < p.Ns; ++sp) P.ua[sp] = p.u_s[3 * sp] / p.alpha_s[3 * sp];
  P.iO0 = 1.0 / p.Omega_cs[0];
  pl->coef.clear();
  pl->gen.clear();
  P.axm = P.ax[1];      // products on the Nx-point grid unless the 1D1V branch picks another
  P.rnm = 1.0;
  P.alias = 0;
  if (onev) {
    P.path = 0;
    pl->coef.resize((size_t)p.Ns * p.Nn * COEF_1V);
    for (int sp = 0; sp < p.Ns; ++sp)
      for (int n = 0; n < p.Nn; ++n) coef_1v(p, sp, n, &pl->coef[((size_t)sp * p.Nn + n) * COEF_1V]);
    const int N = p.Nx;
    const long long planes = (long long)p.Ns * p.Nn;
    int T = tile > 0 ? tile : (int)((planes + pl->nsm - 1) / pl->nsm);
    T = std::max(1, std::min(T, 16));
    // shared memory of the widest user: lines_1v(T, Ns)*N double2 + table
    while (T > 1 && pl->smem_tab + (size_t)lines_1v(T, p.Ns) * N * sizeof(double2) > smem_max) --T;
    int ntiles = (p.Nn + T - 1) / T;
    T = (p.Nn + ntiles - 1) / ntiles;   // even out the tiles
    P.tile = T;
    P.ntiles = ntiles;
    // product grid of the stepper (axm); its twiddles extend the table
    std::vector<int> mr;
    const int M = mgrid ? choose_product_grid(N, p.cut_x, mgrid == 2, mr) : N;
    if (M != N) {
      std::vector<double2> tab2 = pl->tab;
      AxisPlan am;
      if ((rc = build_axis(M, p.cut_x, p.Lx, tab2, am, &mr, false)) != SPX_OK) return rc;
      const size_t tab2_bytes = (tab2.size() * sizeof(double2) + 255) / 256 * 256;
      // the staged stage kernel must still fit with one staged epilogue operand
      const size_t stage = tab2_bytes + (size_t)stage_area_1v(T, p.Ns, N, M) * sizeof(double2) +
                           64 * sizeof(double) + (size_t)T * N * sizeof(double2);
      if (stage <= smem_max) {
        pl->tab.swap(tab2);
        P.tab_len = (int)pl->tab.size();
        pl->smem_tab = tab2_bytes;
        P.axm = am;
        P.rnm = (double)N / (double)M;
        P.alias = (3 * p.cut_x == N) ? 1 : 0;
      }
    }
    pl->smem_1v = pl->smem_tab + (size_t)lines_1v(T, p.Ns) * N * sizeof(double2) + 16 * 4 * sizeof(double);
    // the VJP keeps one partial field line per (species, tile); the fused
    // VJP + parameter kernel adds per-CTA parameter partials and one partial
    // line per group of 8 tiles
    pl->ws_bytes = (size_t)p.Ns * ntiles * N * sizeof(double2) +
                   (size_t)(p.Ns * ntiles + 1) * (2 + SPX_MAX_SPECIES) * sizeof(double) +
                   (size_t)p.Ns * ((ntiles + 7) / 8) * N * sizeof(double2);
  } else {
    P.path = 1;
    // shared-memory rows padded to an odd length (see fft_planes_t)
    P.prow = p.Nx * p.Nz;
    if (p.Ny > 1 && (P.prow & 1) == 0) P.prow += 1;
    P.pplane = p.Ny * P.prow;
    pl->smem_gen = pl->smem_tab + 2 * (size_t)P.pplane * sizeof(double2);
    pl->big = pl->smem_gen > smem_max;
    if (pl->big) {
      // the plane does not fit: spx_rhs transforms one axis at a time over
      // batches of lines staged through shared memory (k_big_lines)
      const int nmax = std::max(p.Nx, std::max(p.Ny, p.Nz));
      const size_t per_line = 2 * (size_t)nmax * sizeof(double2);
      if (pl->smem_tab + per_line > smem_max) {
        set_error("an FFT line of this length does not fit in shared memory");
        return SPX_E_UNSUPPORTED;
      }
      pl->big_nl = (int)std::min<size_t>(32, (smem_max - pl->smem_tab) / per_line);
      pl->smem_big = pl->smem_tab + (size_t)pl->big_nl * per_line;
    }
    const int nplanes = p.Ns * P.nh;
    // forward table (GenPlane per plane), then the transposed bracket (GenPlaneT per plane)
    std::vector<GenPlane> fwd((size_t)nplanes);
    for (int id = 0; id < nplanes; ++id) fwd[id] = gen_plane(P, id);
    std::vector<GenPlaneT> tr((size_t)nplanes);
    if (!gen_plane_t(fwd.data(), nplanes, tr.data())) {
      set_error("internal: a Hermite plane has too many transposed bracket terms");
      return SPX_E_UNSUPPORTED;
    }
    pl->gen.resize((size_t)nplanes * (sizeof(GenPlane) + sizeof(GenPlaneT)));
    std::memcpy(pl->gen.data(), fwd.data(), (size_t)nplanes * sizeof(GenPlane));
    std::memcpy(pl->gen.data() + (size_t)nplanes * sizeof(GenPlane), tr.data(),
                (size_t)nplanes * sizeof(GenPlaneT));
    // real-space planes of y (RHS), of y and v (JVP); of y, the forward
    // transforms of w and 6 Ns partial field sums per chunk of planes (VJP)
    const size_t nreal = (size_t)p.Ns * P.nh + 3 * (size_t)p.Ns + 3;
    const size_t nws = std::max(2 * nreal, nreal + (size_t)nplanes + 6 * (size_t)p.Ns * vjp_nchunk(P.nh));
    pl->ws_bytes = nws * P.plane * sizeof(double2);
  }
  if (pl->smem_1v > smem_max) { set_error("Nx too large for the fused path"); return SPX_E_UNSUPPORTED; }
  return SPX_OK;
}

// ------------------------------------------------------------------ kernels
__global__ void __launch_bounds__(NTHREADS, 2) k_rhs1v(const DevPlan* __restrict__ gP,
                                                    const double2* __restrict__ gtab,
                                                    const double2* __restrict__ y,
                                                    double2* __restrict__ dy) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  EpiStore epi{dy};
  const int nblk = P.pb.Ns * P.ntiles;
  if ((int)blockIdx.x == nblk) {
    maxwell_range(P, stab, y, 0, P.plane, epi);
    return;
  }
  const int s = blockIdx.x / P.ntiles, tile = blockIdx.x % P.ntiles;
  const int n0 = tile * P.tile;
  const int nt = min(P.tile, P.pb.Nn - n0);
  if (nt <= 0) return;
  const int N = P.ax[1].n;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)(P.tile + 1) * N;
  double* scoef = reinterpret_cast<double*>(sB + (size_t)(P.tile + 1) * N);
  rhs1v_tile(P, stab, y, s, n0, nt, sA, sB, scoef, epi);
}

__global__ void __launch_bounds__(GEN_THREADS, 1) k_gen_real(const DevPlan* __restrict__ gP,
                                                       const double2* __restrict__ gtab,
                                                       const double2* __restrict__ y,
                                                       double2* __restrict__ ws) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int id = blockIdx.x;
  general_to_real(P, stab, y, id, ws + (size_t)id * P.plane, sA, sB);
}

__global__ void __launch_bounds__(GEN_THREADS, 1) k_gen_nl(const DevPlan* __restrict__ gP,
                                                     const double2* __restrict__ gtab,
                                                     const double2* __restrict__ y,
                                                     const double2* __restrict__ ws,
                                                     double2* __restrict__ dy) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  EpiStore epi{dy};
  const int nplanes = P.pb.Ns * P.nh;
  if ((int)blockIdx.x == nplanes) {
    maxwell_range(P, stab, y, 0, P.plane, epi);
    return;
  }
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const double2* GB = ws + (size_t)nplanes * P.plane;
  general_nl_plane(P, stab, y, ws, GB, blockIdx.x, sA, sB, epi);
}

__global__ void __launch_bounds__(NTHREADS, 2) k_jvp1v(const DevPlan* __restrict__ gP,
                                                    const double2* __restrict__ gtab,
                                                    const double2* __restrict__ y,
                                                    const double2* __restrict__ v,
                                                    double2* __restrict__ out) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  EpiStore epi{out};
  const int nblk = P.pb.Ns * P.ntiles;
  if ((int)blockIdx.x == nblk) {
    maxwell_range(P, stab, v, 0, P.plane, epi);   // Maxwell + current are linear
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
  rhs1v_tile_t<true>(P, stab, y, v, s, n0, nt, sA, sB, scoef, epi);
}

__global__ void __launch_bounds__(NTHREADS, 2) k_vjp1v(const DevPlan* __restrict__ gP,
                                                    const double2* __restrict__ gtab,
                                                    const double2* __restrict__ y,
                                                    const double2* __restrict__ w,
                                                    double2* __restrict__ g,
                                                    double2* __restrict__ part) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const int s = blockIdx.x / P.ntiles, tile = blockIdx.x % P.ntiles;
  const int m0 = tile * P.tile;
  const int nt = min(P.tile, P.pb.Nn - m0);
  const int N = P.ax[1].n;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)(2 * P.tile + 2) * N;
  double* scoef = reinterpret_cast<double*>(sB + (size_t)(2 * P.tile + 2) * N);
  if (nt <= 0) {
    for (int x = threadIdx.x; x < N; x += blockDim.x)
      part[((size_t)s * P.ntiles + tile) * N + x] = make_double2(0.0, 0.0);
    return;
  }
  vjp1v_tile(P, stab, y, w, g, part, s, tile, m0, nt, sA, sB, scoef);
}

__global__ void __launch_bounds__(NTHREADS, 2) k_vjp1v_fields(const DevPlan* __restrict__ gP,
                                                           const double2* __restrict__ gtab,
                                                           const double2* __restrict__ w,
                                                           double2* __restrict__ g,
                                                           const double2* __restrict__ part) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const int N = P.ax[1].n;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)P.pb.Ns * N;
  vjp1v_fields(P, stab, w, g, part, sA, sB);
}

__global__ void __launch_bounds__(GEN_THREADS, 1) k_jvp_real(const DevPlan* __restrict__ gP,
                                                       const double2* __restrict__ gtab,
                                                       const double2* __restrict__ y,
                                                       const double2* __restrict__ v,
                                                       double2* __restrict__ ws) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int nreal = P.pb.Ns * P.nh + 3 * P.pb.Ns + 3;
  const int b = blockIdx.x;
  const bool second = b >= nreal;
  const int id = second ? b - nreal : b;
  general_to_real(P, stab, second ? v : y, id, ws + (size_t)b * P.plane, sA, sB);
}

// wy: real-space planes and field combinations of y; wv: the same of v
__global__ void __launch_bounds__(GEN_THREADS, 1) k_jvp_nl(const DevPlan* __restrict__ gP,
                                                     const double2* __restrict__ gtab,
                                                     const double2* __restrict__ v,
                                                     const double2* __restrict__ wy,
                                                     const double2* __restrict__ wv,
                                                     double2* __restrict__ out) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  EpiStore epi{out};
  const int nplanes = P.pb.Ns * P.nh;
  if ((int)blockIdx.x == nplanes) {
    maxwell_range(P, stab, v, 0, P.plane, epi);
    return;
  }
  const size_t pl = (size_t)P.plane;
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const double2* Cy = wy;
  const double2* Gy = wy + (size_t)nplanes * pl;
  const double2* Cv = wv;
  const double2* Gv = wv + (size_t)nplanes * pl;
  general_nl_plane_t<1>(P, stab, v, Cv, Gy, Cy, Gv, blockIdx.x, sA, sB, epi);
}

// Linearised JVP, pass 2: Gy = y's real-space field combinations, Sy = y's
// bracket sums (6 planes per Hermite plane), wv = v's real-space planes and fields.
__global__ void __launch_bounds__(GEN_THREADS, 1) k_jvp_nl_lin(const DevPlan* __restrict__ gP,
                                                              const double2* __restrict__ gtab,
                                                              const double2* __restrict__ v,
                                                              const double2* __restrict__ Gy,
                                                              const double2* __restrict__ Sy,
                                                              const double2* __restrict__ wv,
                                                              double2* __restrict__ out) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  EpiStore epi{out};
  const int nplanes = P.pb.Ns * P.nh;
  if ((int)blockIdx.x == nplanes) {
    maxwell_range(P, stab, v, 0, P.plane, epi);
    return;
  }
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const double2* Gv = wv + (size_t)nplanes * P.plane;
  general_nl_plane_t<2>(P, stab, v, wv, Gy, Sy, Gv, blockIdx.x, sA, sB, epi);
}

// The bracket sums of every Hermite plane of y (real-space planes R) into S.
__global__ void __launch_bounds__(GEN_THREADS, 1) k_lin_sums(const DevPlan* __restrict__ gP,
                                                            const double2* __restrict__ R,
                                                            double2* __restrict__ S) {
  __shared__ DevPlan P;
  if (threadIdx.x == 0) P = *gP;
  __syncthreads();
  lin_bracket_sums(P, R, blockIdx.x, S + (size_t)blockIdx.x * 6 * P.plane);
}

// General-path VJP, pass 1: y's real-space planes and field combinations
// (blocks [0, nreal)), then W_r of w (blocks [nreal, nreal + nplanes)).
__global__ void __launch_bounds__(GEN_THREADS, 1) k_vjp_real(const DevPlan* __restrict__ gP,
                                                            const double2* __restrict__ gtab,
                                                            const double2* __restrict__ y,
                                                            const double2* __restrict__ w,
                                                            double2* __restrict__ ws) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int nreal = P.pb.Ns * P.nh + 3 * P.pb.Ns + 3;
  const int b = blockIdx.x;
  if (b < nreal) general_to_real(P, stab, y, b, ws + (size_t)b * P.plane, sA, sB);
  else general_w_real(P, stab, w, b - nreal, ws + (size_t)b * P.plane, sA, sB);
}

// Pass 2: the partial field sums, one thread per (point, species, component,
// chunk of VJP_HCHUNK planes): blockIdx.y = s * 6 + j, blockIdx.z = chunk,
// written to plane blockIdx.z * 6 Ns + blockIdx.y of S.
__global__ void __launch_bounds__(NTHREADS) k_vjp_fsum(const DevPlan* __restrict__ gP,
                                                      const double2* __restrict__ ws,
                                                      double2* __restrict__ S) {
  __shared__ DevPlan P;
  if (threadIdx.x == 0) P = *gP;
  __syncthreads();
  const int nreal = P.pb.Ns * P.nh + 3 * P.pb.Ns + 3;
  const double2* W = ws + (size_t)nreal * P.plane;
  const int s = blockIdx.y / 6, j = blockIdx.y % 6;
  const int h0 = blockIdx.z * VJP_HCHUNK, h1 = min(P.nh, h0 + VJP_HCHUNK);
  double2* out = S + ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * P.plane;
  for (size_t pt = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pt < (size_t)P.plane;
       pt += (size_t)gridDim.x * blockDim.x)
    out[pt] = vjp_field_sum(P, ws, W, pt, s, j, h0, h1);
}

// Pass 3: blocks [0, nplanes) the Hermite planes of g, then six field blocks.
__global__ void __launch_bounds__(GEN_THREADS, 1) k_vjp_gen(const DevPlan* __restrict__ gP,
                                                           const double2* __restrict__ gtab,
                                                           const double2* __restrict__ w,
                                                           const double2* __restrict__ ws,
                                                           const double2* __restrict__ S,
                                                           double2* __restrict__ g) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  EpiStore epi{g};
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + P.pplane;
  const int nplanes = P.pb.Ns * P.nh;
  const int nreal = nplanes + 3 * P.pb.Ns + 3;
  const int b = blockIdx.x;
  if (b >= nplanes) {
    vjp_field_plane(P, stab, w + P.nc, S, b - nplanes, sA, sB, epi);
    return;
  }
  const double2* GB = ws + (size_t)nplanes * P.plane;
  const double2* W = ws + (size_t)nreal * P.plane;
  general_nl_plane_t<3>(P, stab, w, W, GB, nullptr, nullptr, b, sA, sB, epi);
}

// ------------------------------------------------------------------------
// Multi-pass general path (planes larger than one CTA's shared memory).  The
// plane transforms run one axis at a time over batches of lines staged through
// shared memory; between passes the planes sit in global memory in natural
// order (standard, unshifted index along every axis).  Workspace planes:
// [0, nplanes) real-space Hermite planes, [nplanes, nreal) field combinations,
// [nreal, nreal + nplanes) bracket products, transformed in place.
// ------------------------------------------------------------------------

// Masked entries of y (Hermite planes, then the field combinations) scattered
// to standard order.
__global__ void __launch_bounds__(NTHREADS) k_big_scatter(const DevPlan* __restrict__ gP,
                                                         const double2* __restrict__ y,
                                                         double2* __restrict__ ws) {
  __shared__ DevPlan P;
  if (threadIdx.x == 0) P = *gP;
  __syncthreads();
  const int Ny = P.ax[0].n, Nx = P.ax[1].n, Nz = P.ax[2].n;
  const int nplanes = P.pb.Ns * P.nh;
  const size_t pl = (size_t)P.plane;
  const size_t total = (size_t)(nplanes + 3 * P.pb.Ns + 3) * pl;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int id = (int)(i / pl);
    const size_t pt = i - (size_t)id * pl;
    const int cz = (int)(pt % Nz), cx = (int)((pt / Nz) % Nx), cy = (int)(pt / ((size_t)Nz * Nx));
    double2 v = make_double2(0.0, 0.0);
    if (kept(cy, Ny, P.ax[0].cut) && kept(cx, Nx, P.ax[1].cut) && kept(cz, Nz, P.ax[2].cut))
      v = id < nplanes ? y[i] : field_combo_point(P, y + P.nc, id - nplanes, pt);
    ws[(size_t)id * pl + ((size_t)std_index(cy, Ny) * Nx + std_index(cx, Nx)) * Nz + std_index(cz, Nz)] = v;
  }
}

// One pass of the plane transforms along `axis` (0 y, 1 x, 2 z) for planes
// blockIdx.y of buf: CTA blockIdx.x stages lines [l0, l0 + nl) in shared
// memory (rows of the axis length), transforms them with the axis plan's
// pruning (DIF = false: inputs masked along the axis; true: only the kept
// outputs are needed) and writes them back.  Loads and stores walk along
// whichever of element and line index is contiguous in memory.
template <bool INV, bool DIF>
__global__ void __launch_bounds__(NTHREADS) k_big_lines(const DevPlan* __restrict__ gP,
                                                       const double2* __restrict__ gtab,
                                                       double2* __restrict__ buf, int axis, int nl) {
  __shared__ DevPlan P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* stab = reinterpret_cast<double2*>(smem_raw);
  load_plan(P, stab, gP, gtab);
  const AxisPlan& ap = P.ax[axis];
  const int n = ap.n;
  const int Nx = P.ax[1].n, Nz = P.ax[2].n;
  const size_t pl = (size_t)P.plane;
  const int nlines = (int)(pl / n);
  const int l0 = blockIdx.x * nl;
  if (l0 >= nlines) return;
  const int nt = min(nl, nlines - l0);
  double2* sA = stab + (P.tab_len + 15) / 16 * 16;
  double2* sB = sA + (size_t)nl * n;
  double2* g = buf + (size_t)blockIdx.y * pl;
  // element e of line l: base(l) + e * stride
  const size_t stride = axis == 2 ? 1 : (axis == 1 ? (size_t)Nz : (size_t)Nx * Nz);
  auto base = [&](int l) -> size_t {
    if (axis == 2) return (size_t)l * Nz;                              // l = y*Nx + x
    if (axis == 1) return (size_t)(l / Nz) * Nx * Nz + (size_t)(l % Nz);  // l = y*Nz + z
    return (size_t)l;                                                  // l = x*Nz + z
  };
  const bool efast = stride == 1;
  const int tot = nt * n;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int j = efast ? i / n : i % nt, e = efast ? i % n : i / nt;
    sA[j * n + e] = g[base(l0 + j) + (size_t)e * stride];
  }
  __syncthreads();
  const double2* r = fft_axis_t<INV, DIF>(sA, sB, ap, stab, Lines{nt, 1, 1, n, 0}, ap.cut);
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int j = efast ? i / n : i % nt, e = efast ? i % n : i / nt;
    g[base(l0 + j) + (size_t)e * stride] = r[j * n + e];
  }
}

// Real-space bracket of every Hermite plane into the product planes.
__global__ void __launch_bounds__(NTHREADS) k_big_bracket(const DevPlan* __restrict__ gP,
                                                         double2* __restrict__ ws) {
  __shared__ DevPlan P;
  if (threadIdx.x == 0) P = *gP;
  __syncthreads();
  const int Ns = P.pb.Ns, nplanes = Ns * P.nh, nreal = nplanes + 3 * Ns + 3;
  const size_t pl = (size_t)P.plane;
  const double2* GB = ws + (size_t)nplanes * pl;
  double2* prod = ws + (size_t)nreal * pl;
  const GenPlane* gp = static_cast<const GenPlane*>(P.gen);
  const size_t total = (size_t)nplanes * pl;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / pl);
    const size_t x = i - (size_t)r * pl;
    const NlCoef& cf = gp[r].cf;
    const bool anyx = cf.ix[0] >= 0 || cf.ix[1] >= 0 || cf.ix[2] >= 0;
    const bool anyy = cf.iy[0] >= 0 || cf.iy[1] >= 0 || cf.iy[2] >= 0;
    const bool anyz = cf.iz[0] >= 0 || cf.iz[1] >= 0 || cf.iz[2] >= 0;
    prod[i] = bracket_point(cf, ws, field_planes(GB, r / P.nh, Ns, pl), pl, x, anyx, anyy, anyz,
                            make_double2(0.0, 0.0));
  }
}

// Output Hermite planes: linear terms plus the transformed bracket.
__global__ void __launch_bounds__(NTHREADS) k_big_epi(const DevPlan* __restrict__ gP,
                                                     const double2* __restrict__ gtab,
                                                     const double2* __restrict__ y,
                                                     const double2* __restrict__ ws,
                                                     double2* __restrict__ dy) {
  __shared__ DevPlan P;
  if (threadIdx.x == 0) P = *gP;
  __syncthreads();
  const int nplanes = P.pb.Ns * P.nh, nreal = nplanes + 3 * P.pb.Ns + 3;
  const size_t pl = (size_t)P.plane;
  const double2* F = ws + (size_t)nreal * pl;
  const size_t total = (size_t)nplanes * pl;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int id = (int)(i / pl);
    dy[i] = big_epi_point(P, gtab, y, F, id, i - (size_t)id * pl);
  }
}

// Current and Maxwell's equations, a range of points per CTA.
__global__ void __launch_bounds__(NTHREADS) k_big_maxwell(const DevPlan* __restrict__ gP,
                                                         const double2* __restrict__ gtab,
                                                         const double2* __restrict__ y,
                                                         double2* __restrict__ dy) {
  __shared__ DevPlan P;
  if (threadIdx.x == 0) P = *gP;
  __syncthreads();
  EpiStore epi{dy};
  const int chunk = (P.plane + gridDim.x - 1) / gridDim.x;
  const int p0 = blockIdx.x * chunk, p1 = min(P.plane, p0 + chunk);
  if (p0 < p1) maxwell_range(P, gtab, y, p0, p1, epi);
}

static bool g_attr_done = false;

// Allow each kernel the opt-in shared memory minus its static part.
template <class K>
static int allow_smem(K kernel, int optin) {
  cudaFuncAttributes fa;
  SPX_CUDA(cudaFuncGetAttributes(&fa, kernel));
  SPX_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                optin - (int)fa.sharedSizeBytes));
  return SPX_OK;
}

int check_plan_device(const spx_plan* pl, const char* who) {
  int dev = -1;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, who);
  if (dev != pl->device) {
    set_error(std::string(who) + ": the current device (" + std::to_string(dev) +
              ") is not the plan's device (" + std::to_string(pl->device) + ")");
    return SPX_E_ARG;
  }
  return SPX_OK;
}

int smem_optin() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return optin;
}

static int set_attrs() {
  if (g_attr_done) return SPX_OK;
  const int optin = smem_optin();
  if (optin <= 0) { set_error("cannot query shared memory limit"); return SPX_E_CUDA; }
  int rc;
  if ((rc = allow_smem(k_rhs1v, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_gen_real, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_gen_nl, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_jvp1v, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_vjp1v, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_vjp1v_fields, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_jvp_real, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_jvp_nl, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_jvp_nl_lin, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_vjp_real, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_vjp_gen, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_big_lines<true, false>, optin)) != SPX_OK) return rc;
  if ((rc = allow_smem(k_big_lines<false, true>, optin)) != SPX_OK) return rc;
  g_attr_done = true;
  return SPX_OK;
}

int launch_rhs(const spx_plan* pl, const double2* y, double2* dy, double2* ws, cudaStream_t st) {
  const DevPlan& P = pl->host;
  if (P.path == 0) {
    const int grid = P.pb.Ns * P.ntiles + 1;
    k_rhs1v<<<grid, pl->threads, pl->smem_1v, st>>>(pl->d_plan, pl->d_tab, y, dy);
  } else if (pl->big) {
    const int nplanes = P.pb.Ns * P.nh, nreal = nplanes + 3 * P.pb.Ns + 3;
    const size_t pln = (size_t)P.plane;
    const int grid = 152 * 8;
    k_big_scatter<<<grid, NTHREADS, 0, st>>>(pl->d_plan, y, ws);
    for (int axis = 2; axis >= 0; --axis) {     // z, x, y
      const int n = P.ax[axis].n;
      if (n == 1) continue;
      const int nb = (int)((pln / n + pl->big_nl - 1) / pl->big_nl);
      k_big_lines<true, false><<<dim3(nb, nreal), NTHREADS, pl->smem_big, st>>>(pl->d_plan, pl->d_tab, ws, axis,
                                                                                pl->big_nl);
    }
    k_big_bracket<<<grid, NTHREADS, 0, st>>>(pl->d_plan, ws);
    for (int axis = 2; axis >= 0; --axis) {
      const int n = P.ax[axis].n;
      if (n == 1) continue;
      const int nb = (int)((pln / n + pl->big_nl - 1) / pl->big_nl);
      k_big_lines<false, true><<<dim3(nb, nplanes), NTHREADS, pl->smem_big, st>>>(
          pl->d_plan, pl->d_tab, ws + (size_t)nreal * pln, axis, pl->big_nl);
    }
    k_big_epi<<<grid, NTHREADS, 0, st>>>(pl->d_plan, pl->d_tab, y, ws, dy);
    k_big_maxwell<<<(int)std::min<size_t>(152, (pln + NTHREADS - 1) / NTHREADS), NTHREADS, 0, st>>>(
        pl->d_plan, pl->d_tab, y, dy);
  } else {
    const int nplanes = P.pb.Ns * P.nh;
    k_gen_real<<<nplanes + 3 * P.pb.Ns + 3, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, y, ws);
    k_gen_nl<<<nplanes + 1, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, y, ws, dy);
  }
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

// Entry points that keep whole planes in shared memory refuse plans whose
// planes do not fit (those run spx_rhs through the multi-pass kernels only).
static int refuse_big(const spx_plan* pl, const char* who) {
  if (!pl || !pl->big) return SPX_OK;
  set_error(std::string(who) + ": a Fourier plane of this size does not fit in shared memory "
                               "(such plans support spx_rhs only)");
  return SPX_E_UNSUPPORTED;
}

}  // namespace spx

// ------------------------------------------------------------------ C ABI
using namespace spx;

extern "C" {

const char* spx_last_error(void) { return g_last_error.c_str(); }

const char* spx_version(void) { return "spectrax_gb300 0.1 (sm_103a, FP64)"; }

int64_t spx_state_len(const spx_problem* pb) {
  if (!pb) return -1;
  const int64_t plane = (int64_t)pb->Nx * pb->Ny * pb->Nz;
  return (int64_t)pb->Ns * pb->Nn * pb->Nm * pb->Np * plane + 6 * plane;
}

int spx_plan_create(const spx_problem* pb, spx_plan** out) { return spx_plan_create_ex(pb, 0, 0, out); }

int spx_plan_create_ex(const spx_problem* pb, int32_t tile, int32_t threads, spx_plan** out) {
  if (!out) { set_error("null output pointer"); return SPX_E_ARG; }
  *out = nullptr;
  if (tile < 0 || tile > 16 || !(threads == 0 || (threads >= 32 && threads <= 256 && threads % 32 == 0))) {
    set_error("spx_plan_create_ex: tile must be 0..16 and threads 0 or a multiple of 32 in 32..256");
    return SPX_E_ARG;
  }
  int dev = 0;
  SPX_CUDA(cudaGetDevice(&dev));
  int nsm = 0;
  SPX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  spx_plan* pl = new spx_plan();
  pl->device = dev;
  pl->threads = threads > 0 ? threads : NTHREADS;
  int rc = build_plan_host(pb, nsm, pl, tile);
  if (rc != SPX_OK) { delete pl; return rc; }
  {
    // streaming and Maxwell terms keep C(-k) = conj C(k) only if k(N-1-c) == -k(c) exactly
    const DevPlan& H = pl->host;
    bool anti = H.path == 0 && (H.ax[1].n & 1);
    for (int c = 0; anti && c < H.ax[1].n; ++c)
      if (!(pl->tab[H.ax[1].kofs + c].x == -pl->tab[H.ax[1].kofs + H.ax[1].n - 1 - c].x)) anti = false;
    pl->herm_ok = anti;
  }
  rc = set_attrs();
  if (rc != SPX_OK) { delete pl; return rc; }
  const size_t hdr = (sizeof(DevPlan) + 255) / 256 * 256;
  const size_t tab_bytes = (pl->tab.size() * sizeof(double2) + 255) / 256 * 256;
  // tickets: [0] the fused VJP's completion ticket, from [64] one counter per
  // group of 8 Hermite tiles (its group-partial reduction)
  const size_t ngroups = (size_t)pb->Ns * ((pl->host.ntiles + 7) / 8 + 1);
  const size_t ticket_bytes = (256 + 4 * ngroups + 255) / 256 * 256;
  const size_t coef_bytes = (pl->coef.size() * sizeof(double) + 255) / 256 * 256;
  const size_t gen_bytes = (pl->gen.size() + 255) / 256 * 256;
  const size_t bytes = hdr + tab_bytes + ticket_bytes + coef_bytes + gen_bytes;
  cudaError_t e = cudaMalloc(&pl->d_block, bytes);
  if (e != cudaSuccess) { delete pl; return cuda_fail(e, "cudaMalloc(plan)"); }
  pl->d_plan = reinterpret_cast<DevPlan*>(pl->d_block);
  pl->d_tab = reinterpret_cast<double2*>(reinterpret_cast<char*>(pl->d_block) + hdr);
  pl->d_ticket = reinterpret_cast<unsigned int*>(reinterpret_cast<char*>(pl->d_block) + hdr + tab_bytes);
  double* d_coef = reinterpret_cast<double*>(reinterpret_cast<char*>(pl->d_block) + hdr + tab_bytes + ticket_bytes);
  pl->host.coef = pl->coef.empty() ? nullptr : d_coef;
  char* d_gen = reinterpret_cast<char*>(pl->d_block) + hdr + tab_bytes + ticket_bytes + coef_bytes;
  pl->host.gen = pl->gen.empty() ? nullptr : d_gen;
  e = cudaMemset(pl->d_ticket, 0, ticket_bytes);
  if (e == cudaSuccess && !pl->coef.empty())
    e = cudaMemcpy(d_coef, pl->coef.data(), pl->coef.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !pl->gen.empty())
    e = cudaMemcpy(d_gen, pl->gen.data(), pl->gen.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(pl->d_plan, &pl->host, sizeof(DevPlan), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !pl->tab.empty())
    e = cudaMemcpy(pl->d_tab, pl->tab.data(), pl->tab.size() * sizeof(double2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(pl->d_block); delete pl; return cuda_fail(e, "cudaMemcpy(plan)"); }
  *out = pl;
  return SPX_OK;
}

int spx_plan_destroy(spx_plan* pl) {
  if (!pl) return SPX_OK;
  if (pl->d_block) cudaFree(pl->d_block);
  delete pl;
  return SPX_OK;
}

int spx_set_product_grid(int32_t mode) {
  if (mode < 0 || mode > 2) { set_error("spx_set_product_grid: mode must be 0 (auto), 1 (Nx) or 2 (least FP64)"); return SPX_E_ARG; }
  g_product_grid = mode;
  return SPX_OK;
}

int spx_plan_product_grid(const spx_plan* pl) { return pl ? pl->host.axm.n : 0; }

int spx_plan_product_radices(const spx_plan* pl, int32_t* radices, int32_t max) {
  if (!pl || (!radices && max > 0) || max < 0) { set_error("spx_plan_product_radices: bad argument"); return SPX_E_ARG; }
  const AxisPlan& am = pl->host.axm;
  for (int i = 0; i < am.nst && i < max; ++i) radices[i] = am.radix[i];
  return am.nst;
}

int spx_product_grid_for(int32_t nx, int32_t cut, int32_t mode) {
  if (nx < 1 || mode < 0 || mode > 2) { set_error("spx_product_grid_for: bad argument"); return SPX_E_ARG; }
  std::vector<int> rads;
  return choose_product_grid(nx, cut, false, rads, mode);
}

size_t spx_rhs_workspace_bytes(const spx_plan* pl) { return pl ? pl->ws_bytes : 0; }

int spx_plan_info(const spx_plan* pl, int32_t* tile, int32_t* ntiles, int32_t* threads, int32_t* path) {
  if (!pl) { set_error("spx_plan_info: null plan"); return SPX_E_ARG; }
  if (tile) *tile = pl->host.tile;
  if (ntiles) *ntiles = pl->host.ntiles;
  if (threads) *threads = pl->threads;
  if (path) *path = pl->big ? 2 : pl->host.path;
  return SPX_OK;
}

int spx_rhs(const spx_plan* pl, const void* y, void* dy, void* ws, size_t ws_bytes, void* stream) {
  if (!pl || !y || !dy) { set_error("spx_rhs: null argument"); return SPX_E_ARG; }
  if (y == dy) { set_error("spx_rhs: y and dy must not alias"); return SPX_E_ARG; }
  if (((uintptr_t)y | (uintptr_t)dy) & 15) { set_error("spx_rhs: pointers must be 16-byte aligned"); return SPX_E_ARG; }
  if (pl->ws_bytes > 0 && (!ws || ws_bytes < pl->ws_bytes || ((uintptr_t)ws & 15))) {
    set_error("spx_rhs: workspace too small or misaligned");
    return SPX_E_WORKSPACE;
  }
  if (int rd = check_plan_device(pl, "spx_rhs")) return rd;
  return launch_rhs(pl, static_cast<const double2*>(y), static_cast<double2*>(dy),
                    static_cast<double2*>(ws), static_cast<cudaStream_t>(stream));
}

static int check_vec_args(const spx_plan* pl, const void* a, const void* b, const void* c, void* ws,
                          size_t ws_bytes, const char* who) {
  if (!pl || !a || !b || !c) { set_error(std::string(who) + ": null argument"); return SPX_E_ARG; }
  if (c == a || c == b) { set_error(std::string(who) + ": output must not alias an input"); return SPX_E_ARG; }
  if (((uintptr_t)a | (uintptr_t)b | (uintptr_t)c) & 15) {
    set_error(std::string(who) + ": pointers must be 16-byte aligned"); return SPX_E_ARG;
  }
  if (pl->ws_bytes > 0 && (!ws || ws_bytes < pl->ws_bytes || ((uintptr_t)ws & 15))) {
    set_error(std::string(who) + ": workspace too small or misaligned"); return SPX_E_WORKSPACE;
  }
  return check_plan_device(pl, who);
}

int spx_jvp(const spx_plan* pl, const void* y, const void* v, void* Jv, void* ws, size_t ws_bytes,
            void* stream) {
  int rc = check_vec_args(pl, y, v, Jv, ws, ws_bytes, "spx_jvp");
  if (rc == SPX_OK) rc = refuse_big(pl, "spx_jvp");
  if (rc != SPX_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const DevPlan& P = pl->host;
  const double2* yy = static_cast<const double2*>(y);
  const double2* vv = static_cast<const double2*>(v);
  double2* out = static_cast<double2*>(Jv);
  double2* w = static_cast<double2*>(ws);
  if (P.path == 0) {
    k_jvp1v<<<P.pb.Ns * P.ntiles + 1, pl->threads, pl->smem_1v, st>>>(pl->d_plan, pl->d_tab, yy, vv, out);
  } else {
    const int nplanes = P.pb.Ns * P.nh;
    const int nreal = nplanes + 3 * P.pb.Ns + 3;
    k_jvp_real<<<2 * nreal, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, yy, vv, w);
    k_jvp_nl<<<nplanes + 1, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, vv, w,
                                                            w + (size_t)nreal * P.plane, out);
  }
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

size_t spx_linearize_bytes(const spx_plan* pl) {
  if (!pl) return 0;
  const DevPlan& P = pl->host;
  if (P.path == 0) return (size_t)(P.nc + 6LL * P.plane) * sizeof(double2);
  // real-space planes and field combinations of y, then 6 bracket sums per plane
  const size_t nplanes = (size_t)P.pb.Ns * P.nh;
  const size_t nreal = nplanes + 3 * (size_t)P.pb.Ns + 3;
  return (nreal + 6 * nplanes) * (size_t)P.plane * sizeof(double2);
}

int spx_linearize(const spx_plan* pl, const void* y, void* lin, size_t lin_bytes, void* stream) {
  if (!pl || !y || !lin) { set_error("spx_linearize: null argument"); return SPX_E_ARG; }
  if (((uintptr_t)y | (uintptr_t)lin) & 15) { set_error("spx_linearize: pointers must be 16-byte aligned"); return SPX_E_ARG; }
  if (lin_bytes < spx_linearize_bytes(pl)) { set_error("spx_linearize: lin too small"); return SPX_E_WORKSPACE; }
  if (int rb = refuse_big(pl, "spx_linearize")) return rb;
  if (int rd = check_plan_device(pl, "spx_linearize")) return rd;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const DevPlan& P = pl->host;
  if (P.path == 0) {
    SPX_CUDA(cudaMemcpyAsync(lin, y, spx_linearize_bytes(pl), cudaMemcpyDeviceToDevice, st));
    return SPX_OK;
  }
  const int nplanes = P.pb.Ns * P.nh;
  const int nreal = nplanes + 3 * P.pb.Ns + 3;
  double2* L = static_cast<double2*>(lin);
  k_gen_real<<<nreal, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, static_cast<const double2*>(y), L);
  k_lin_sums<<<nplanes, GEN_THREADS, 0, st>>>(pl->d_plan, L, L + (size_t)nreal * P.plane);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_jvp_lin(const spx_plan* pl, const void* lin, const void* v, void* Jv, void* ws, size_t ws_bytes,
                void* stream) {
  int rc = check_vec_args(pl, lin, v, Jv, ws, ws_bytes, "spx_jvp_lin");
  if (rc == SPX_OK) rc = refuse_big(pl, "spx_jvp_lin");
  if (rc != SPX_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const DevPlan& P = pl->host;
  const double2* ll = static_cast<const double2*>(lin);
  const double2* vv = static_cast<const double2*>(v);
  double2* out = static_cast<double2*>(Jv);
  if (P.path == 0) {
    k_jvp1v<<<P.pb.Ns * P.ntiles + 1, pl->threads, pl->smem_1v, st>>>(pl->d_plan, pl->d_tab, ll, vv, out);
  } else {
    const int nplanes = P.pb.Ns * P.nh;
    const int nreal = nplanes + 3 * P.pb.Ns + 3;
    double2* w = static_cast<double2*>(ws);
    k_gen_real<<<nreal, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, vv, w);
    k_jvp_nl_lin<<<nplanes + 1, GEN_THREADS, pl->smem_gen, st>>>(
        pl->d_plan, pl->d_tab, vv, ll + (size_t)nplanes * P.plane, ll + (size_t)nreal * P.plane, w, out);
  }
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

int spx_vjp(const spx_plan* pl, const void* y, const void* wv, void* g, void* ws, size_t ws_bytes,
            void* stream) {
  int rc = check_vec_args(pl, y, wv, g, ws, ws_bytes, "spx_vjp");
  if (rc == SPX_OK) rc = refuse_big(pl, "spx_vjp");
  if (rc != SPX_OK) return rc;
  const DevPlan& P = pl->host;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (P.path != 0) {
    // workspace: y's real planes (nreal), W (nplanes), 6 Ns partial field sums per chunk
    const int nplanes = P.pb.Ns * P.nh;
    const int nreal = nplanes + 3 * P.pb.Ns + 3;
    const double2* yy = static_cast<const double2*>(y);
    const double2* ww = static_cast<const double2*>(wv);
    double2* W = static_cast<double2*>(ws);
    double2* S = W + (size_t)(nreal + nplanes) * P.plane;
    k_vjp_real<<<nreal + nplanes, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, yy, ww, W);
    const int fx = (int)std::min<long long>((P.plane + NTHREADS - 1) / NTHREADS, 65535LL);
    k_vjp_fsum<<<dim3(fx, 6 * P.pb.Ns, vjp_nchunk(P.nh)), NTHREADS, 0, st>>>(pl->d_plan, W, S);
    k_vjp_gen<<<nplanes + 6, GEN_THREADS, pl->smem_gen, st>>>(pl->d_plan, pl->d_tab, ww, W, S,
                                                              static_cast<double2*>(g));
    SPX_CUDA(cudaGetLastError());
    return SPX_OK;
  }
  double2* part = static_cast<double2*>(ws);
  k_vjp1v<<<P.pb.Ns * P.ntiles, pl->threads, pl->smem_1v, st>>>(
      pl->d_plan, pl->d_tab, static_cast<const double2*>(y), static_cast<const double2*>(wv),
      static_cast<double2*>(g), part);
  k_vjp1v_fields<<<1, pl->threads, pl->smem_1v, st>>>(pl->d_plan, pl->d_tab, static_cast<const double2*>(wv),
                                                   static_cast<double2*>(g), part);
  SPX_CUDA(cudaGetLastError());
  return SPX_OK;
}

}  // extern "C"
