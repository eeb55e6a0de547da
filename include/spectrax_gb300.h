/*
 * spectrax_gb300 — C ABI of the GB300 (sm_103a) Hermite-Fourier Vlasov-Maxwell
 * right-hand side and its device time steppers.
 *
 * State layout (identical to SPECTRAX): a flat complex128 vector
 *   y = concat(Ck.ravel(), Fk.ravel()),
 *   Ck[(s, p, m, n), ky, kx, kz]  shape (Ns*Np*Nm*Nn, Ny, Nx, Nz),
 *   Fk[(Ex, Ey, Ez, Bx, By, Bz), ky, kx, kz],
 * Fourier axes in fftshift order (index c <-> wavenumber c - N//2), axis order (y, x, z).
 * Complex values are interleaved (re, im) doubles; all device pointers must be
 * 16-byte aligned.  Every function returns 0 (SPX_OK) or a negative SPX_E* code.
 * Streams are passed as `void*` (a cudaStream_t; NULL = legacy default stream).
 */
#ifndef SPECTRAX_GB300_H
#define SPECTRAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPX_MAX_SPECIES 8
#define SPX_MAX_AXIS 256        /* largest Nx, Ny or Nz */

enum {
  SPX_OK = 0,
  SPX_E_ARG = -1,        /* null pointer, bad size, unsupported shape */
  SPX_E_CUDA = -2,       /* a CUDA call failed (see spx_last_error) */
  SPX_E_WORKSPACE = -3,  /* workspace too small or misaligned */
  SPX_E_UNSUPPORTED = -4 /* valid input that this build does not handle */
};

/* Stepper status words (per solve / per batch instance). */
enum {
  SPX_ST_RUNNING = 0,
  SPX_ST_DONE = 1,
  SPX_ST_MAX_STEPS = 2,
  SPX_ST_DT_UNDERFLOW = 3,
  SPX_ST_NONFINITE = 4,
  SPX_ST_WAIT_TIMEOUT = 5   /* a bounded device-side wait for staged data gave up (solve stopped) */
};

/*
 * Problem description: the entries of the reference's 28-tuple `args`
 * (spectrax/_simulation.py:154-161) that are not derivable, plus the 2/3-mask
 * cutoffs.  The k-grids, nabla, k2, collision and ladder tables are rebuilt from
 * these with the formulas of spectrax/_initialization.py:114-146.
 */
typedef struct spx_problem {
  int32_t Nx, Ny, Nz;          /* Fourier modes per axis */
  int32_t Nn, Nm, Np;          /* Hermite modes per velocity axis */
  int32_t Ns;                  /* species, <= SPX_MAX_SPECIES */
  int32_t cut_x, cut_y, cut_z; /* 2/3 mask: largest |k| kept per axis (-1 keeps none) */
  double Lx, Ly, Lz;           /* box lengths */
  double nu, D;                /* hypercollision and hyperdiffusion coefficients */
  double qs[SPX_MAX_SPECIES];
  double Omega_cs[SPX_MAX_SPECIES];
  double alpha_s[3 * SPX_MAX_SPECIES];
  double u_s[3 * SPX_MAX_SPECIES];
} spx_problem;

typedef struct spx_plan spx_plan;  /* opaque: device tables for one problem */

/* Text of the last error recorded by this thread (never NULL). */
const char* spx_last_error(void);

/* Library build info ("sm_103a ..."). */
const char* spx_version(void);

/*
 * Build the device tables (FFT twiddles, k-grids, ladder and collision
 * coefficients) of one problem.  Allocates a small device buffer on the
 * current device.  Replaces the host-side table set-up of
 * spectrax/_initialization.py:114-154.
 */
int spx_plan_create(const spx_problem* pb, spx_plan** out);
/* Same, with the launch shape fixed: `tile` Hermite planes per CTA on the 1D1V
 * path (1..16, 0 = automatic) and `threads` per CTA (multiple of 32 up to 256,
 * 0 = 256).  Used by the autotuner. */
int spx_plan_create_ex(const spx_problem* pb, int32_t tile, int32_t threads, spx_plan** out);
int spx_plan_destroy(spx_plan* plan);
/* Launch shape chosen for a plan (any pointer may be NULL); path 0 = fused 1D1V,
 * 1 = general, 2 = general with planes larger than one CTA's shared memory
 * (about 6.9k points): spx_rhs then transforms one axis at a time over batches
 * of lines through global memory, and spx_jvp, spx_jvp_lin, spx_linearize,
 * spx_vjp and spx_dopri8_create return SPX_E_UNSUPPORTED. */
int spx_plan_info(const spx_plan* plan, int32_t* tile, int32_t* ntiles, int32_t* threads, int32_t* path);

/*
 * Grid of the nonlinear products in the 1D1V Dopri8 stage kernels (the device
 * stepper, the adjoint's recomputation and every batch instance).  The masked factors hold
 * |k| <= K, so the kept modes of their product are exact on any grid of
 * M >= 3K + 1 points (adding back the one term the reference's Nx-point grid
 * folds onto |k| = K when Nx = 3K).  For plans created afterwards: mode 0
 * (default) gives an Nx with a prime factor >= 5 the length M = 2^a 3^b of
 * least modeled time in register butterflies of radices 4, 3 and 2 (129 -> 144
 * = 4*4*3*3, 65 -> 64, 33 -> 36, 17 -> 16, 97 -> 108, 127 -> 128), and keeps
 * Nx = 2^a 3^b; mode 1 always Nx points; mode 2 the cheapest grid of <= 0.8x
 * the FP64 count of the Nx-point transforms, one with more Stockham stages than
 * Nx only at <= 0.5x (129 -> 136, 65 -> 64).  Only plans with 3K <= Nx get
 * M != Nx (with 3K > Nx the Nx-point product folds more than the one term).
 * Results agree to rounding.  spx_plan_product_grid returns the grid length M
 * of a plan.
 */
int spx_set_product_grid(int32_t mode);
int spx_plan_product_grid(const spx_plan* plan);
/* The Stockham radices of that grid in stage order (the first max of them into
 * `radices`); returns their count (0 for a grid of one point). */
int spx_plan_product_radices(const spx_plan* plan, int32_t* radices, int32_t max);
/* The product grid a 1D1V plan with Nx = nx and mask cut `cut` gets under
 * `mode` (host only; no device, no plan).  It applies the selection rule only:
 * plan creation additionally keeps Nx points when the stage kernel with the
 * longer table would not fit in shared memory, which this query does not model. */
int spx_product_grid_for(int32_t nx, int32_t cut, int32_t mode);

/* Number of complex128 entries of the flat state (N_C + N_F). */
int64_t spx_state_len(const spx_problem* pb);

/* Device scratch spx_rhs / spx_jvp need for this plan (bytes; may be 0). */
size_t spx_rhs_workspace_bytes(const spx_plan* plan);

/*
 * dy = f(t, y): the Hermite-Fourier right-hand side.  Replaces
 * spectrax/_simulation.py:55-111 `ode_system` (with spectrax/_model.py:15-212).
 * y and dy are device arrays of spx_state_len() complex128 (must not overlap).
 * Allocates nothing; `ws` must hold spx_rhs_workspace_bytes().
 */
int spx_rhs(const spx_plan* plan, const void* y, void* dy, void* ws, size_t ws_bytes,
            void* stream);

/*
 * Jv = J(y) v: the linearised right-hand side (the JVP that
 * spectrax/midpoint_solver.py:75 obtains with jax.linearize).
 */
int spx_jvp(const spx_plan* plan, const void* y, const void* v, void* Jv, void* ws,
            size_t ws_bytes, void* stream);

/*
 * Repeated JVPs at one state, the split jax.linearize makes
 * (spectrax/midpoint_solver.py:75: linearise once per Newton iteration, then one
 * product per GMRES iteration).  spx_linearize stores in `lin`
 * (spx_linearize_bytes() bytes, 16-byte aligned) what J(y) v needs from y: the
 * real-space Hermite planes and field combinations of y and the six bracket sums
 * of every plane on the general layout (saving one inverse transform per plane
 * and half of the bracket arithmetic in every later product), a copy of y on
 * the 1D1V layout.  `lin` no longer refers to y.  spx_jvp_lin then returns
 * J(y) v bit for bit as spx_jvp(y, v) would; `ws` as for spx_jvp.
 */
size_t spx_linearize_bytes(const spx_plan* plan);
int spx_linearize(const spx_plan* plan, const void* y, void* lin, size_t lin_bytes, void* stream);
int spx_jvp_lin(const spx_plan* plan, const void* lin, const void* v, void* Jv, void* ws,
                size_t ws_bytes, void* stream);

/*
 * out[n * nv + j] = H_n(xi[j]) / (sqrt(pi) 2^(n/2) sqrt(n!)) for n < N: the
 * per-axis Hermite basis of the f(x, v) reconstruction in
 * spectrax/_inverse_transform.py:79-84 (xi and out device arrays), by the
 * recurrence of the normalised Hermite functions (finite for every n).
 */
int spx_hermite_basis(int32_t N, const double* xi, int64_t nv, double* out, void* stream);
/*
 * f(x, v) of spectrax/_inverse_transform.py:97-125 for `nlead` sets of coefficient
 * planes Ck (nlead x Nn*Nm*Np planes, centred order, complex128, device):
 * f[(l, point), v] = exp(-|xi_v|^2) sum_{n,m,p} C_l,(n,m,p)(point) bx[n, v] by[m, v] bz[p, v]
 * with C = Re ifftn(ifftshift(Ck)) (1/N).  The plan: one species, every Fourier mode
 * kept (cut >= N/2 on every axis).  bx, by, bz: (Nn | Nm | Np) x nv per-axis bases
 * (spx_hermite_basis), xi: 3 x nv (xi_x, xi_y, xi_z), f: nlead*plane x nv, all on the
 * device; ws: spx_fxv_workspace_bytes(plan, nlead) bytes (the real-space planes).
 */
size_t spx_fxv_workspace_bytes(const spx_plan* plan, int64_t nlead);
int spx_fxv(const spx_plan* plan, const void* Ck, int64_t nlead, const double* bx, const double* by, const double* bz,
            const double* xi, int64_t nv, double* f, void* ws, size_t ws_bytes, void* stream);

/*
 * Initial Hermite-Fourier coefficients of drifting Maxwellians on the device
 * (spectrax/_initialize_maxwellian.py:15-66): for every species s and Hermite
 * mode (n, m, p) of the plan, fftshift(fftn(C, norm="forward")) over (y, x, z) of
 *   C(x) = sqrt(2^(n+m+p) / (n! m! p!)) / (a_x^(n+1) a_y^(m+1) a_z^(p+1))
 *          (U_x - u_x)^n (U_y - u_y)^m (U_z - u_z)^p,
 * with a, u the plan's alpha_s, u_s and Us (device, Ns x 3 x Ny x Nx x Nz
 * doubles) the sampled bulk velocities; then the same transform of `nreal`
 * extra real planes xreal (device, nreal x plane; e.g. the fields E, B).
 * out (device) gets Ns*Nn*Nm*Np + nreal planes of complex128 in the state's
 * order.  The plan must keep every Fourier mode (cut >= N/2 on every axis).
 */
int spx_maxwellian(const spx_plan* plan, const double* Us, const double* xreal, int32_t nreal, void* out,
                   void* stream);

/*
 * Krylov-basis kernels of the implicit midpoint's restarted GMRES (the reference
 * uses jax.scipy's GMRES, spectrax/midpoint_solver.py:37-98).  V: device basis of
 * rows of n complex128 entries (row i at V + i*n); only rows i < k are read.
 * spx_krylov_cgs2: classical Gram-Schmidt with one re-orthogonalisation pass,
 *   h = V[:k]^H w, w -= V[:k]^T h, h2 = V[:k]^H w, w -= V[:k]^T h2;
 *   writes out[i] = h[i] + h2[i] (i < k) and out[k] = (||w||_2, 0) (device,
 *   k + 1 complex128); ws holds spx_krylov_ws_bytes(n) bytes.  Sums in a fixed
 *   order (deterministic).
 * spx_krylov_axpy: x += sum_{i<k} c[i] V_i (c: k complex128 on the device).
 */
#define SPX_KRYLOV_MAX_ROWS 64
size_t spx_krylov_ws_bytes(int64_t n);
int spx_krylov_cgs2(const void* V, int64_t n, int32_t k, void* w, void* out, void* ws, size_t ws_bytes,
                    void* stream);
int spx_krylov_axpy(const void* V, int64_t n, int32_t k, const void* c, void* x, void* stream);
/*
 * Implicit-midpoint Newton glue (spectrax/midpoint_solver.py:44-53), one pass each:
 * spx_midpoint_residual: r = y1 - y0 - dt f (stored when r != NULL) and, on the
 *   device, sums[0] = sum |r / (atol + rtol max(|y0|, |y1|))|^2, sums[1] = the
 *   number of non-finite entries of r (fixed-order reduction; ws as for
 *   spx_krylov_cgs2).  f = f(y_mid): the Newton residual, whose scaled 2-norm
 *   decides convergence; f = f(y0): the error estimate y1 - y1_init of the
 *   adaptive step controller.
 * spx_midpoint_update: y1 += sign * delta (delta may be NULL), ymid = (y0 + y1) / 2.
 */
int spx_midpoint_residual(int64_t n, const void* y0, const void* y1, const void* f, double dt, double rtol,
                          double atol, void* r, double* sums, void* ws, size_t ws_bytes, void* stream);
int spx_midpoint_update(int64_t n, const void* y0, void* y1, const void* delta, double sign, void* ymid,
                        void* stream);

/*
 * g = J(y)^T w (plain transpose, no conjugation): the vector-Jacobian product of
 * the holomorphic right-hand side.  conj(J^T conj(w)) = J^H w is what
 * torch autograd needs; the Python layer applies the conjugations.  Every
 * layout: 1D1V (two launches) and the general 2-D / 3-D one (three launches:
 * real-space planes of y and forward transforms of w, the real-space field
 * gradients, then one block per Hermite plane and per field component).
 * ws as for spx_rhs (spx_rhs_workspace_bytes).
 */
int spx_vjp(const spx_plan* plan, const void* y, const void* w, void* g, void* ws,
            size_t ws_bytes, void* stream);

/*
 * Allocation-free g = J(y)^T w for the 1D1V layout (no counterpart in the
 * reference).  For callers that cannot allocate device memory where they need
 * the VJP — inside a CUDA stream capture, in real-time loops that must not
 * allocate after start-up, or under a host framework that owns every device
 * byte — this variant keeps spx_vjp's scratch (the per-tile partial sums of the
 * field gradient) in a fixed file-scope device array of
 * SPX_VJP_NOALLOC_MAX_ENTRIES complex128 values (1 MiB, held by every GPU that
 * loads the library until exit) and allocates nothing.  Problems needing more
 * than that (Ns * Hermite tiles * Nx entries) get SPX_E_UNSUPPORTED.  All calls
 * share the array: calls that overlap on the GPU race, so serialise them.  The
 * first call on a device looks up the array's address and should come before
 * any stream capture.  `plan` comes from spx_plan_create at set-up.
 */
#define SPX_VJP_NOALLOC_MAX_ENTRIES 65536
int spx_vjp_noalloc(const spx_plan* plan, const void* y, const void* w, void* g, void* stream);

/* ------------------------------------------------------- adjoint building blocks */
/*
 * One fixed Prince-Dormand 8(7) step of size h from y (1D1V layout) that keeps
 * every stage input Ystages[j] (13 x state_len; Ystages[0] = y) and stage
 * derivative Kstages[j] = f(Ystages[j]) (13 x state_len), and writes
 * ynext = y + h sum_j b_j K_j.  y may be Ystages itself (no copy then).  The discrete adjoint linearises at the stage
 * inputs.  (The reference differentiates through diffeqsolve with jax.grad;
 * this is the device-side replacement of that forward recomputation.)
 */
int spx_rk_step_store(const spx_plan* plan, const void* y, double h, void* Ystages, void* Kstages,
                      void* ynext, void* stream);
/* The same with `hermitian` = 1 for an exactly Hermitian y (C(-k) == conj C(k) on
 * every line; odd Nx): packed real transforms, as the Dopri8 solver's
 * `hermitian` option uses, so the stage inputs match its forward solve.  Fails
 * with SPX_E_ARG on a plan whose wavenumber grid does not allow it. */
int spx_rk_step_store_ex(const spx_plan* plan, const void* y, double h, void* Ystages, void* Kstages,
                         void* ynext, int32_t hermitian, void* stream);
/* Status word of spx_rk_step_store since the last call (SPX_ST_RUNNING = 0: no
 * problem; SPX_ST_WAIT_TIMEOUT: a bounded wait for staged data gave up and the
 * outputs are invalid); reading it resets it.  Synchronises `stream`. */
int spx_rk_status(int32_t* status, void* stream);
/* out = sum_{i < nterms} coefs[i] * vecs[i] over len complex128 entries
 * (vecs: host array of device pointers, nterms <= 16; out may alias an input). */
int spx_lincomb(int64_t len, int32_t nterms, const void* const* vecs, const double* coefs, void* out,
                void* stream);
/*
 * acc[0] += Re sum_e g_e (d f/d nu)_e ; acc[1] += Re sum_e g_e (k d f/d k)_e (the parts
 * of f linear in the wavenumbers, with L = 2 pi / k) ; acc[2+s] += Re sum_e g_e
 * (d f / d u_x,s)_e, all at state y (1D1V layout; acc is a device array of
 * 2 + Ns doubles the caller zeroes).
 */
int spx_param_dots(const spx_plan* plan, const void* y, const void* g, double* acc, void* stream);
/* g = J(y)^T w together with acc[k] += Re sum_e w_e (df/dtheta_k)_e for
 * theta = (nu, k (as k d/dk), u_x of each species): spx_vjp and spx_param_dots
 * in one launch, the parameter sums added in a fixed order.  ws as for spx_rhs
 * (spx_rhs_workspace_bytes); 1D1V layout only.  On a plan with its own product
 * grid (spx_plan_product_grid != Nx) and 3K != Nx the transposed products run on
 * that grid, agreeing with the Nx-point grid to rounding.  Calls on one plan must
 * not run concurrently (the plan holds the kernel's completion ticket). */
int spx_vjp_param(const spx_plan* plan, const void* y, const void* w, void* g, double* acc, void* ws,
                  size_t ws_bytes, void* stream);
/* The same with `hermitian` = 1 for exactly Hermitian y and w: every real-space
 * line is real, two share one complex transform, only the k <= 0 half of each
 * output plane is evaluated and g is written exactly Hermitian. */
int spx_vjp_param_ex(const spx_plan* plan, const void* y, const void* w, void* g, double* acc, void* ws,
                     size_t ws_bytes, int32_t hermitian, void* stream);

/* ------------------------------------------------------------------ Dopri8 */
typedef struct spx_dopri8_opts {
  double t0, t1;     /* integration interval */
  double dt0;        /* first step (adaptive) or the constant step */
  double rtol, atol; /* PID controller tolerances (adaptive only) */
  int32_t adaptive;  /* 1: Diffrax PIDController defaults; 0: ConstantStepSize */
  int32_t nsave;     /* number of save times (may be 0) */
  const double* save_ts; /* host array of nsave increasing times in [t0, t1] */
  int64_t max_steps; /* accepted + rejected steps before SPX_ST_MAX_STEPS */
  int32_t save_states; /* 1: keep every saved state (nsave * state_len complex128) */
  const double* masses; /* host array of Ns species masses for the kinetic energy (NULL: ones);
                           spectrax/_diagnostics.py:44-68 uses (1, mi_me) for two species */
  int32_t hermitian;  /* 1: at reset, test y0 for exact Hermitian symmetry (C(-k) == conj C(k)
                           bit for bit, every plane) on the fused 1D1V path with odd Nx; when it
                           holds, evaluate stages with packed real transforms (half the FFTs).
                           The symmetry is then kept exactly by every stage.  0: never. */
  int32_t persistent; /* 1: on the fused 1D1V path, run all attempts of a replay in one
                           cooperative launch whose CTAs chain stages through completion
                           counters (used when every CTA fits on the GPU at once, the
                           plan's product grid is Nx points and saveat is 1); 0: one launch
                           per stage. */
  int32_t saveat;     /* 0: Diffrax SaveAt(ts) -- steps end only on t1 and a save time inside
                           an accepted step gets the step's dense output (a degree-8
                           continuous extension of the 13 stages: order 4, order 8 on linear
                           problems); 1: every step is shortened to end on the next save
                           time, which then gets the step's 8th-order solution. */
} spx_dopri8_opts;

typedef struct spx_dopri8 spx_dopri8;   /* opaque: stage buffers + CUDA graph */

/* Device-side counters of a solve, copied out by spx_dopri8_stats. */
typedef struct spx_dopri8_stats {
  double t, dt;
  int64_t accepted, rejected, rhs_evals;
  int32_t status, saved;
  int32_t hermitian;  /* 1 if the packed real-transform stages are in use */
  int32_t persistent; /* 1 if attempts run in the persistent cooperative kernel */
} spx_dopri8_stats;

/*
 * Adaptive / constant-step Prince-Dormand 8(7) solve of y' = f(t, y) on the
 * device, replacing the diffeqsolve call of spectrax/_simulation.py:164-180.
 * create() allocates the stage buffers and captures one step attempt as a CUDA
 * graph; run() replays it until the solve ends.
 */
int spx_dopri8_create(const spx_plan* plan, const spx_dopri8_opts* opts, spx_dopri8** out);
int spx_dopri8_destroy(spx_dopri8* s);
/* Fault-handling test hook (no counterpart in the reference).  The persistent
 * kernel's waits on other CTAs' completion counters give up after `polls` polls
 * (0: the default, about a second) and end the solve with SPX_ST_WAIT_TIMEOUT.
 * unreachable != 0 makes those waits ask for a count no CTA ever publishes, so
 * the first one runs out: a way to exercise the time-out path without a fault.
 * Each such wait sits between stages, when the CTA has no bulk copy in flight.
 * Takes effect at the next spx_dopri8_reset; affects only persistent solvers. */
int spx_dopri8_set_wait_test(spx_dopri8* s, int32_t polls, int32_t unreachable);
/* Copy y0 in (device memory or page-locked host memory) and reset the
 * clock/controller; stream-ordered, the host does not wait. */
int spx_dopri8_reset(spx_dopri8* s, const void* y0, void* stream);
/* Replay up to `max_attempts` step attempts (accepted or rejected); returns
 * after the solve ends or the attempts are used.  *status_out gets the status. */
int spx_dopri8_advance(spx_dopri8* s, int64_t max_attempts, void* stream, int32_t* status_out);
/* Enqueue exactly `attempts` step attempts on `stream` without waiting (attempts
 * after the end of the solve do nothing).  For timing and for callers that poll
 * the status themselves. */
int spx_dopri8_enqueue(spx_dopri8* s, int64_t attempts, void* stream);
/* Run to the end (advance in chunks until status != RUNNING). */
int spx_dopri8_run(spx_dopri8* s, void* stream, int32_t* status_out);
int spx_dopri8_stats_get(spx_dopri8* s, spx_dopri8_stats* out, void* stream);
/* Device pointers owned by the solver: current state, saved states
 * (nsave x state_len, or NULL), per-save energies (nsave x (2 + Ns) doubles:
 * EM_energy, kinetic_energy, kinetic_energy_species[0..Ns-1]). */
const void* spx_dopri8_state(spx_dopri8* s);
const void* spx_dopri8_saved_states(spx_dopri8* s);
const double* spx_dopri8_saved_energies(spx_dopri8* s);
/* Copy solver data to `dst` (host or device; cudaMemcpyDefault) on `stream`:
 * what = 0: current state (state_len complex128), 1: saved states
 * (nsave*state_len complex128), 2: saved energies (nsave*(2+Ns) doubles).
 * `bytes` must equal the size of that item. */
int spx_dopri8_copy(spx_dopri8* s, int32_t what, void* dst, size_t bytes, void* stream);

/* ------------------------------------------------------------------ batch */
/*
 * Many independent 1D1V instances (different Nx, Nn, Ns, L, nu, alpha, u),
 * each integrated by adaptive (or constant-step) Dopri8 to t1, all in ONE
 * persistent launch: each thread-block cluster of `cluster` CTAs takes the next
 * instance from a largest-first work queue.  Replaces the serial scan loop of
 * Examples/1D_Landau_damping_dr_curve.py:88-110 (one simulation() per k).
 * The launch is captured once as a CUDA graph.
 */
typedef struct spx_batch_opts {
  double t1, dt0, rtol, atol;
  int64_t max_steps;     /* per instance */
  int32_t adaptive;      /* 1: Diffrax PIDController defaults; 0: constant step dt0 */
  int32_t nsave;         /* shared save times (energies recorded at each) */
  const double* save_ts; /* host, nsave increasing times in [0, t1] */
  int32_t cluster;       /* CTAs per instance, 1..16 (above 8: non-portable cluster sizes) */
  int32_t tile;          /* Hermite planes per tile (0: 8; at most 32); -1: per instance, the
                            height whose tiles fill the fewest whole rounds of the cluster */
  const double* masses;  /* host, n x SPX_MAX_SPECIES species masses (NULL: ones) */
  int32_t hermitian;     /* 1: an instance with odd Nx whose initial state is exactly Hermitian
                            (C(-k) == conj C(k) on every line) uses packed real transforms */
  int32_t saveat;        /* as spx_dopri8_opts.saveat: 0 dense output at save times, 1 land on them */
  const double* costs;   /* host, n relative costs ordering the work queue (largest first), e.g.
                            durations measured on a short horizon; NULL: an estimate from the
                            FFT work per evaluation and the stability-limited step count */
} spx_batch_opts;

typedef struct spx_batch_stats {
  double t, dt;
  int64_t accepted, rejected, rhs_evals;
  int32_t status, saved;
  int32_t hermitian;     /* 1 if the instance ran with packed real transforms */
  int32_t pad;
  double start_s, end_s; /* when its cluster took and finished it, seconds after the first start */
} spx_batch_stats;

typedef struct spx_batch spx_batch;

int spx_batch_create(int32_t n, const spx_problem* problems, const spx_batch_opts* opts, spx_batch** out);
int spx_batch_destroy(spx_batch* b);
/* Offset (complex128 entries) of instance i in the packed state arrays; i = n gives the total. */
int64_t spx_batch_offset(const spx_batch* b, int32_t i);
/* Offset (doubles) of instance i in the packed energies (nsave x (2 + Ns) per instance). */
int32_t spx_batch_energy_offset(const spx_batch* b, int32_t i);
/* CTAs of the persistent grid. */
int32_t spx_batch_grid(const spx_batch* b);
/* Copy the packed initial states in (host or device), replay the graph, copy the
 * packed final states out (if y_final is not NULL).  Asynchronous on `stream`. */
int spx_batch_run(spx_batch* b, const void* y0, void* y_final, void* stream);
/* Per-instance counters (host array of n, synchronises) and packed energies
 * (host or device, may be NULL). */
int spx_batch_results(spx_batch* b, spx_batch_stats* stats, double* energies, void* stream);

/* ------------------------------------------------------------ measurement */
/*
 * FP64 issue-rate probe (no counterpart in the reference): `blocks` CTAs of 256
 * threads each run 8 independent FMA chains of `iters` steps and write one
 * double per thread to `out` (device, blocks*256 doubles).  Timed by the caller;
 * FLOP/s = 16 * iters * blocks * 256 / seconds.  Used as the compute roofline.
 */
int spx_probe_fp64(void* out, int blocks, int iters, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SPECTRAX_GB300_H */
