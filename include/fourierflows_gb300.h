/*
 * libfourierflows_gb300 -- C ABI of the GB300 (sm_103a) pseudospectral time-stepping path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream handle
 * (cudaStream_t passed as void*, NULL = legacy default stream) and returns an int status
 * (FF_OK = 0).  On failure ff_last_error() returns a message for the calling thread.
 * Nothing here synchronises the stream unless it returns a host scalar (the Parseval
 * reductions), mirroring the reference, whose GPU reductions return host numbers.
 *
 * Layout is the reference's (Julia, column-major): the first index is fastest.  A 2D
 * real field is (nx, ny), its real transform (nkr, ny) with nkr = nx/2 + 1; complex
 * numbers are interleaved (re, im) doubles (FF_F64) or floats (FF_F32).  Arrays beyond
 * the grid's dimensions (fields, ensemble members) are trailing "batch" dimensions.
 *
 * Citations are FourierFlows.jl source lines (path:line) of the interface each entry
 * point replaces.
 */
#ifndef FOURIERFLOWS_GB300_H
#define FOURIERFLOWS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define FF_OK 0
#define FF_ERR_ARG 1         /* bad argument (shape, size, pointer, alignment)           */
#define FF_ERR_CUDA 2        /* a CUDA runtime call failed                                */
#define FF_ERR_UNSUPPORTED 3 /* valid request this build does not implement (e.g. radix) */
#define FF_ERR_ALLOC 4       /* device allocation failed                                 */
#define FF_ERR_TIMEOUT 5     /* a bounded device-side wait gave up                       */

/* ---- precisions ---------------------------------------------------------------------- */
#define FF_F64 0
#define FF_F32 1

/* ---- coefficient descriptors --------------------------------------------------------- */
/* A per-mode coefficient such as the linear operator L of Equation(L, calcN!, grid)
 * (src/problem.jl:11-34): absent, a real or complex device array with one entry per
 * state element, or a scalar (Diffusion with varying kappa uses L = 0,
 * src/diffusion.jl:89-90).  Arrays are in the state's precision unless stated. */
#define FF_COEF_NONE 0
#define FF_COEF_REAL 1
#define FF_COEF_COMPLEX 2
#define FF_COEF_SCALAR 3 /* re (+ i im) */

typedef struct {
  const void* ptr;
  int32_t kind;
  int32_t pad_;
  double re;
  double im;
} ff_coef;

/* ---- library ------------------------------------------------------------------------- */
int ff_version(void);                       /* (major << 16) | (minor << 8) | patch        */
int ff_last_error(char* buf, size_t len);   /* copies the calling thread's last message   */

/* FP64 FMA throughput of the current device (TFLOP/s, one timed launch): the ceiling of
 * the FP64 transforms, which on this part are FP64-pipe bound rather than HBM bound. */
int ff_fp64_peak(double* tflops, void* stream);

/* ---- FFT plans ----------------------------------------------------------------------- */
typedef struct ff_plan ff_plan;

/* Real-to-complex plan over all ndim (1..3) dimensions n[0..ndim-1], applied to `batch`
 * consecutive arrays.  Replaces plan_flows_rfft (src/domains.jl:3,5) as built by the
 * grid constructors (src/domains.jl:87,208,349).  Every n must be even in dimension 0
 * (odd sizes are rejected by the grids, src/domains.jl:66,179,316) and factor into
 * primes <= 31 in every dimension, with n[d] <= 4096 (FF_F64) or 8192 (FF_F32). */
int ff_plan_create(int ndim, const int64_t n[3], int prec, int64_t batch, ff_plan** plan);

/* Complex-to-complex plan; replaces plan_flows_fft (src/domains.jl:2,4,86,207,348). */
int ff_cplan_create(int ndim, const int64_t n[3], int prec, int64_t batch, ff_plan** plan);

int ff_plan_destroy(ff_plan* plan);

/* mul!(out, rfftplan, in): unnormalised forward transform, exp(-i k x) (src/diffusion.jl:139,171). */
int ff_rfft(const ff_plan* plan, const void* in_real, void* out_complex, void* stream);

/* ldiv!(out, rfftplan, in): inverse normalised by 1/(nx ny nz) (src/diffusion.jl:137,154-155).
 * Unlike FFTW's c2r it never modifies its input. */
int ff_irfft(const ff_plan* plan, const void* in_complex, void* out_real, void* stream);

/* mul!/ldiv! with the complex plan; in == out is allowed. */
int ff_fft(const ff_plan* plan, const void* in, void* out, void* stream);
int ff_ifft(const ff_plan* plan, const void* in, void* out, void* stream);

/* ---- dealias! (src/domains.jl:428-476) ------------------------------------------------ */
/* Zero the index ranges [lo[d], hi[d]) (0-based, lo >= hi = empty) along dimension d of
 * the array fh of complex size dims[0] x dims[1] x dims[2] x dims[3] (dims[3] = batch). */
int ff_dealias(int prec, void* fh, const int64_t dims[4], const int64_t lo[3], const int64_t hi[3],
               void* stream);

/* ---- fused time-stepper substeps (src/timesteppers.jl) --------------------------------- */
/* All act elementwise on n complex values; `filter` is a real array (state precision) or
 * NULL; each is one pass over HBM.                                                       */

/* ForwardEuler / FilteredForwardEuler update (src/timesteppers.jl:113,144):
 *   sol = [filter *] (sol + dt (L sol + N)) */
int ff_euler_update(int prec, int64_t n, void* sol, const void* N, ff_coef L, double dt, const void* filter,
                    void* stream);

/* RK4 addlinearterm! + substepsol! (src/timesteppers.jl:225-235,239-255):
 *   RHS += L x;   if newsol: newsol = sol + c RHS          (x may alias newsol) */
int ff_rk4_substep(int prec, int64_t n, void* RHS, ff_coef L, const void* x, const void* sol, void* newsol,
                   double c, void* stream);

/* last RK4 substep + RK4update! (+ filter) (src/timesteppers.jl:255,260-262,279):
 *   RHS4 += L x;  sol = [filter *] (sol + c6 (RHS1 + 2 RHS2 + 2 RHS3 + RHS4)),
 * c6 = dt/6 rounded to the state precision as the reference computes it. */
int ff_rk4_update(int prec, int64_t n, void* sol, void* RHS4, ff_coef L, const void* x, const void* RHS1,
                  const void* RHS2, const void* RHS3, double c6, const void* filter, void* stream);

/* one LSRK54 stage (src/timesteppers.jl:383-395, + filter :408 when filter != NULL):
 *   RHS += L sol;  S2 = A S2 + dt RHS (S2 = dt RHS if first);  sol = [filter *](sol + B S2) */
int ff_lsrk54_stage(int prec, int64_t n, void* sol, void* RHS, void* S2, ff_coef L, double A, double B,
                    double dt, int first, const void* filter, void* stream);

/* nsteps whole steps of a linear equation (N = 0, as the Diffusion module's calcN! gives
 * for constant kappa, src/diffusion.jl:129-133) in one pass over the state.
 * stepper FF_STEP_ETDRK4: c = exp(L dt); each step is sol = [filter *] (c sol), which is
 *   what ETDRK4substeps! + ETDRK4update! (src/timesteppers.jl:501-547,552) compute when
 *   N1..N4 are zero.
 * stepper FF_STEP_RK4: c = L; each step runs RK4's four stages with N = 0 in the order of
 *   ff_rk4_substep / ff_rk4_update (src/timesteppers.jl:225-285), + filter.
 * The stepper's intermediate buffers (sol1, N1, ...) are neither read nor written. */
int ff_linear_step(int prec, int stepper, int64_t n, void* sol, ff_coef c, double dt, const void* filter,
                   int64_t nsteps, void* stream);

/* ETDRK4substep12! (src/timesteppers.jl:506-510): out = e_half sol + zeta N */
int ff_etdrk4_substep12(int prec, int64_t n, void* out, ff_coef e_half, const void* sol, ff_coef zeta,
                        const void* N, void* stream);

/* ETDRK4substep3! (src/timesteppers.jl:512-516): out = e_half sol1 + zeta (2 N3 - N1) */
int ff_etdrk4_substep3(int prec, int64_t n, void* out, ff_coef e_half, const void* sol1, ff_coef zeta,
                       const void* N1, const void* N3, void* stream);

/* ETDRK4update! (+ filter) (src/timesteppers.jl:501-504,552):
 *   sol = [filter *] (expL sol + alpha N1 + 2 beta (N2 + N3) + Gamma N4) */
int ff_etdrk4_update(int prec, int64_t n, void* sol, ff_coef expL, ff_coef alpha, ff_coef beta, ff_coef Gamma,
                     const void* N1, const void* N2, const void* N3, const void* N4, const void* filter,
                     void* stream);

/* AB3 step (src/timesteppers.jl:628-651,658): RHS += L sol; sol += dt RHS (euler != 0) or
 * dt (23/12 RHS - 16/12 RHSm1 + 5/12 RHSm2); [sol *= filter]; RHSm2 = RHSm1; RHSm1 = RHS */
int ff_ab3_update(int prec, int64_t n, void* sol, void* RHS, void* RHSm1, void* RHSm2, ff_coef L, double dt,
                  int euler, const void* filter, void* stream);

/* The ETDRK4 coefficients zeta, alpha, beta, Gamma of a real linear operator L (n values,
 * state precision) for step dt, by the ncirc-point contour means of getetdcoeffs
 * (src/timesteppers.jl:689-718, ncirc = 32, rcirc = 1 there), evaluated in FP64 on the
 * device and rounded to the state precision.  Used to set up large ensembles; the
 * drop-in ETDRK4TimeStepper computes them on the host as the reference does. */
int ff_etdrk4_coefficients(int prec, int64_t n, const void* L, double dt, int ncirc, double rcirc, void* zeta,
                           void* alpha, void* beta, void* gamma, void* stream);

/* sol .*= filter (src/timesteppers.jl:279,408,552,658) */
int ff_filter_mul(int prec, int64_t n, void* sol, const void* filter, void* stream);

/* ---- spectral helpers ------------------------------------------------------------------ */
/* out = i k in, k broadcast along dimension 0 (k has n0 entries), the pattern of
 * `@. cxh = im * kr * sol` (src/diffusion.jl:136,140,154).  out may alias in. */
int ff_mul_ik(int prec, int64_t n0, int64_t nrest, void* out, const void* in, const void* k, void* stream);

/* x .*= a for real arrays of n elements, a real array of n or of n0 (broadcast along
 * the trailing dimensions) -- `@. cx *= kappa` (src/diffusion.jl:138). */
int ff_real_mul(int prec, int64_t n, int64_t na, void* x, const void* a, void* stream);

/* parsevalsum2 / parsevalsum (src/utils.jl:113-183).  uh has n0 x nrest complex values;
 * rfft_form != 0 counts rows 1..n0-2 twice (conjugate-symmetric half spectrum).  The
 * result times `norm` is written to *out (host memory); the stream is synchronised. */
int ff_parsevalsum2(int prec, const void* uh, int64_t n0, int64_t nrest, int rfft_form, double norm,
                    double* out, void* stream);
int ff_parsevalsum(int prec, const void* uh, int64_t n0, int64_t nrest, int rfft_form, double norm,
                   double* out, void* stream);

/* parsevalsum2 of uh .* sqrt(wt) for a real weight array wt (NULL = 1), e.g. the energy
 * 1/2 parsevalsum2(zeta_hat sqrt(invKrsq)) / (Lx Ly) with wt = invKrsq.  With dev_out
 * non-NULL the result goes to that device double and nothing synchronises (the
 * diagnostic can be recorded inside a captured step); otherwise *out as above. */
int ff_parsevalsum2_weighted(int prec, const void* uh, const void* wt, int64_t n0, int64_t nrest, int rfft_form,
                             double norm, double* out, double* dev_out, void* stream);

/* radialspectrum(fh, grid; n, m) (src/utils.jl:239-283) for a TwoDGrid nk x nl with
 * domain Lx x Ly: fh is (n0, nl) with n0 = nk/2 + 1 (conjugate-symmetric form, angles
 * in [-pi/2, pi/2]) or n0 = nk (full form, angles in [0, 2 pi]), real or complex
 * (is_complex) in the given precision.  out[i] = [2] rho_i sum_j fh(rho_i, theta_j)
 * dtheta over `ntheta` angles (the reference's m, halved for the conjugate-symmetric
 * form), rho_i = i rhomax / (nrho - 1), rhomax = min((nk/2 - 1) 2pi/Lx, (nl/2 - 1)
 * 2pi/Ly), with fh bilinearly interpolated from its fftshifted layout; out[0] = fh[0].
 * out has nrho elements of fh's type; sums are FP64. */
int ff_radialspectrum(int prec, int is_complex, const void* fh, int64_t n0, int64_t nk, int64_t nl, double Lx,
                      double Ly, int64_t nrho, int64_t ntheta, void* out, void* stream);

/* parsevalsum2 that allocates no device memory.  No counterpart in the reference: it
 * serves callers that cannot call cudaMalloc because another allocator owns the GPU's
 * memory (a pooling allocator that has reserved it, or a fixed-budget embedded code).
 * The caller passes uh and a device double `out` (written on `stream`, no host
 * synchronisation); the scratch is a 32 KiB static device array, so n0 * nrest is limited
 * to 33,554,432 modes (larger sizes return FF_ERR_ARG).  The first call in each CUDA
 * context looks up that array's device address (cached by the context's unique ID, so
 * a device reset or a re-created primary context looks it up again); make that first
 * call before any stream capture.  All calls share the array: calls that overlap on the
 * GPU race. */
int ff_parsevalsum2_noalloc(int prec, const void* uh, int64_t n0, int64_t nrest, int rfft_form, double norm,
                            double* out, void* stream);

/* u_hat = -i l psi_hat, v_hat = i kr psi_hat with psi_hat = -zeta_hat invKrsq on the
 * (nkr, ny) half spectrum: the velocity spectra of a vorticity field. */
int ff_vort_velocities(int prec, int64_t nkr, int64_t ny, const void* zh, const void* kr, const void* l,
                       const void* invKrsq, void* uh, void* vh, void* stream);

/* ---- fused 2D vorticity steppers ------------------------------------------------------- */
/* The nonlinear term N = -J(psi, zeta), psi_hat = -zeta_hat / |k|^2, of the 2D vorticity
 * equation, with 2/3 dealiasing of its input and output, fused with the substeps of a
 * time stepper.  The reference's call stack it replaces is stepforward!(prob) ->
 * ETDRK4substeps! / RK4substeps! / LSRK54update! (src/timesteppers.jl:518-547,237-274,
 * 383-404) -> the user calcN! built on jacobianh (src/utils.jl:190-205), rfftplan
 * mul!/ldiv! and dealias! (src/domains.jl:428-476).  One handle advances one problem or
 * an ensemble of problems of different sizes; every substep is three persistent
 * launches over all problems, and a step is replayed from a captured CUDA graph. */
typedef struct ff_vort ff_vort;

#define FF_STEP_ETDRK4 0
#define FF_STEP_RK4 1
#define FF_STEP_LSRK54 2

typedef struct {
  int64_t nx, ny;       /* physical grid; nkr = nx/2 + 1                                    */
  int64_t nkd;          /* kept kr columns [0, nkd): the first of kralias, or nkr if none   */
  int64_t la, lb;       /* aliased l rows [la, lb) (0-based lalias); la == lb: none         */
  const void* kr;       /* nkr wavenumbers (state precision)                                 */
  const void* l;        /* ny wavenumbers                                                    */
  const void* invKrsq;  /* nkr*ny, 1/(kr^2 + l^2) with the mean mode 0                       */
  void* sol;            /* nkr*ny complex state, advanced in place                           */
  void* buf[5];         /* ETDRK4: sol1, sol2, N1, N2, N3; RK4: sol1, RHS1, RHS2, RHS3;
                           LSRK54: S2 -- nkr*ny complex each, owned by the caller            */
  const void* coef[6];  /* ETDRK4: expLdt, exp_half_Ldt, zeta, alpha, beta, Gamma;
                           RK4 / LSRK54: L -- nkr*ny real arrays (state precision)           */
  const void* filter;   /* nkr*ny real filter of the Filtered* steppers, or NULL             */
  double lsrk_A[5];     /* LSRK54 coefficients in the state precision (problem 0 is used)    */
  double lsrk_B[5];
} ff_vort_problem;

/* Create a fused stepper for nprob problems (all of precision prec and one stepper kind).
 * `filtered` applies each problem's filter at the end of the step as the Filtered*
 * steppers do (src/timesteppers.jl:279,408,552).  The pointers in probs must stay valid
 * for the handle's lifetime.  kr and l are read once here (and again by set_split and
 * autotune) into scaled copies: like the grid they come from, they must not change. */
int ff_vort_create(int prec, int stepper, int filtered, double dt, int64_t nprob, const ff_vort_problem* probs,
                   ff_vort** out);
int ff_vort_destroy(ff_vort* h);

/* Advance every problem nsteps steps on `stream` (no host synchronisation).  The first
 * call captures a CUDA graph of one step (set FF_NO_GRAPH=1 to launch kernels directly). */
int ff_vort_step(ff_vort* h, int64_t nsteps, void* stream);

/* The bare nonlinear term N = calcN!(sol) of problem `prob` (nkr*ny complex each).
 * Each call stages its descriptor and work lists through one buffer of the handle and
 * uses the handle's workspace, so calls on one handle must be serialised on one stream
 * (as ff_vort_step's are); concurrent calls need separate handles. */
int ff_vort_calcN(ff_vort* h, int64_t prob, const void* sol, void* N, void* stream);

/* ff_vort_calcN with its descriptor staged once.  bind stores problem `prob`'s descriptor,
 * work lists and the (sol, N) pointers in slot `slot` (0 .. FF_VORT_CALC_SLOTS-1; it
 * synchronises the device, so not during stream capture); calcN_slot launches the three
 * passes of a bound slot with no host staging, so it can be captured in a CUDA graph (a
 * checkpointed adjoint replays one per step).  A later set_config, set_split or autotune
 * invalidates the slots: calcN_slot then fails until they are bound again.  Binding a slot
 * again frees its previous staging buffer, so a CUDA graph that captured calcN_slot on it
 * must not be replayed after that.  The same serialisation rule as ff_vort_calcN applies
 * (the handle's workspace). */
#define FF_VORT_CALC_SLOTS 16
int ff_vort_calcN_bind(ff_vort* h, int slot, int64_t prob, const void* sol, void* N);
int ff_vort_calcN_slot(ff_vort* h, int slot, void* stream);

/* Average device time (ms) of each of the three passes over `reps` launches, timed with
 * CUDA events on `stream`: ms = {A, B, C}; C runs as in the first substep (its epilogue
 * writes only the stepper's intermediate buffers).  ETDRK4 and RK4 handles only
 * (FF_ERR_UNSUPPORTED otherwise: an LSRK54 stage advances the state). */
int ff_vort_profile(ff_vort* h, int reps, void* stream, double ms[3]);


/* ---- discrete adjoint of the 2D vorticity term and of an ETDRK4 step -------------------- */
/* No counterpart in FourierFlows.jl (whose gradients would come from an AD system through
 * `stepforward!`); these serve a ChainRulesCore `rrule` for stepforward! over the fused
 * vorticity step.  The state is the stored half spectrum read as a real vector of its
 * real and imaginary parts (inner product sum Re(conj(a) b)). */
typedef struct ff_vadj ff_vadj;

int ff_vadj_create(int prec, int64_t nx, int64_t ny, int64_t nkd, int64_t la, int64_t lb, const void* kr,
                   const void* l, const void* invKrsq, ff_vadj** out);
int ff_vadj_destroy(ff_vadj* h);

/* out = J(s)^T lam: the transpose of the linearisation of N at state s applied to lam
 * (nkr*ny complex each; out may alias lam). */
int ff_vadj_apply(ff_vadj* h, const void* s, const void* lam, void* out, void* stream);

/* Arrays of one adjoint ETDRK4 step: the adjoints of the new state and of sol1 (a), of
 * the first sol2 (b) and of the second sol2 (c); the step's s, a and N1..N4; and the
 * derivatives with respect to the viscosity of expLdt, exp_half_Ldt, zeta, alpha, beta and
 * Gamma (real arrays). */
typedef struct {
  const void *lam, *lam_a, *lam_b, *lam_c, *s, *a, *n1, *n2, *n3, *n4;
  const void *dE, *dE2, *dZ, *dA, *dB, *dG;
} ff_adj_nu;

/* *dev_acc += scale * d(step)/d(nu) contracted with the adjoints, accumulated in FP64 on
 * the device (no host synchronisation). */
int ff_vort_adj_nu_terms(ff_vadj* h, const ff_adj_nu* args, double scale, double* dev_acc, void* stream);

/* Launch geometry: cfg = {tile A, tile C, rows B, radix order, threads A, B, C, graph};
 * radix order -1 marks the register-resident power-of-two path.  set_config's
 * radix_variant (0..2) picks the generic path's radix order. */
int ff_vort_config(const ff_vort* h, int32_t cfg[8]);
int ff_vort_set_config(ff_vort* h, int tla, int tlc, int tlr, int radix_variant);

/* Pass C split by field (register path, where pass C does not also run the next pass A):
 * two work items per kept column tile, one per transformed field, the second to finish
 * running the epilogue; for grids with few kept column tiles per SM.  mode -1 lets the
 * library decide from the tile count (the default), 0 and 1 turn it off and on;
 * get_split reports whether the current geometry uses it.  It forms the flux by the
 * unsplit form's formula in another kernel, whose compiled arithmetic may round
 * differently in the last bit. */
int ff_vort_set_split(ff_vort* h, int mode);
int ff_vort_get_split(const ff_vort* h, int32_t* on);

/* Time every tile / radix-order (and split) candidate for `steps_per_trial` steps and keep
 * the fastest; the trial steps advance the state, so pass scratch states or restore them. */
int ff_vort_autotune(ff_vort* h, int steps_per_trial, void* stream, double* best_ms);

#ifdef __cplusplus
}
#endif

#endif /* FOURIERFLOWS_GB300_H */
