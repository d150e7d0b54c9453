/*
 * gbspec.h — C ABI of libgbspec, the GB300 (sm_103a) pseudo-spectral time
 * step behind fluidsim's fluidfft plugin / operator / time-stepping API.
 *
 * Conventions
 *   - Every entry point returns 0 on success or a negative errno-like code
 *     (GBS_E*); gbs_last_error() gives a message for the calling thread.
 *     No C++ exception crosses this boundary.
 *   - Arrays are device pointers, C order, in fluidfft's sequential layout:
 *       physical  (nz, ny, nx)        / (ny, nx)          real
 *       spectral  (nz, ny, nx/2 + 1)  / (ny, nx/2 + 1)    complex (re, im)
 *     with `batch` (or nvar) such fields stored back to back.
 *   - dtype GBS_F64: double / complex128;  GBS_F32: float / complex64.
 *   - The forward transform is divided by the number of points, the
 *     inverse is not normalised (fluidsim/base/state.py:385-392).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous unless stated; plans / solvers own their workspaces and
 *     allocate nothing after creation.  A handle is not re-entrant; distinct
 *     handles are independent.
 */
#ifndef GBSPEC_H
#define GBSPEC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBS_OK 0
#define GBS_EINVAL (-22) /* bad argument (maps to ValueError)            */
#define GBS_ENOMEM (-12) /* device allocation failed (MemoryError)       */
#define GBS_ECUDA (-5)   /* CUDA runtime error (RuntimeError)            */
#define GBS_ENAN (-33)   /* NaN in the state after a step (ValueError)   */
#define GBS_ETIMEDOUT (-110) /* a bounded device-side wait ran out (RuntimeError) */

#define GBS_F32 0
#define GBS_F64 1

typedef struct gbs_fft_plan gbs_fft_plan;
typedef struct gbs_ns gbs_ns;

/* Message describing the last error on the calling thread ("" if none). */
const char* gbs_last_error(void);

/* Library version string. */
const char* gbs_version(void);

/* ------------------------------------------------------------- FFT plans
 * Replaces the fluidfft fft2d/fft3d class constructor and transforms
 * (fluidfft 0.4.2, selected at fluidsim/operators/operators3d.py:222-231 and
 * operators2d.py:137-144; called as oper.fft_as_arg / ifft_as_arg /
 * ifft_as_arg_destroy, e.g. fluidsim/solvers/ns3d/solver.py:210-241).
 * shapeX = (nz, ny, nx) for ndim 3, (ny, nx) for ndim 2; nx must be even.
 */
int gbs_fft_plan_create(int ndim, const int64_t* shapeX, int dtype, int batch,
                        gbs_fft_plan** plan);
int gbs_fft_plan_destroy(gbs_fft_plan* plan);

/* fft_as_arg: k = rfftn(x) / N for each of `batch` fields. */
int gbs_fft_r2c(gbs_fft_plan* plan, const void* x, void* k, void* stream);

/* ifft_as_arg (may_destroy = 0: k is preserved, the plan workspace is used)
 * and ifft_as_arg_destroy (may_destroy = 1: k is used as workspace). */
int gbs_fft_c2r(gbs_fft_plan* plan, void* k, void* x, int may_destroy,
                void* stream);

/* ifft_as_arg without any device allocation (no counterpart in the
 * reference: fluidfft always works on preallocated plan buffers).  For
 * callers that cannot allocate device memory themselves or let a library
 * do it (e.g. an application whose device memory is reserved up front by
 * its own pool allocator).  Same result as gbs_fft_c2r(may_destroy = 0) on
 * a plan of this shape; k is preserved.  Twiddles and workspace live in one
 * static 32 MiB device array that every GPU loading the library holds until
 * exit; shapes needing more (3*align256 twiddle tables + batch * nK
 * complex) are rejected with GBS_EINVAL.  The first call on a device (and
 * the first after a cudaDeviceReset) looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  Under lazy module loading (the CUDA default) that first call is
 * also where the driver allocates the 32 MiB array: make one small call on
 * each device before a pool takes all device memory, or set
 * CUDA_MODULE_LOADING=EAGER.  All calls share the array: calls whose GPU
 * work overlaps race. */
int gbs_fft_c2r_noalloc(int ndim, const int64_t* shapeX, int dtype, int batch,
                        const void* k, void* x, void* stream);

/* ----------------------------------------------------- ns2d / ns3d solver
 * Parameters of the fused pseudo-spectral step.  ndim 2: ns2d (one state
 * variable rot_fft, fluidsim/solvers/ns2d/solver.py:111-194); ndim 3: ns3d
 * (vx_fft, vy_fft, vz_fft, fluidsim/solvers/ns3d/solver.py:180-263).
 * Dissipation sigma(k) = nu_2 k^2 + nu_4 k^4 + nu_8 k^8 (+ nu_m4 / k^4)
 * as fluidsim/base/solvers/pseudo_spect.py:134-191.
 * Cubic dealiasing removes modes with |k_adim| >= kcut_* along any axis
 * (kcut = n: nothing removed along that axis).
 */
typedef struct gbs_ns_params {
  int ndim;
  int64_t nx, ny, nz; /* nz = 1 for ndim 2 */
  double Lx, Ly, Lz;
  double nu_2, nu_4, nu_8, nu_m4;
  double beta;  /* ns2d: beta-plane term of compute_Frot              */
  double f;     /* ns3d: Coriolis parameter added to omega_z(k=0)      */
  int has_f;    /* ns3d: 1 when params.f is not None                   */
  int64_t kcut_x, kcut_y, kcut_z;
  int dtype;
  int strat;    /* buoyancy solvers, power-of-two grids only: ns3d.strat
                   (fluidsim/solvers/ns3d/strat/solver.py), state
                   (vx, vy, vz, b); ns2d.strat (ns2d/strat/solver.py),
                   state (rot, b)                                        */
  double N;     /* Brunt-Vaisala frequency (params.N): the -N^2 v_z (u_y)
                   term of the b tendency and EA = |b|^2 / (2 N^2)       */
  int bouss;    /* with strat: ns3d.bouss / ns2d.bouss (ns3d/bouss/
                   solver.py, ns2d/bouss/solver.py), the same tendencies
                   without the -N^2 v_z term (N then only sets EA)       */
} gbs_ns_params;

int gbs_ns_create(const gbs_ns_params* params, gbs_ns** solver);
int gbs_ns_destroy(gbs_ns* solver);

/* Simul.tendencies_nonlin(state_spect): tend = dealias(P_perp FFT(v x w))
 * (ns3d) or dealias(FFT(-u.grad(rot) - beta u_y)) (ns2d). */
int gbs_ns_tendencies(gbs_ns* solver, const void* state_spect, void* tend,
                      void* stream);

/* flags of gbs_ns_step / gbs_ns_step_rk4 */
#define GBS_STEP_CHECK_NAN 1 /* check state_spect[0] for NaN (synchronises)  */
#define GBS_STEP_DEALIASED 2 /* state_spect is zero at every mode removed by
                                the truncation (true after any completed
                                step): lets the passes skip those modes     */

/* One RK4 step with exact integrating factor, followed by projection
 * (ns3d), dealiasing and the NaN check: TimeSteppingPseudoSpectral
 * ._time_step_RK4 (fluidsim/base/time_stepping/pseudo_spect.py:798-984) +
 * one_time_step_computation (pseudo_spect.py:236-243,
 * fluidsim/solvers/ns3d/time_stepping.py:8-20).  state_spect is updated in
 * place.  *dt is the time increment; when cfl != NULL the CFL rule of
 * fluidsim/base/time_stepping/base.py:320-354 is applied first (from the
 * velocity of the current state, which the step computes anyway) and *dt is
 * updated: cfl[0] = CFL coefficient, cfl[1] = deltat_max.  That path
 * synchronises the stream once.  With GBS_STEP_CHECK_NAN, returns GBS_ENAN
 * (after completing the step) when state_spect[0] holds a NaN.  With
 * GBS_STEP_DEALIASED the caller asserts that the state is dealiased; the
 * result is the same, the transforms skip the modes the 2/3 rule zeroes.
 * The FP32 ns3d x pass stages its inputs with bulk copies awaited on
 * mbarriers (bounded waits, 1 s); if a wait runs out the step completes
 * with an invalid result and, at the next step with GBS_STEP_CHECK_NAN,
 * returns GBS_ETIMEDOUT (once).  GBS_STEP_TEST_STALL (test hook, defined
 * below) withholds one staging copy of the step's first x pass and waits
 * 1 ms for it. */
int gbs_ns_step_rk4(gbs_ns* solver, void* state_spect, double* dt,
                    const double* cfl, int flags, void* stream);

/* Time schemes of TimeSteppingPseudoSpectral (params.time_stepping
 * .type_time_scheme), all with the exact integrating factor. */
#define GBS_SCHEME_RK4 0            /* _time_step_RK4, pseudo_spect.py:798-984 */
#define GBS_SCHEME_EULER 1          /* _time_step_Euler, 245-280             */
#define GBS_SCHEME_RK2 2            /* _time_step_RK2, 469-517               */
#define GBS_SCHEME_RK2_TRAPEZOID 3  /* _time_step_RK2_trapezoid, 519-569     */
#define GBS_SCHEME_EULER_PHASESHIFT 4      /* _time_step_Euler_phaseshift, 374-419 */
#define GBS_SCHEME_RK2_PHASESHIFT 5        /* _time_step_RK2_phaseshift, 571-639   */
#define GBS_SCHEME_RK2_PHASESHIFT_EXACT 6  /* _time_step_RK2_phaseshift_exact,
                                              712-796 (allocates one more state
                                              buffer at its first step)          */
#define GBS_SCHEME_EULER_PHASESHIFT_RANDOM 7  /* _time_step_Euler_phaseshift_random,
                                                 421-467                          */
#define GBS_SCHEME_RK2_PHASESHIFT_RANDOM 8    /* _time_step_RK2_phaseshift_random,
                                                 641-710                          */

/* One step of `scheme`, otherwise as gbs_ns_step_rk4 (same flags, CFL rule,
 * projection, dealiasing and NaN check).  The phase-shift schemes evaluate
 * tendencies on exp(i phi) S with phi = a_x dx kx + a_y dy ky + a_z dz kz:
 * a = (1/2, 1/2, 1/2) for the fixed-shift schemes (pseudo_spect.py:282-300);
 * the random ones use the pair (alpha, beta) last given to
 * gbs_ns_set_phase_shifts, alpha for their first evaluation and beta for
 * their second.  They are rejected with GBS_EINVAL when a turbulence model
 * is set. */
int gbs_ns_step(gbs_ns* solver, int scheme, void* state_spect, double* dt,
                const double* cfl, int flags, void* stream);

/* The shift pair of the random phase-shift schemes for the next steps, in
 * grid spacings per axis (3 doubles each; z ignored in 2D): the caller draws
 * them as TimeSteppingPseudoSpectral._get_phaseshift_random does
 * (pseudo_spect.py:302-372) from get_phases_random (operators3d.py:
 * 1128-1146): alpha_i uniform in (-1/2, 1/2), beta_i = alpha_i +- 1/2. */
int gbs_ns_set_phase_shifts(gbs_ns* solver, const double* alpha, const double* beta);

/* Turbulence model added to the ns3d tendencies before projection and
 * dealiasing, in every stage (fluidsim/solvers/ns3d/solver.py:246-249,
 * TurbModel.get_forcing fluidsim/base/turb_model/base.py:87-88).
 *   type 0: none;
 *   type 1: Smagorinsky with constant C (turb_model/smagorinsky.py:56-110,
 *           Delta = Lx / nx);
 *   type 2: learned closure, tau_ij = MLP(d_j u_i) (9 -> 64 -> 64 -> 6, tanh,
 *           BF16 weights, FP32 activations and accumulation), forcing
 *           -d_j tau_ij;
 *   type 3: the same network in BF16 form (activations rounded to BF16,
 *           hardware tanh; relative error ~3e-3, see gbs_mlp_forward_bf16).
 * The weights are device pointers owned by the caller, read at every step.
 * Allocates the model's work buffers (synchronises the device). */
typedef struct gbs_mlp_weights {
  const void* W1;  /* bf16 [64][9]  */
  const void* W2;  /* bf16 [64][64] */
  const void* W3;  /* bf16 [6][64]  */
  const float* b1; /* [64] */
  const float* b2; /* [64] */
  const float* b3; /* [6]  */
  const float* in_scale;  /* [9]: network input = d_j u_i * in_scale   */
  const float* out_scale; /* [6]: tau = network output * out_scale     */
} gbs_mlp_weights;

int gbs_ns_set_turb_model(gbs_ns* solver, int type, double C,
                          const gbs_mlp_weights* weights);

/* Forcing added to the tendencies in every stage, before projection and
 * dealiasing (`tendencies_fft += self.forcing.get_forcing()`,
 * fluidsim/solvers/ns3d/solver.py:243-244, ns2d/solver.py:189-190):
 * device pointer to nvar spectral fields owned by the caller and read at
 * every stage (the caller updates it between steps, as
 * sim.forcing.compute() does once per step); NULL disables. */
int gbs_ns_set_forcing(gbs_ns* solver, const void* forcing);

/* One step of fluidsim's coarse normalized forcings, computed on the device
 * into the dense `forcing` array given to gbs_ns_set_forcing (replaces
 * SpecificForcingPseudoSpectralCoarse / NormalizedForcing.compute /
 * normalize_forcingc_2nd_degree_eq / coef_normalization_from_abc and
 * Proportional.compute, fluidsim/base/forcing/specific.py:137-727, for
 * TimeCorrelatedRandomPseudoSpectral and RandomSimplePseudoSpectral,
 * 729-868).  The coarse grid has nc points per axis (coarse spectral shape
 * (nc, nc, nc/2+1), 2D (nc, nc/2+1)); coarse mode ic maps to the full-grid
 * mode ic if ic <= nc/2, else ic - nc + n (kx unchanged).  For each forced
 * state variable keys[k]:
 *   type 0 (normalized): fr = f1 - mix (f1 - f0) from the coarse complex128
 *     device arrays f0, f1; R = root of (dt/2 sum w|fr|^2) R^2 +
 *     (sum w Re(conj(v) fr)) R - forcing_rate = 0, which_root 0: "minabs",
 *     1: "positive";
 *   type 1 (proportional): fr = v on the modes where no_forcing[i] == 0,
 *     R = (sqrt(1 + dt P / Z) - 1) / dt with Z = sum w |fr|^2 / 2;
 * forcing[keys[k]] = R fr on the coarse modes (nothing else written).  Sums
 * in FP64 with the coarse grid's Hermitian weights.  coef (device, nkeys
 * doubles, may be NULL) receives R.  One CTA; no host synchronisation. */
typedef struct gbs_forcing_params {
  int ndim;
  int64_t nx, ny, nz; /* full grid (nz ignored in 2D) */
  int64_t nc;         /* coarse points per axis (even) */
  int nvar;           /* state variables in state_spect / forcing */
  int nkeys;          /* forced variables, 1..8 */
  int keys[8];
  int type;           /* 0 normalized, 1 proportional */
  int which_root;     /* 0 minabs, 1 positive */
  double forcing_rate;
  int dtype;          /* GBS_F32 / GBS_F64: state and forcing arrays */
} gbs_forcing_params;

int gbs_forcing_coarse(const gbs_forcing_params* params, const void* state_spect,
                       const void* f0, const void* f1,
                       const unsigned char* no_forcing, double mix, double dt,
                       void* forcing, double* coef, void* stream);

/* ------------------------------------------------ batched ns2d ensembles
 * nruns independent ns2d runs of one grid (power-of-two nx/2, ny in
 * 64..512), float32, advanced together: one launch per pass covers the
 * whole batch, every run with its own nu_2, nu_8 and dt (host arrays of
 * nruns).  The runs of fluidsim are independent simulations
 * (fluidsim/solvers/ns2d/solver.py); there is no reference batching.
 * gbs_ens2d_step enqueues nsteps RK4 steps of every run on `stream`
 * without host synchronisation, so it can be captured in a CUDA graph;
 * state: (nruns, ny, nx/2+1) complex64.  gbs_ens2d_set_tuning picks the
 * compiled tile shapes (y-pass column widths 4/8/16, x-pass rows 1/2/4/8).
 * gbs_ens2d_nan_flag reads and clears the flag set when a run's state holds
 * a NaN (synchronises). */
typedef struct gbs_ens2d gbs_ens2d;
int gbs_ens2d_create(int64_t nx, int64_t ny, double Lx, double Ly, int64_t nruns,
                     int64_t kcut_x, int64_t kcut_y, double beta, gbs_ens2d** ens);
int gbs_ens2d_destroy(gbs_ens2d* ens);
int gbs_ens2d_set_params(gbs_ens2d* ens, const double* nu_2, const double* nu_8,
                         const double* dt);
int gbs_ens2d_set_tuning(gbs_ens2d* ens, int tx_inverse, int rows_x,
                         int tx_forward);
int gbs_ens2d_step(gbs_ens2d* ens, void* state_spect, int nsteps, int flags,
                   void* stream);
int gbs_ens2d_nan_flag(gbs_ens2d* ens, int* flag);

/* Groups of different sizes stepped together: one launch per pass of an RK4
 * stage covers every run of every group (up to 4 groups; they are not
 * owned and must outlive the object).  states[k] is group k's state.
 * Enqueue only, as gbs_ens2d_step. */
typedef struct gbs_ens2d_mixed gbs_ens2d_mixed;
int gbs_ens2d_mixed_create(gbs_ens2d* const* groups, int ngroups, gbs_ens2d_mixed** mixed);
int gbs_ens2d_mixed_destroy(gbs_ens2d_mixed* mixed);
/* threads per CTA of the inverse y, x and forward y launches (128, 256 or
 * 512; default 512), within what every group's size allows */
int gbs_ens2d_mixed_set_tuning(gbs_ens2d_mixed* mixed, int th_inverse, int th_x,
                               int th_forward);
int gbs_ens2d_mixed_step(gbs_ens2d_mixed* mixed, void* const* states, int nsteps, int flags,
                         void* stream);

/* The same nsteps RK4 steps in ONE persistent cooperative launch (replaces
 * the pass-by-pass launches of the batched form; fluidsim itself steps one
 * run at a time, fluidsim/base/time_stepping/pseudo_spect.py:798-984).  The
 * CTAs (`threads` each: 256 or 512) take work items from a device queue in
 * the order (stage, pass, group, run, tile); each item first waits until
 * the items of its own run that it reads are done (per-run counters, no
 * grid-wide barrier).  Every wait gives up after timeout_s seconds: the
 * launch then stops early, leaves the states undefined, and
 * gbs_ens2d_persistent_status returns GBS_ETIMEDOUT with *status = 1 (and
 * clears it).  Without GBS_STEP_DEALIASED the first step runs as
 * gbs_ens2d_mixed_step.  GBS_STEP_TEST_STALL (test hook) makes one wait
 * need an item that does not exist, so that it runs out. */
#define GBS_STEP_TEST_STALL 64
int gbs_ens2d_persistent_step(gbs_ens2d_mixed* mixed, void* const* states, int nsteps,
                              int threads, double timeout_s, int flags, void* stream);
int gbs_ens2d_persistent_status(gbs_ens2d_mixed* mixed, int* status);
/* work items a CTA of the persistent step takes from the queue at a time
 * (1..64, default 4): its completions are published per (run, pass) group,
 * before any wait and at the end of each chunk */
int gbs_ens2d_persistent_set_chunk(gbs_ens2d_mixed* mixed, int chunk);

/* Filtered-DNS data for the learned closure (no reference counterpart):
 *   gbs_spectral_resample: nfields spectral fields of shape_in (nz, ny, nx)
 *     onto shape_out, keeping |k_a| < m_a / 2, multiplied by the top-hat
 *     filter transfer prod_a sinc(k_a delta / 2) when delta > 0
 *     (L = Lz, Ly, Lx);
 *   gbs_products6: physical products (xx, yy, zz, xy, xz, yz) of 3 fields of
 *     n points, or sub - products when sub != NULL;
 *   gbs_velocity_gradients: 9 spectral fields 1j k_j v_i (index 3 i + j) of a
 *     (3, nz, ny, nx/2+1) state, zero where |k_a| >= kcut_a (z, y, x). */
int gbs_spectral_resample(const int64_t* shape_in, const int64_t* shape_out,
                          int nfields, const double* L, double delta, int dtype,
                          const void* in, void* out, void* stream);
int gbs_products6(const void* u, void* out, int64_t n, const void* sub, int dtype,
                  void* stream);
int gbs_velocity_gradients(const int64_t* shape, const double* L,
                           const int64_t* kcut, int dtype, const void* S,
                           void* G, void* stream);

/* Learned-closure network: inference and training (no reference
 * counterpart; the reference's turbulence models are analytic).
 * Fields are structure-of-arrays float32: g[c * ld + i] (9 rows, the
 * velocity gradients d_j u_i with c = 3 i + j), tau[o * ld + i] (6 rows,
 * xx yy zz xy xz yz).
 *   gbs_mlp_forward: tau = MLP(g) for points 0..n-1 (FP32 activations:
 *     three BF16 terms per tensor-core operand).
 *   gbs_mlp_forward_bf16: the same in BF16 form, the activations rounded to
 *     BF16 operands and tanh by the hardware approximation (relative error
 *     ~3e-3 against gbs_mlp_forward, a third of its tensor-core work).
 *   gbs_mlp_grad: loss over the `batch` points idx[0..batch-1] (device
 *     int64): mean squared error of MLP(g) / out_scale against
 *     tau / out_scale, plus pi_weight (>= 0) times the mean of
 *     (Pi(MLP(g)) - Pi(tau))^2 with the subgrid dissipation
 *     Pi(t) = t_ij S_ij, S_ij = (d_j u_i + d_i u_j) / 2; its gradient w.r.t.
 *     the 5190 parameters (layout W1, b1, W2, b2, W3, b3) into grad (device)
 *     and the loss into *loss (device); workspace of
 *     gbs_mlp_grad_workspace(batch) bytes.  Deterministic.
 *   gbs_mlp_adam: one Adam step on the FP32 master parameters (same layout)
 *     with moments m, v; writes the BF16 copies W1, W2, W3 of w_bf16. */
int64_t gbs_mlp_grad_workspace(int64_t batch);
int gbs_mlp_forward(const gbs_mlp_weights* w, const float* g, int64_t ld,
                    float* tau, int64_t n, void* stream);
int gbs_mlp_forward_bf16(const gbs_mlp_weights* w, const float* g, int64_t ld,
                         float* tau, int64_t n, void* stream);
int gbs_mlp_grad(const gbs_mlp_weights* w, const float* g, const float* tau,
                 int64_t ld, const int64_t* idx, int64_t batch,
                 double pi_weight, void* workspace, float* grad, float* loss,
                 void* stream);
int gbs_mlp_adam(float* master, float* m, float* v, const float* grad,
                 int64_t step, double lr, double beta1, double beta2,
                 double eps, const gbs_mlp_weights* w_bf16, void* stream);

/* max |u_i| over the physical grid of state_spect (ns2d: ux, uy; ns3d: vx,
 * vy, vz) into out[ndim] (host).  Synchronises the stream. */
int gbs_ns_max_velocity(gbs_ns* solver, const void* state_spect, double* out,
                        void* stream);

/* Host-only CFL update, fluidsim/base/time_stepping/base.py:334-354:
 * tmp = sum_i max|u_i| / dx_i.  Returns the new dt (dt if the relative
 * change is <= 2 %). */
double gbs_cfl_update(double dt, double tmp, double cfl_coef,
                      double deltat_max);

/* FP64 spatial means from the spectral state (Hermitian-weighted sums,
 * fluidsim/solvers/ns2d/output/spatial_means.py:23-36,
 * fluidsim/solvers/ns3d/output/spatial_means.py:23-40).
 * out (host, 9 doubles): ns2d {E, Z, epsK, epsK_hypo, epsZ, epsZ_hypo, 0, 0, 0};
 *   ns3d {EK, EKx, EKy, EKz, epsK, epsK_hypo, EA, epsA, epsA_hypo} with the
 *   potential-energy terms of ns3d.strat (EA = |b|^2 / (2 N^2),
 *   ns3d/strat/output/spatial_means.py:27-61; zero otherwise).
 *   Synchronises. */
int gbs_ns_spatial_means(gbs_ns* solver, const void* state_spect, double* out,
                         void* stream);

/* Per-kernel timing of a solver's launches with CUDA events recorded on the
 * launching stream (no counterpart in the reference, which times whole runs
 * with time(): fluidsim/util/console/util.py:329-390).  enable = 1 clears
 * the totals and starts recording, 0 stops.  Kinds: 0 = inverse z pass with
 * the curl (ns2d: inverse y), 1 = inverse y pass (ns3d), 2 = x pass with the
 * products, 3 = forward y pass (ns3d), 4 = last forward pass with the RK4
 * stage.  The report synchronises on the recorded events; *launches counts
 * every kernel the solver launched since creation. */
int gbs_ns_timing(gbs_ns* solver, int enable);
int gbs_ns_timing_report(gbs_ns* solver, double* ms, int64_t* count,
                         int nkinds, int64_t* launches);

/* Shell energy spectrum in FP64 (device output spectrum[nk], nk from
 * gbs_ns_spectrum_size): bins round(|k| / dk_min), E summed with Hermitian
 * weights, divided by dk_min. */
int gbs_ns_spectrum_size(gbs_ns* solver, int64_t* nk);
int gbs_ns_spectrum(gbs_ns* solver, const void* state_spect, double* spectrum,
                    void* stream);

/* FP64 spectra of a real spectral energy density `energy` (shape (nz, ny,
 * nx/2+1), 2D: (ny, nx/2+1); dtype GBS_F32 or GBS_F64), replacing the
 * operator methods compute_1dspectra / compute_3dspectrum /
 * compute_spectrum_kzkh (3D) and spectra1D_from_fft / spectrum2D_from_fft
 * (2D) that fluidsim's spectra outputs call
 * (fluidsim/solvers/ns3d/output/spectra.py:15-100,
 * fluidsim/solvers/ns2d/output/spectra.py:16-27, bound at
 * fluidsim/base/output/spectra.py:373-374; the methods live in fluidfft).
 * Hermitian weights (1 for kx = 0 and the Nyquist column, else 2), each
 * output divided by its bin width: skx[nx/2+1] per kx; sky[ny/2+1] and
 * skz[nz/2+1] binned by |k_adim|; shell[n3] binned by floor(|k|/dk + 0.5),
 * dk = min(deltak); kzkh[(nz/2+1) * nkh] by |kz_adim| and
 * floor(kh/dkh + 0.5), dkh = min(dkx, dky).  deltak = (dkx, dky[, dkz]).
 * Any output may be NULL (skz and kzkh must be in 2D); device pointers.
 * gbs_spectra_sizes writes (nx/2+1, ny/2+1, nz/2+1 or 0, n3, nkh or 0). */
int gbs_spectra_sizes(int ndim, const int64_t* shapeX, const double* deltak,
                      int64_t* sizes);
int gbs_spectra(int ndim, const int64_t* shapeX, const double* deltak, int dtype,
                const void* energy, double* skx, double* sky, double* skz,
                double* shell, double* kzkh, void* stream);

/* ns3d projection of the tendencies and of the state after each step
 * (Simul.project_state_spect, fluidsim/solvers/ns3d/solver.py:147-175,
 * 255-263): params.projection None / "toroidal" ("vortical") / "poloidal"
 * -> project_perpk3d / project_toroidal / project_poloidal
 * (fluidsim/operators/operators3d.py:788-959); no_vz_kz0 != 0 also zeroes
 * vz at kz = 0. */
#define GBS_PROJ_PERPK 0
#define GBS_PROJ_TOROIDAL 1
#define GBS_PROJ_POLOIDAL 2
int gbs_ns_set_projection(gbs_ns* solver, int projection, int no_vz_kz0);

/* *out = 1 when every mode that the 2/3 truncation removes is +0 (all bits
 * zero) in every field of state_spect, else 0; synchronises the stream.  A
 * step may then be called with GBS_STEP_DEALIASED and gives exactly the
 * unpruned result (no reference counterpart: the reference has no pruned
 * passes; the truncation is dealiasing_setofvar, operators3d.py:38-59). */
int gbs_ns_is_dealiased(gbs_ns* solver, const void* state_spect, int* out,
                        void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBSPEC_H */
