/* heomgb.h -- C ABI of the GB300-native HEOM propagation engine.
 *
 * Drop-in for libheom's propagation path: the heom_hilb / heom_liou / heom_ado
 * models built from H, the bath couplings V, the exponential noise
 * decomposition and the hierarchy depth, stepped by rk4 / lsrk4 / rkdp through
 * qme_solver.  Each entry point names the reference interface it replaces
 * (file:line in the libheom tree).  Plain pointers and sizes only; complex
 * numbers are two doubles (re, im); matrices are row-major (the reference's
 * `row_major` order).  Every call returns a heomgb_status; nothing exits the
 * process (the reference's CUDA_CALL/std::exit is replaced by status codes).
 *
 * Threading: one qme / solver object must not be used from two host threads
 * at once (the reference's engines are not re-entrant either).
 */
#ifndef HEOMGB_H
#define HEOMGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum heomgb_status {
  HEOMGB_OK = 0,
  HEOMGB_ERR_INVALID_ARGUMENT = 1, /* bad size, index, null pointer, missing kwarg   */
  HEOMGB_ERR_STATE = 2,            /* call out of order (e.g. solve before set_param) */
  HEOMGB_ERR_CUDA = 3,             /* CUDA runtime error (message via last_error)     */
  HEOMGB_ERR_ALLOC = 4,            /* device or host allocation failed                */
  HEOMGB_ERR_UNSUPPORTED = 5,      /* option outside what this build implements       */
  HEOMGB_ERR_NUMERIC = 6,          /* non-finite step-size control / attempt cap hit  */
  HEOMGB_ERR_CAPACITY = 7          /* request above a documented fixed maximum        */
} heomgb_status;

/* Model forms: heom_hilb (heom_hilb.h:18-216), heom_liou (heom_liou.h:18-259),
 * heom_ado (heom_ado.h:18-204); and the Redfield models redfield_hilb
 * (redfield_hilb.h:18-91) and redfield_liou (redfield_liou.h:18-104), built
 * from the same H and noise members (redfield.h:42-173; max_depth is ignored,
 * the state is one n x n matrix, main_size() = n^2). */
typedef enum heomgb_form {
  HEOMGB_HILB = 0,
  HEOMGB_LIOU = 1,
  HEOMGB_ADO = 2,
  HEOMGB_REDFIELD_HILB = 3,
  HEOMGB_REDFIELD_LIOU = 4
} heomgb_form;

/* Integrators: rk4 (solver/rk4.h:15-66), lsrk4 (solver/lsrk4.h:15-48),
 * rkdp (solver/rkdp.h:15-180). */
typedef enum heomgb_solver_kind { HEOMGB_RK4 = 0, HEOMGB_LSRK4 = 1, HEOMGB_RKDP = 2 } heomgb_solver_kind;

/* Arithmetic of the right-hand side.  FP64: everything in double (the plain
 * drop-in).  MIXED: the bulk complex products and the stage inputs in FP32,
 * while the state vector, stage accumulation, error norm and step control
 * stay FP64. */
typedef enum heomgb_precision { HEOMGB_FP64 = 0, HEOMGB_MIXED = 1 } heomgb_precision;

typedef struct heomgb_qme heomgb_qme;
typedef struct heomgb_solver heomgb_solver;
typedef struct heomgb_qme_solver heomgb_qme_solver;

/* The reference's kwargs_t (type.h:49) with the keys its solvers read:
 * "dt" (fixed_step_size_solver.h:37, adaptive_step_size_solver.h:40),
 * "atol", "rtol" (adaptive_step_size_solver.h:42-43).  A key the solver needs
 * but whose has_* flag is 0 gives HEOMGB_ERR_INVALID_ARGUMENT (the reference
 * throws std::out_of_range). */
typedef struct heomgb_kwargs {
  double dt, atol, rtol;
  int has_dt, has_atol, has_rtol;
} heomgb_kwargs;

/* Called at every output time, as solver_base::solve does (solver_base.h:72-78). */
typedef void (*heomgb_callback)(double t, void* user);

/* ---- diagnostics -------------------------------------------------------- */
const char* heomgb_last_error(void);             /* thread-local message of the last failure */
const char* heomgb_version(void);
int heomgb_abi_version(void);
/* Number of kernels this library has launched so far (graph nodes included). */
long long heomgb_launch_count(void);

/* ---- model (qme) --------------------------------------------------------- */
/* heom_hilb/heom_liou/heom_ado(int max_depth, int n_inner_threads,
 * int n_outer_threads) -- heom_hilb.h:41-43, heom.h:44-50.  The thread counts
 * are accepted for interface parity; the device path does not use them. */
heomgb_status heomgb_qme_create(heomgb_form form, int max_depth, int n_inner_threads, int n_outer_threads,
                                heomgb_qme** out);
/* Fails with HEOMGB_ERR_STATE while qme_solvers created from q still exist. */
heomgb_status heomgb_qme_destroy(heomgb_qme* q);

/* Public members n_level / n_level_2 / H (qme_base.h:32-36).  H: n*n complex. */
heomgb_status heomgb_qme_set_hamiltonian(heomgb_qme* q, int n_level, const double* H);
/* alloc_noises(n_noise) -- qme_base.h:47-60. */
heomgb_status heomgb_qme_alloc_noises(heomgb_qme* q, int n_noise);
/* V[u], len_gamma[u], gamma[u], phi_0[u], sigma[u], S[u], A[u], s_delta[u]
 * (qme_base.h:38-45).  V: n*n, gamma/S/A: len*len, phi_0/sigma: len, s_delta: 1
 * complex.  Off-diagonal gamma entries are accepted and, as in the reference
 * (heom.h:110 clears gamma[u] before reading them), never contribute. */
heomgb_status heomgb_qme_set_noise(heomgb_qme* q, int u, const double* V, int len_gamma, const double* gamma,
                                   const double* phi_0, const double* sigma, const double* S, const double* A,
                                   const double* s_delta);
heomgb_status heomgb_qme_set_precision(heomgb_qme* q, heomgb_precision p);
/* Normalisation of the auxiliary density operators, the reference's
 * compile-time LIBHEOM_SQRT_NORMALIZATION switch made a model option: INTEGER
 * (the reference's default) or SQRT, where the +1 terms scale by sqrt(n_k+1)
 * and the -1 terms by sqrt(n_k) instead of 1 and n_k (heom_hilb.h:140-196,
 * heom_liou.h:188-230, heom_ado.h:93-97,131-139).  Set before set_param. */
typedef enum heomgb_normalization { HEOMGB_NORM_INTEGER = 0, HEOMGB_NORM_SQRT = 1 } heomgb_normalization;
heomgb_status heomgb_qme_set_normalization(heomgb_qme* q, heomgb_normalization norm);
/* Storage order of every ADO in the state vectors the caller passes (rho,
 * drho, the solve state and the callback's view of it): the reference's
 * `order` template argument (row_major / col_major, type.h; lil_matrix.h.j2:
 * 156-163).  Parameter matrices are always given row-major (logical entries).
 * The device keeps row-major ADOs and transposes at the boundary. */
typedef enum heomgb_order { HEOMGB_ROW_MAJOR = 0, HEOMGB_COL_MAJOR = 1 } heomgb_order;
heomgb_status heomgb_qme_set_order(heomgb_qme* q, heomgb_order order);
/* Hierarchy filter: alloc_hrchy_space's hrchy_filter with filter_flag = true
 * (hrchy_space.h:29-36, hrchy_space.cc:182-191; heom::set_param passes none,
 * heom.h:80-91).  At set_param the filter is called, on the host, for every
 * candidate multi-index (n_dim ints) of total `depth` whose parent was kept, in
 * the reference's breadth-first order; nonzero keeps it.  A rejected index
 * takes the indices it would have spawned with it.  NULL: no filter (the
 * default).  Not with the learned terminator. */
typedef int (*heomgb_hrchy_filter)(const int* index, int n_dim, int depth, void* user);
heomgb_status heomgb_qme_set_hrchy_filter(heomgb_qme* q, heomgb_hrchy_filter filter, void* user);
/* Precision after set_param (no reference counterpart: the reference has one
 * compile-time precision).  A MIXED request runs with FP64 arithmetic
 * (effective = FP64) when the bath expansion makes FP32 arithmetic unsafe.
 * With growth_log10 = max_k N log10((|s_k| + |a_k|) / |Re gamma_kk|) (how far
 * deep ADOs outgrow rho_0 under the integer normalisation) and cancel_log10 =
 * max_u log10(sum_k |s_k| / |sum_k s_k|) (how strongly one bath's coefficients
 * cancel, e.g. a Matsubara frequency near the Drude pole), that is when
 * cancel_log10 > 0.8, or growth_log10 > 7.5, or both growth_log10 > 2 and
 * cancel_log10 > 0.2. */
heomgb_status heomgb_qme_get_precision(const heomgb_qme* q, int* requested, int* effective, double* growth_log10,
                                       double* cancel_log10);
/* Run the model's CUDA work on this stream (a cudaStream_t); NULL restores the
 * library's own stream.  Must precede heomgb_qme_solver_create to affect it. */
heomgb_status heomgb_qme_set_stream(heomgb_qme* q, void* cuda_stream);
/* set_param(engine) -- heom_hilb.h:57-68 / heom.h:57-139 / heom_liou.h:66-119 /
 * heom_ado.h:62-189.  Builds the hierarchy tables on the device, uploads H/V and
 * the per-ADO damping, and builds the superoperators of the Liouville forms.
 * Fails with HEOMGB_ERR_STATE while qme_solvers created from q still exist
 * (their captured launches hold the model's device pointers). */
heomgb_status heomgb_qme_set_param(heomgb_qme* q);
/* get_n_hrchy() -- heom.h:52-55. */
heomgb_status heomgb_qme_get_n_hrchy(const heomgb_qme* q, int* n_hrchy);
/* Number of linear noise modes (hs.n_dim, heom.h:62-63). */
heomgb_status heomgb_qme_get_n_dim(const heomgb_qme* q, int* n_dim);
/* main_size() = n_level^2 * n_hrchy -- heom_hilb.h:45-49. */
heomgb_status heomgb_qme_main_size(const heomgb_qme* q, long long* size);
/* Hierarchy tables hs.n, hs.ptr_p1, hs.ptr_m1 (hrchy_space.h:18-27), copied
 * from the device: n is n_hrchy*n_dim, ptr_p1/ptr_m1 are (n_hrchy+1)*n_dim
 * with the sentinel ptr_void = n_hrchy.  Any pointer may be NULL. */
heomgb_status heomgb_qme_get_hrchy(const heomgb_qme* q, int* n, int* ptr_p1, int* ptr_m1);
/* calc_diff_impl(obj, drho_dt, rho, alpha, beta, temp) -- heom_hilb.h:70-215:
 * drho = beta*drho - alpha*D(rho) with host arrays of main_size() complex.
 * (The reference's qme_solver::calc_diff is an empty stub, qme_solver.h:37-42;
 * this is the model-level operator it would call.) */
heomgb_status heomgb_qme_calc_diff(heomgb_qme* q, double* drho, const double* rho, const double* alpha,
                                   const double* beta);
/* Same with device pointers (double2 arrays of main_size()), on the qme stream. */
heomgb_status heomgb_qme_calc_diff_device(heomgb_qme* q, void* drho, const void* rho, const double* alpha,
                                          const double* beta);

/* ---- solvers --------------------------------------------------------------- */
/* rk4<...>(), lsrk4<...>(), rkdp<...>() default constructors. */
heomgb_status heomgb_solver_create(heomgb_solver_kind kind, heomgb_solver** out);
heomgb_status heomgb_solver_destroy(heomgb_solver* s);

/* qme_solver(engine, qme, solver) -- qme_solver.h:26-35: allocates the state
 * and stage buffers of `s` for `q` (solver_base::init, rk4::init, ...). */
heomgb_status heomgb_qme_solver_create(heomgb_qme* q, heomgb_solver* s, heomgb_qme_solver** out);
heomgb_status heomgb_qme_solver_destroy(heomgb_qme_solver* qs);

/* Batched form without a reference counterpart: one qme_solver over `count`
 * set-up heom_hilb models with diagonal couplings (uneven n_level and depth
 * allowed) that share a precision; every stage of every instance runs in the
 * same kernel launch.  The state passed to solve is the concatenation of the
 * models' states in the given order (heomgb_qme_solver_main_size elements).
 * rk4 / lsrk4 only (one dt for all instances).  A batch solver runs on a CUDA
 * stream of its own; each solve first waits for the work already queued on
 * the first model's stream.  Solves of different batch solvers may be issued
 * from different host threads and then run concurrently (the Python batch
 * solver does so for its mixed and FP64 sub-batches); calls on one solver
 * must not overlap. */
heomgb_status heomgb_batch_solver_create(heomgb_qme* const* qmes, int count, heomgb_solver* s,
                                         heomgb_qme_solver** out);
/* Elements of the state a solve of qs expects (main_size(), summed over a batch). */
heomgb_status heomgb_qme_solver_main_size(const heomgb_qme_solver* qs, long long* size);
/* Tile shape the autotuner picked for the diagonal-coupling kernel: CTA size,
 * elements per thread, number of tiles and the kernel variant's minimum
 * resident CTAs (1, or 3 for the mixed form's register-capped variant); 0 for
 * the other kernels.  The environment variable
 * HEOMGB_TILE=<64|128|256>x<1..8>[x<1|3|4>] (e.g. "128x2") pins the shape
 * instead of searching, for reproducible profiles. */
heomgb_status heomgb_qme_solver_tuning(const heomgb_qme_solver* qs, int* block, int* elems_per_thread,
                                       int* n_tiles, int* min_blocks);
/* 1 when the autotuner put the mixed form's commutators [H, rho] on the
 * tensor cores (3xTF32 tcgen05 MMAs with tensor-memory accumulators; real
 * symmetric H, n_level in {8, 12, 16, 24, 32}), else 0.  HEOMGB_TILE=tc pins
 * that variant, HEOMGB_TCORE=0 keeps it out of the search.  No reference
 * counterpart: the reference evaluates every term on CUDA cores. */
heomgb_status heomgb_qme_solver_tensor_cores(const heomgb_qme_solver* qs, int* on);
/* 1 when the autotuner picked the stage kernel for site-local baths (every V_u
 * diagonal with a single nonzero entry, as in exciton aggregates; real H;
 * n_level a multiple of 4, at least 8; mixed form): per tile of consecutive
 * ADOs, the commutator in register blocks, then the bath terms one warp per
 * ADO over its occupied modes, then a coalesced compile-time stage epilogue;
 * cp.async-staged tiles.  Same values as the general kernel (bit-identical
 * states).  ados_per_tile (may be NULL) receives its tile.  HEOMGB_SITES=0
 * keeps it out of the search, HEOMGB_TILE=sites:<block>x<tile>x<CTAs per
 * SM>[x<rows 4|2>] pins it.  No reference counterpart:
 * heom_hilb::calc_diff_impl (heom_hilb.h:70-215) visits every mode of every
 * ADO. */
heomgb_status heomgb_qme_solver_site_kernel(const heomgb_qme_solver* qs, int* on, int* ados_per_tile);
/* 1 when the solver runs each output interval (rkdp, rk4, lsrk4 in the mixed
 * form; rk4, and rkdp for site-local baths, in the FP64 form) as one resident
 * cooperative launch (one model on the diagonal-coupling path,
 * state held in the CTAs' shared memory between stages), else 0; grid and
 * ados_per_cta (may be NULL) receive its CTAs and the ADOs each owns.
 * HEOMGB_RESIDENT=0 keeps the per-stage kernels.  No reference counterpart:
 * rkdp::solve_adaptive_step (rkdp.h:81-179), rk4::solve_fixed_step
 * (rk4.h:40-65) and lsrk4::solve_fixed_step (lsrk4.h:32-47) issue every
 * stage's BLAS calls from the host. */
heomgb_status heomgb_qme_solver_resident(const heomgb_qme_solver* qs, int* on, int* grid, int* ados_per_cta);
/* 1 when the solver runs each fixed-step (rk4, lsrk4) output interval as one launch of
 * instance-resident bins (diagonal-coupling path, every instance inside one
 * CTA: its stage inputs in shared memory, no grid-wide synchronisation), else
 * 0; bins and block (may be NULL) receive the CTAs and their threads.  Chosen
 * where it beats the per-stage kernels; HEOMGB_LOCAL=0 keeps them,
 * HEOMGB_LOCAL=1 takes it wherever it applies.  No reference counterpart:
 * rk4::solve_fixed_step (rk4.h:40-65) and lsrk4::solve_fixed_step
 * (lsrk4.h:32-47) step one model at a time. */
heomgb_status heomgb_qme_solver_local(const heomgb_qme_solver* qs, int* on, int* bins, int* block);

/* qme_solver::solve(rho, t_list, n_t, callback, kwargs) -- qme_solver.h:44-52,
 * solver_base.h:64-79.  rho: host array of main_size() complex, updated in
 * place; the state crosses host<->device once per output interval exactly as
 * in the reference (host2dev before, dev2host after each interval).  The
 * callback may be NULL. */
heomgb_status heomgb_qme_solver_solve(heomgb_qme_solver* qs, double* rho, const double* t_list, int n_t,
                                      heomgb_callback cb, void* user, const heomgb_kwargs* kwargs);
/* Same with rho already resident on the device (double2 array of main_size());
 * no host<->device traffic of the state. */
heomgb_status heomgb_qme_solver_solve_device(heomgb_qme_solver* qs, void* rho, const double* t_list, int n_t,
                                             heomgb_callback cb, void* user, const heomgb_kwargs* kwargs);
/* Step statistics of the last solve: right-hand-side evaluations, step
 * attempts, accepted steps, and the step size kept for the next call
 * (rkdp's dt_save, adaptive_step_size_solver.h:21,55). */
heomgb_status heomgb_qme_solver_stats(const heomgb_qme_solver* qs, long long* n_rhs, long long* n_attempts,
                                      long long* n_accepted, double* dt_save);
/* Diagnostic without a reference counterpart: device time of the last solve
 * spent inside graph replays of fused stage kernels (CUDA events on the
 * solver's stream around every replay batch), and the number of kernels those
 * replays launched.  busy_ms / kernels is the average stage-kernel duration. */
heomgb_status heomgb_qme_solver_timing(const heomgb_qme_solver* qs, double* busy_ms, long long* kernels);

/* Diagnostic without a reference counterpart: FP64 and FP32 FMA throughput of
 * the current GPU in TFLOP/s, from register-only FMA chains (a few ms). */
heomgb_status heomgb_probe_fma_peaks(double* fp64_tflops, double* fp32_tflops);

/* ---- learned terminator (no reference counterpart) --------------------------
 * A small MLP x(d_in) -> Linear(d_hidden) -> GELU -> Linear(d_hidden) -> GELU ->
 * Linear(d_out), FP32 master weights + BF16 copies, FP32 accumulation, trained
 * with this library's forward / backward / Adam kernels.  Parameters are packed
 * [W1 (h x d_in), b1, W2 (h x h), b2, W3 (d_out x h), b3], row-major, FP32.
 * As a terminator of a model with n_level n and n_dim K it maps
 * [Re rho_n / s, Im rho_n / s, onehot(k), Re A / s, Im A / s] (4n^2 + K) of a
 * tier-N ADO, with A the adiabatic estimate of rho_{n+1_k} (its own time
 * derivative and the commutator with H dropped) and s = max_e |rho_n[e]|, to
 * an elementwise gain (2n^2 outputs: Re C_e, z_e) with
 *   C_e = Re C_e - i sign(v_a - v_b) softplus(z_e),
 *   rho_{n+1_k}[e] ~ C_e rho_n[e] / sigma_k,
 * i.e. it stands in for the ADOs that plain truncation drops
 * (ptr_p1 == ptr_void) through a closure term that can only damp. */
typedef struct heomgb_mlp heomgb_mlp;
heomgb_status heomgb_mlp_create(int d_in, int d_hidden, int d_out, unsigned long long seed, heomgb_mlp** out);
heomgb_status heomgb_mlp_destroy(heomgb_mlp* mlp);
heomgb_status heomgb_mlp_sizes(const heomgb_mlp* mlp, int* d_in, int* d_hidden, int* d_out, long long* n_params);
heomgb_status heomgb_mlp_get_params(heomgb_mlp* mlp, float* params);       /* host, n_params floats */
heomgb_status heomgb_mlp_set_params(heomgb_mlp* mlp, const float* params); /* host, n_params floats */
/* y = mlp(x) for `batch` rows; x_dev / y_dev are device float arrays. */
heomgb_status heomgb_mlp_forward(heomgb_mlp* mlp, const float* x_dev, float* y_dev, int batch);
/* Loss used by gradients / train_step.  kind 0 (default): mean((mlp(x) - t)^2),
 * t has d_out floats per row.  kind 1: the terminator's closure loss, with
 * d_out = 2 n2 and t rows [Re t, Im t, Re r, Im r, sg] (5 n2 floats;
 * t = rho_{n+1_k}/s, r = rho_n/(s sigma_k), sg = sign(v_a - v_b)): the mean over
 * rows of sum_e |sg_e| |C_e r_e - t_e|^2 / (sum_e |sg_e| (|t_e|^2 + 1e-2 |r_e|^2) + 1e-6). */
heomgb_status heomgb_mlp_set_loss(heomgb_mlp* mlp, int kind, int n2);
/* Gradient of the loss with respect to the packed parameters
 * (grad_host: n_params floats, may be NULL) and the loss; no update. */
heomgb_status heomgb_mlp_gradients(heomgb_mlp* mlp, const float* x_dev, const float* t_dev, int batch,
                                   float* grad_host, float* loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on that loss. */
heomgb_status heomgb_mlp_train_step(heomgb_mlp* mlp, const float* x_dev, const float* t_dev, int batch, float lr,
                                    float* loss);
/* Use `mlp` (not owned; must outlive the model's solvers) for the truncated
 * tier of q: an inference launch before every right-hand side fills the
 * predicted tier-(N+1) ADOs that the +1 coupling term reads.  NULL restores
 * plain truncation.  heom_hilb with diagonal V only; fails while solvers of q
 * exist. */
heomgb_status heomgb_qme_set_terminator(heomgb_qme* q, heomgb_mlp* mlp);

/* ---- building blocks ------------------------------------------------------ */
/* errnrm1(e, x_1, x_2, atol, rtol) -- linalg_engine_cuda.cu:176-201 and
 * linalg_engine_eigen.h.j2:360-379: sqrt(mean_i (|e_i|/(atol+rtol*max(|x1_i|,|x2_i|)))^2)
 * over n complex elements, device pointers (double2).  The per-block partial
 * sums go to a caller-provided device scratch array of heomgb_errnrm1_scratch(n)
 * doubles; the result is written to *result (host).  stream may be NULL. */
size_t heomgb_errnrm1_scratch(long long n);
heomgb_status heomgb_errnrm1_device(const void* e, const void* x1, const void* x2, double atol, double rtol,
                                    long long n, double* scratch, double* result, void* cuda_stream);

/* ---- allocation-free variant ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (code inside a framework that owns the device heap, or a plugin whose
 * allocations are audited) but do own device memory for the outputs: builds
 * the hierarchy tables hs.n, hs.ptr_p1, hs.ptr_m1 (as heomgb_qme_get_hrchy
 * returns them) into caller-owned device buffers of C(n_dim+max_depth,
 * max_depth)*n_dim, (C+1)*n_dim and (C+1)*n_dim ints, enqueued on cuda_stream
 * (NULL: legacy stream); *n_hrchy receives C.  Its scratch (a binomial table)
 * lives in a fixed device array, so n_dim + max_depth + 2 may not exceed
 * HEOMGB_NOALLOC_MAX_BINOM_DIM (HEOMGB_ERR_CAPACITY otherwise).  The first call
 * on a device looks up that array's device address; make it before any stream
 * capture.  The address is kept for the life of the process, so a caller that
 * resets a device (cudaDeviceReset) must not call this entry point on that
 * device afterwards.  All calls share the array: calls that overlap on the GPU
 * race. */
#define HEOMGB_NOALLOC_MAX_BINOM_DIM 96
heomgb_status heomgb_hrchy_build_noalloc(int n_dim, int max_depth, int* n_dev, int* ptr_p1_dev, int* ptr_m1_dev,
                                         int* n_hrchy, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* HEOMGB_H */
