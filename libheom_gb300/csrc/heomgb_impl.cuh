// Internal declarations shared by the kernels (kernels.cu) and the C ABI (api.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <atomic>

#include <cstddef>
#include <cstdint>

struct heomgb_mlp;

namespace heomgb {

// Which epilogue a right-hand-side launch runs after computing D for its elements.
//   DIFF   out = beta*out - alpha*D                        (heom_hilb.h:354-355)
//   RK4_s  classic RK4 stage s, accumulation fused         (solver/rk4.h:40-65)
//   LS     2N-storage RK4 stage                            (solver/lsrk4.h:32-47)
//   DP     Dormand-Prince stage 1..6                       (solver/rkdp.h:111-132)
//   DP7    Dormand-Prince stage 7 + error norm + control   (solver/rkdp.h:136-177)
enum EpiKind : int { EPI_DIFF = 0, EPI_RK4_1, EPI_RK4_2, EPI_RK4_3, EPI_RK4_4, EPI_LS, EPI_DP, EPI_DP7 };

// Device-resident step control state.  The Dormand-Prince controller
// (rkdp.h:150-177, adaptive_step_size_solver.h:45-55) runs on the device in
// the last CTA of the stage-7 launch, so an attempt needs no host round trip.
struct DpCtl {
  double t, dt, t_bound, atol, rtol, err;
  double dt_fixed;          // step of the fixed-step integrators
  int cur;                  // index of the current state buffer (0/1)
  int count;                // attempts in the current step (give up after 1000)
  int done;                 // the output interval is finished
  int status;               // 0 ok; nonzero: numeric failure
  long long attempts, accepted;
  unsigned int arrive;      // CTA arrival counter of the error-norm reduction
  unsigned int pad;
};

// Per-model constants of the right-hand side (all device pointers).
struct RhsModel {
  int n, n2, K, U, n_hrchy;
  int h_real;                       // H has zero imaginary part
  int sqrt_norm;                    // see DiagInst::sqrt_norm
  const int* p1;                    // (n_hrchy+1)*K, sentinel n_hrchy
  const int* m1;                    // (n_hrchy+1)*K
  const int* nidx;                  // n_hrchy*K
  const double2* ngd;               // n_hrchy: sum_k n_k gamma_kk
  const float2* ngd_f;
  const double2* H;                 // n2
  const float2* H_f;
  // diagonal-V path: per element e=(a,b), the modes whose bath couples e,
  // with nonzero coefficients only:
  //   +1 term  c_plus  = i(v_a - v_b) sigma_k                      (plus_ptr/plus_mode)
  //   -1 term  c_minus = i(v_a - v_b) s_k - (v_a + v_b) a_k, x n_k  (minus_ptr/minus_mode)
  const int* plus_ptr;              // n2+1
  const int* plus_mode;
  const int* minus_ptr;             // n2+1
  const int* minus_mode;
  const double2* c_plus;
  const double2* c_minus;
  const float2* c_plus_f;
  const float2* c_minus_f;
  const double2* c_sd;              // n2: sum_u s_delta_u (v_ua - v_ub)^2
  const float2* c_sd_f;
  // general-V and Liouville paths
  const double2* V;                 // U*n2
  const float2* V_f;
  const int* bath_ptr;              // U+1: linear modes of bath u
  const double2* sigma;             // K
  const double2* s;                 // K
  const double2* a;                 // K
  const double2* sdelta;            // U
  const double2* gdiag;             // K: gamma_kk of every linear mode
  const float2* sigma_f;
  const float2* s_f;
  const float2* a_f;
  const float2* sdelta_f;
  // Redfield path: Lambda_u and Lambda_u^dagger (U*n2 each, redfield.h:101-173)
  const double2* lam;
  const float2* lam_f;
  const double2* lamd;
  const float2* lamd_f;
  // Liouville path: CSR superoperators (n2 x n2): R_0 = L + sum_u Xi_u, Phi_u, Psi_u
  const int* r0_ptr;                // n2+1
  const int* r0_idx;
  const double2* r0_val;
  const float2* r0_val_f;
  const int* phi_ptr;               // U*(n2+1), offsets into phi_idx/phi_val
  const int* phi_idx;
  const double2* phi_val;
  const float2* phi_val_f;
  const int* psi_ptr;
  const int* psi_idx;
  const double2* psi_val;
  const float2* psi_val_f;
};

// Arguments of one fused right-hand-side + stage launch.
struct Stage {
  int kind;                  // EpiKind
  int dp_stage;              // EPI_DP: 0..5
  int y_sel;                 // RHS input: 0 y_fixed, 1 Yb[cur], 2 Yb[1-cur]
  int beta_zero;             // EPI_DIFF: beta == 0 (output not read)
  const void* y_fixed;
  double2 alpha, beta;       // EPI_DIFF
  double2* out;              // EPI_DIFF
  DpCtl* ctl;                // dt, cur, reduction state (solver stages)
  double2* S[2];             // FP64 state buffers
  void* Yb[2];               // bulk-precision copies of S (alias S in FP64 mode)
  void* Ynext;               // bulk stage input written by this stage
  double2* acc;              // RK4 accumulator / LSRK4 buffer (FP64)
  void* K[6];                // Dormand-Prince stage vectors (bulk precision)
  double coef;               // LSRK4 stage weight
  int ls_first;              // LSRK4 stage 1 (beta = 0)
  int ls_in;                 // LSRK4 input buffer index
  int bulk_separate;         // Yb are separate (mixed precision) buffers
  double* partials;          // EPI_DP7 per-CTA partial sums
};

enum Path : int { PATH_DIAG = 0, PATH_GENERAL = 1, PATH_LIOU = 2, PATH_REDFIELD = 3 };

// One instance of the diagonal-coupling kernel: a model's sizes, where its
// elements start in the (possibly concatenated) state vector, and its tables.
// A single model is a set of one instance; a batch concatenates many.
struct DiagInst {
  int n, n2, K, nh;
  int h_real;
  int tile;                 // ADOs per CTA tile
  long long elem_off;       // first element of this instance in the state vector
  const int* p1;
  const int* m1;
  const int* nidx;
  const double2* ngd;
  const float2* ngd_f;
  const double2* H;
  const float2* H_f;
  const int* plus_ptr;
  const int* plus_mode;
  const int* minus_ptr;
  const int* minus_mode;
  const double2* c_plus;
  const double2* c_minus;
  const float2* c_plus_f;
  const float2* c_minus_f;
  const double2* c_sd;
  const float2* c_sd_f;
  // learned terminator: predicted rho_{n+1_k} of the tier-N ADOs, row
  // (l - term_first)*K + k, used where ptr_p1 is the sentinel; null = truncation
  const float2* term_p;
  int term_first;
  int sqrt_norm;            // 1: +1 terms scale by sqrt(n_k+1), -1 terms by sqrt(n_k) (else 1 and n_k)
  int h_sym;                // H real and symmetric (the tensor-core commutator's condition)
  int max_terms;            // max over elements of max(+1 terms, -1 terms)
  const int* plus_any;      // per ADO: 1 if any ptr_p1 entry is a real ADO (0 on the deepest tier)
  // FP64 coefficients scaled by the occupation n_k = 0..max_depth (row p*(max_depth+1) + n_k):
  // -1 terms n_k c_minus[p] (sqrt(n_k) c_minus[p] under sqrt normalisation); +1 terms
  // sqrt(n_k + 1) c_plus[p] (sqrt normalisation only, else null)
  const double2* c_minus_n;
  const double2* c_plus_n;
  int occ_rows;             // max_depth + 1
  // Site-local baths (every V_u diagonal with a single nonzero entry, at site
  // s_u; exciton aggregates): per ADO a 16-byte header {occupied modes, 1 if
  // any ptr_p1 entry is a real ADO, ngd_f bits x, y} followed by site_w
  // entries {k, ptr_m1[l][k], n_k, s_u(k)} of its modes with n_k > 0 (in
  // increasing k, real -1 neighbours only); site_cm3 holds per mode k the -1
  // coefficient of an element in its site's row (a == s != b), column
  // (b == s != a) or diagonal (a == b == s), the same values as c_minus_f.
  int site_local;           // 1: the tables below are set
  int site_w;               // entries per ADO (max(1, min(K, max_depth)))
  const int4* site_rec;     // nh * (1 + site_w)
  const float2* site_cm3;   // K * 3
  const float2* site_cp2;   // K * 2: the +1 coefficient of mode k in its site's row / column
  const int* site_ptr;      // n + 1: the modes of site s are site_modes[site_ptr[s] .. site_ptr[s+1])
  const int* site_modes;    // K, per site in increasing k
  const double2* site_cm3_d;  // K * 3 and K * 2: the same coefficients in FP64 (the FP64 resident interval)
  const double2* site_cp2_d;
};
struct DiagTile {
  int inst, l0, nt, pad;
};
struct DiagSet {
  const DiagInst* inst;     // device array
  const DiagTile* tiles;    // device array
  int n_tiles;
  long long total;          // elements over all instances
  size_t smem;              // dynamic shared memory of the largest tile
  int min_blocks;           // 1, 3 or 4: the mixed kernel compiled for 3 (<= 80 registers) or 4 (<= 64) resident 256-thread CTAs
  int tcore;                // 1: micro-tiled commutators on the tensor cores (k_rhs_diag_tc)
  int tmem_cols;            // tensor-memory columns a CTA of k_rhs_diag_tc allocates
  int sites;                // 1: the site-local-bath kernel (k_rhs_sites; one instance, mixed form)
  int sites_tile;           // its ADOs per tile
  int sites_hreal;          // its instance has a real H
  int sites_minb;           // its resident CTAs per SM (2, 3 or 4)
  int sites_rt;             // its rows per register block (4 or 2)
};

// Resident intervals (k_dp_resident: Dormand-Prince; k_rk4_resident and
// k_ls_resident: fixed RK4 / LSRK4 steps): one cooperative launch of CTAs of at most kResidentMaxBlock
// threads, CTA b owning ADOs [b*ados_per_cta, ...).
constexpr int kResidentMaxBlock = 320;
constexpr int kResidentMaxEpt = 2;         // elements per thread (1 or 2, fixed for the interval)
constexpr int kResidentTerms = 8;          // bath-term slots per element: 4 (+1 terms) + 4 (-1 terms)
constexpr int kResidentBarWords = 32;       // grid-barrier counter and flag (64-bit words)
struct ResidentArgs {
  DiagInst inst;            // the model (diagonal coupling, mixed form, one instance)
  DpCtl* ctl;               // controller: initialised before the launch, final state written back
  double2* S[2];            // FP64 states; S[ctl->cur] holds the interval's initial state
  float2* Yb[2];            // FP32 copies of the states (Yb[ctl->cur] valid at launch)
  float2* Ytmp[2];          // stage inputs 2..6 for the neighbour gathers (alternating)
  double* partials;         // per-CTA error-norm partial sums (grid entries)
  unsigned long long* bar;  // grid barrier: kResidentBarWords words, zero at launch (grid_barrier)
  long long n_total;        // elements of the state
  long long max_attempts;   // attempts before the interval gives up (status 3)
  long long n_steps;        // RK4, LSRK4: steps of dt_step before the last step of dt_last
  double dt_step, dt_last;
  int ados_per_cta;
  int skip_arrive_cta;      // fault injection for tests: this CTA never arrives at a grid barrier (-1: none)
  long long spin_limit;     // polls before a grid-barrier wait gives up (2^24 in normal use)
};
// the resident kernels: Dormand-Prince, fixed-step RK4, fixed-step LSRK4
constexpr int kResidentDp = 0, kResidentRk4 = 1, kResidentLs = 2;
constexpr int kResidentRk4F64 = 4;  // fixed-step RK4 in the FP64 form (k_rk4_resident64)
constexpr int kResidentDpF64 = 5;   // Dormand-Prince in the FP64 form, site-local baths (k_dp_resident64)
// k_dp_resident64 (resident64.cu): shared memory of a CTA owning ados_per_cta ADOs, and its kernel instance
size_t resident_dp64_smem(const DiagInst& I, int ados_per_cta);
const void* resident_dp64_kernel(bool hreal, int ept);
// smem of a CTA owning ados_per_cta ADOs in the given scheme's kernel
size_t resident_smem(int n2, int ados_per_cta, int scheme);
int resident_blocks_per_sm(int scheme, bool hreal, int ept, int n, int block, size_t smem);
cudaError_t launch_resident(const ResidentArgs& args, int scheme, bool hreal, int ept, int grid, int block,
                            size_t smem, cudaStream_t s);

// Instance-resident fixed-step RK4 / LSRK4 intervals of a batch (k_fixed_local): CTA b
// holds the whole instances of bin b and runs every step of the interval with
// no grid barrier (its instances' neighbour gathers never leave the CTA): the
// two stage-input copies live in its shared memory, the FP64 state, the RK4
// accumulator and (mixed form) the state's FP32 copy stay in global memory,
// each element touched only by the thread that owns it.  The scheme is
// kResidentRk4 or kResidentLs (the resident kernels' scheme numbers).
constexpr int kLocalMaxInst = 32;   // instances per bin
constexpr int kLocalMaxN2 = 256;    // n_state <= 16 (an element index packs into 8 bits)
constexpr int kLocalMaxAdo = 65535; // ADOs per instance (16 bits)
struct LocalArgs {
  const DiagInst* inst;     // device array of the batch's instances
  const int* bin_ptr;       // bin b holds instances bin_inst[bin_ptr[b] .. bin_ptr[b+1])
  const int* bin_inst;
  double2* S;               // FP64 state (updated in place every step)
  double2* acc;             // RK4 accumulator / LSRK4 buffer (mixed: FP32, the first half)
  float2* Yf;               // mixed form: the state's FP32 copy (the stage-1 input); null in FP64 form
  long long n_steps;        // steps of dt_step before the last step of dt_last
  double dt_step, dt_last;
};
// shared memory of a bin: H of every instance (16-byte rounded), two
// stage-input copies and one packed element descriptor per element
size_t local_bin_smem(const int* n2, const int* nh, int count, bool mixed);
int local_blocks_per_sm(bool mixed, int scheme, int block, size_t smem);
cudaError_t launch_local(const LocalArgs& args, bool mixed, int scheme, int grid, int block, size_t smem,
                         cudaStream_t s);

// Launchers (kernels.cu).  `mixed` selects FP32 bulk arithmetic; `in_double`
// says the RHS input is a double2 array even in mixed mode.  `ds` describes
// the diagonal-coupling work (PATH_DIAG only).
cudaError_t launch_rhs(const RhsModel& m, const DiagSet* ds, const Stage& st, int path, bool mixed, bool in_double,
                       int grid, int block, cudaStream_t s);
int rhs_block_size(const RhsModel& m, int path);
int rhs_grid_size(const RhsModel& m, int path, int block, int n_sm);
size_t rhs_smem_bytes(const RhsModel& m, int path, bool mixed);
size_t diag_tile_smem(int n2, int K, int tile, bool mixed);
// tensor-core variant: shared memory of one tile, ADOs per tile, tensor-memory columns
size_t diag_tile_smem_tc(int n, int K, int tile);
int tc_tile(int n);
int tc_tmem_cols(int n);

// The site-local-bath stage kernel (sites.cu): eligibility, shared memory of
// a CTA, set-up of the per-ADO records, and the launch (mixed form, FP32 stage
// input).
bool sites_eligible(const DiagInst& I, bool mixed);
size_t sites_smem(int n, int K, int tile, int w);
bool sites_variant(int rows, int min_blocks, int block);  // a compiled (rows, CTAs per SM, CTA size) variant
cudaError_t launch_site_records(const DiagInst& I, const int* msite, int4* rec, cudaStream_t s);
cudaError_t launch_sites(const DiagSet& ds, const Stage& st, int grid, int block, cudaStream_t s);

cudaError_t launch_hrchy_build(int K, int depth, int n_hrchy, const long long* binom, int binom_dim, int* nidx,
                               int* p1, int* m1, cudaStream_t s);
cudaError_t launch_ngd(int K, int n_hrchy, const int* nidx, const double2* gdiag, double2* ngd, float2* ngd_f,
                       cudaStream_t s);
cudaError_t launch_to_bulk(const double2* src, float2* dst, long long n, cudaStream_t s);
cudaError_t launch_plus_any(int K, int n_hrchy, const int* p1, int* out, cudaStream_t s);
// out[p*rows + i] = scale(i) * c[p]: scale n (minus, integer), sqrt(n) (minus, sqrt) or sqrt(n+1) (plus, sqrt)
cudaError_t launch_scaled_coef(int n_terms, int rows, const double2* c, double2* out, bool plus, bool sqn,
                               cudaStream_t s);
cudaError_t launch_transpose_ados(const double2* in, double2* out, int n, long long count, cudaStream_t s);
cudaError_t launch_ctl_init(DpCtl* c, double t, double dt, double t_bound, double atol, double rtol, int cur,
                            cudaStream_t s);
cudaError_t launch_ctl_set_fixed(DpCtl* c, double dt, cudaStream_t s);
cudaError_t launch_errnrm1(const double2* e, const double2* x1, const double2* x2, double atol, double rtol,
                           long long n, double* partials, double* out, unsigned int* counter, int grid,
                           cudaStream_t s);
int errnrm1_grid(long long n);
cudaError_t probe_fma_peaks(int n_sm, double* fp64_tflops, double* fp32_tflops, cudaStream_t s);

// BF16 tensor-core GEMM (tcgemm.cu): C[m][n] = sum_k A(m, k) B(n, k) (+ bias[n]),
// FP32 accumulation; an operand element (r, k) is p[r * sm + k * sk], FP32 or BF16.
struct GemmOperand {
  const void* p;
  int bf16;           // 1: BF16 elements, 0: FP32
  long long sm, sk;   // strides (elements) of the row and of k
};
enum GemmEpi : int { GEMM_STORE = 0, GEMM_GELU = 1, GEMM_GELU_GRAD = 2 };
struct GemmArgs {
  GemmOperand a, b;
  float* c;           // M x N, row stride ldc
  long long ldc;
  const float* bias;  // N or null
  float* pre;         // GEMM_GELU: receives the pre-activation (may be null); GEMM_GELU_GRAD: read
  int M, N, K;
  int epi;            // GemmEpi: store; bias + GELU; times gelu'(pre)
  int bn, tmem_cols;  // set by the launcher
  int* err;           // set to 1 if a tensor-core wait ran out
};
cudaError_t launch_gemm_bf16(GemmArgs g, cudaStream_t s);

// Buffers of one terminator inference over the tier-N ADOs [first, first+n_tier).
struct TermBuffers {
  int first = 0, n_tier = 0, n2 = 0, K = 0;
  float* X = nullptr;      // rows x (2 n2 + K)
  float* A1 = nullptr;     // rows x hidden
  float* A2 = nullptr;
  float* Y = nullptr;      // rows x 2 n2
  float* scale = nullptr;  // n_tier
  float2* P = nullptr;     // rows x n2 predictions
};
// Where the terminator reads its input: as a stage kernel picks its own
// (0: y_fixed, 1: yb[cur], 2: yb[1-cur], with cur from ctl).
struct TermInput {
  const void* y_fixed = nullptr;
  const void* yb[2] = {nullptr, nullptr};
  int y_sel = 0;
  const DpCtl* ctl = nullptr;
};
// Model constants the terminator's input features use (device pointers).
struct TermModel {
  int n = 0, K = 0, U = 0;
  const int* nidx = nullptr;      // n_hrchy*K
  const double2* ngd = nullptr;   // n_hrchy
  const double2* gdiag = nullptr; // K: gamma_kk
  const double2* s = nullptr;     // K
  const double2* a = nullptr;     // K
  const double2* sigma = nullptr; // K
  const double2* V = nullptr;     // U*n2
  const int* bath_ptr = nullptr;  // U+1
  // set-up tables of the fused inference (k, e = a n + b): the adiabatic
  // estimate's coefficient -i s_k (v_a - v_b) + a_k (v_a + v_b) and the gain
  // head's sign(Re(v_a - v_b)), for V of mode k's bath
  const float2* cke = nullptr;    // K * n2
  const float* sgn = nullptr;     // K * n2
};
cudaError_t term_enqueue(heomgb_mlp* M, const TermBuffers& tb, const TermModel& tm, const TermInput& in,
                         bool y_float, cudaStream_t s);
// The fused inference (tcgemm.cu): features, three tensor-core layers and the
// gain head of the terminator in one launch.
struct TermMlpArgs {
  TermInput in;
  TermModel tm;
  int first, n_tier, apt;      // tier-N ADOs [first, first + n_tier); ADOs per CTA (apt K <= 128)
  int din, h, dout;
  const __nv_bfloat16* W1;
  const __nv_bfloat16* W2;
  const __nv_bfloat16* W3;
  const float* b1;
  const float* b2;
  const float* b3;
  float2* P;                   // n_tier K rows of n2 predictions
  int* err;                    // set to 1 if a tensor-core wait ran out
};
bool term_fused_ok(int din, int h, int dout, int K);
cudaError_t launch_term_fused(const TermMlpArgs& a, bool y_float, cudaStream_t s);
void mlp_dims(const heomgb_mlp* M, int* din, int* h, int* dout);
// true (and the flag cleared) if a tensor-core GEMM of M's inference gave up a wait
bool mlp_take_error(heomgb_mlp* M, cudaStream_t s);

// Kernels launched (incremented by the launchers and graph replays), safe for
// solvers driven from several host threads: an atomic total plus a per-thread
// count (graph capture measures the kernels of one unit on its own thread).
struct LaunchCounter {
  std::atomic<long long> total{0};
  static long long& mine() {
    thread_local long long c = 0;
    return c;
  }
  void operator++() {
    total.fetch_add(1, std::memory_order_relaxed);
    ++mine();
  }
  void operator+=(long long k) {
    total.fetch_add(k, std::memory_order_relaxed);
    mine() += k;
  }
};
extern LaunchCounter g_launches;

}  // namespace heomgb
