// C ABI of the engine (include/heomgb.h): parameter ingest, device set-up,
// and the solver loops that replay CUDA graphs of fused stage launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "heomgb.h"
#include "heomgb_impl.cuh"

// NVTX ranges around the host-side phases (model set-up, planning and tile
// search, solves, output intervals, graph replays): named regions on a
// profiler's timeline, no-ops without one (the role of the reference's
// CALL_TRACE stack, utility.h:21-25).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

using cd = std::complex<double>;
using namespace heomgb;

namespace {

thread_local std::string g_err;

heomgb_status fail(heomgb_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

struct cuda_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct arg_error : std::invalid_argument {
  using std::invalid_argument::invalid_argument;
};
struct state_error : std::logic_error {
  using std::logic_error::logic_error;
};
struct unsupported_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct numeric_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw cuda_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class F>
heomgb_status guard(F&& f) {
  try {
    f();
    return HEOMGB_OK;
  } catch (const arg_error& e) {
    return fail(HEOMGB_ERR_INVALID_ARGUMENT, e.what());
  } catch (const state_error& e) {
    return fail(HEOMGB_ERR_STATE, e.what());
  } catch (const unsupported_error& e) {
    return fail(HEOMGB_ERR_UNSUPPORTED, e.what());
  } catch (const numeric_error& e) {
    return fail(HEOMGB_ERR_NUMERIC, e.what());
  } catch (const cuda_error& e) {
    return fail(HEOMGB_ERR_CUDA, e.what());
  } catch (const std::bad_alloc&) {
    return fail(HEOMGB_ERR_ALLOC, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(HEOMGB_ERR_INVALID_ARGUMENT, e.what());
  }
}

cd C(const double* p, size_t i) { return cd(p[2 * i], p[2 * i + 1]); }

// Device allocations owned by one object, freed together.
struct DeviceArena {
  std::vector<void*> ptrs;
  void* alloc(size_t bytes) {
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw cuda_error(std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
    }
    ptrs.push_back(p);
    return p;
  }
  template <class T>
  T* upload(const std::vector<T>& v, cudaStream_t s) {
    T* d = static_cast<T*>(alloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty()) ck(cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s), "upload");
    return d;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
  ~DeviceArena() { release(); }
};

// ------------------------------------------------------------------ LIL algebra (set-up only)
// The reference builds its superoperators in std::map-of-map LIL matrices
// (lil_matrix.h.j2:22-183); the same container keeps the summation order and
// the pruning rule of optimize() (entries with |v| <= eps*max are dropped).
using Lil = std::map<int, std::map<int, cd>>;

void lil_optimize(Lil& m) {
  double mx = 0.0;
  for (auto& r : m)
    for (auto& e : r.second) mx = std::max(mx, std::abs(e.second));
  if (mx == 0.0) mx = 1.0;
  const double tol = std::numeric_limits<double>::epsilon() * mx;
  for (auto it = m.begin(); it != m.end();) {
    for (auto jt = it->second.begin(); jt != it->second.end();) {
      if (std::abs(jt->second) <= tol)
        jt = it->second.erase(jt);
      else
        ++jt;
    }
    if (it->second.empty())
      it = m.erase(it);
    else
      ++it;
  }
}

// Y += alpha * (X (x) 1) and Y += alpha * (1 (x) X^T) on row-major vec(rho).
void kron_x_1(const std::vector<cd>& X, int n, cd alpha, Lil& Y) {
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      const cd v = X[r * n + c];
      if (v == cd(0.0, 0.0)) continue;
      const cd p = v * alpha;
      for (int k = 0; k < n; ++k) Y[r * n + k][c * n + k] += p;
    }
}
void kron_1_x_T(const std::vector<cd>& X, int n, cd alpha, Lil& Y) {
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      const cd v = X[r * n + c];
      if (v == cd(0.0, 0.0)) continue;
      const cd p = v * alpha;
      for (int k = 0; k < n; ++k) Y[k * n + c][k * n + r] += p;
    }
}
Lil lil_gemm(cd alpha, const Lil& A, const Lil& B) {
  Lil Cm;
  for (auto& ar : A)
    for (auto& ae : ar.second) {
      auto it = B.find(ae.first);
      if (it == B.end()) continue;
      for (auto& be : it->second) Cm[ar.first][be.first] += alpha * ae.second * be.second;
    }
  lil_optimize(Cm);
  return Cm;
}
void lil_axpy(cd alpha, const Lil& X, Lil& Y) {
  for (auto& r : X)
    for (auto& e : r.second) Y[r.first][e.first] += alpha * e.second;
}
struct Csr {
  std::vector<int> ptr, idx;
  std::vector<cd> val;
};
Csr to_csr(const Lil& m, int rows) {
  Csr c;
  c.ptr.assign(rows + 1, 0);
  for (int r = 0; r < rows; ++r) {
    auto it = m.find(r);
    if (it != m.end())
      for (auto& e : it->second) {
        c.idx.push_back(e.first);
        c.val.push_back(e.second);
      }
    c.ptr[r + 1] = static_cast<int>(c.idx.size());
  }
  return c;
}

std::vector<double2> to_d2(const std::vector<cd>& v) {
  std::vector<double2> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = make_double2(v[i].real(), v[i].imag());
  return o;
}
std::vector<float2> to_f2(const std::vector<cd>& v) {
  std::vector<float2> o(v.size());
  for (size_t i = 0; i < v.size(); ++i)
    o[i] = make_float2(static_cast<float>(v[i].real()), static_cast<float>(v[i].imag()));
  return o;
}

long long binom_sat(long long a, long long b) {
  if (b < 0 || b > a) return 0;
  b = std::min(b, a - b);
  long double r = 1;
  for (long long i = 1; i <= b; ++i) r = r * (a - b + i) / i;
  if (r > static_cast<long double>(LLONG_MAX / 4)) return LLONG_MAX / 4;
  return static_cast<long long>(std::llround(r));
}

struct Bath {
  bool set = false;
  int len = 0;
  std::vector<cd> V, gamma, phi0, sigma, S, A;
  cd sdelta;
};

// Tiles of the diagonal-coupling kernel over a list of instances, with the
// device copies of the instance descriptors and the tile list.
struct DiagPlan {
  std::vector<DiagInst> inst;
  DeviceArena arena;
  DiagSet ds{};
  int block = 128, ept = 4, grid = 1, min_blocks = 1;
  bool tcore = false;  // commutators on the tensor cores (k_rhs_diag_tc)
  bool sites = false;  // the site-local-bath kernel (k_rhs_sites)
};

// Whether an instance can take the tensor-core commutator: mixed form, a
// micro-tiled n_state whose operands fit (n in {8, 12, 16, 24, 32}), real
// symmetric H, no terminator.
bool tcore_eligible(const DiagInst& I, bool mixed) {
  const bool mt4 = (I.n & 3) == 0 && I.n >= 8;
  return mixed && mt4 && I.n <= 32 && I.n != 20 && I.n != 28 && I.h_sym && !I.term_p;
}

void build_plan(DiagPlan& P, const std::vector<DiagInst>& insts, int block, int ept, int min_blocks, bool mixed,
                int n_sm, cudaStream_t s, bool tcore = false, int sites_tile = 0, int sites_rt = 4) {
  P.arena.release();
  P.inst = insts;
  std::vector<DiagTile> tiles;
  size_t smem = 0;
  long long total = 0;
  const size_t cap = 200 * 1024;
  int tmem_cols = 32;
  if (tcore) {
    if (block != 128 && block != 256) throw unsupported_error("tensor-core commutator: 128- or 256-thread CTAs");
    for (const DiagInst& I : insts)
      if (!tcore_eligible(I, mixed)) throw unsupported_error("tensor-core commutator: instance not eligible");
  }
  if (sites_tile > 0) {
    if (insts.size() != 1 || !sites_eligible(insts[0], mixed) || !sites_variant(sites_rt, min_blocks, block))
      throw unsupported_error("site-local-bath kernel: one eligible instance and a compiled variant");
    if (sites_smem(insts[0].n, insts[0].K, sites_tile, insts[0].site_w) > cap)
      throw unsupported_error("site-local-bath tile exceeds shared memory");
    // a thread owns at most one register block of a tile
    if (static_cast<long long>(sites_tile) * (insts[0].n / sites_rt) * (insts[0].n / 4) > block)
      throw unsupported_error("site-local-bath tile: more register blocks than threads");
  }
  for (size_t i = 0; i < P.inst.size(); ++i) {
    DiagInst& I = P.inst[i];
    int tile;
    if (sites_tile > 0) {
      tile = sites_tile;
      smem = sites_smem(I.n, I.K, tile, I.site_w);
    } else if (tcore) {  // the tile is fixed by the GEMM shape (4 n rows per ADO, 128-row blocks)
      tile = tc_tile(I.n);
      if (diag_tile_smem_tc(I.n, I.K, tile) > cap) throw unsupported_error("tensor-core tile exceeds shared memory");
      smem = std::max(smem, diag_tile_smem_tc(I.n, I.K, tile));
      tmem_cols = std::max(tmem_cols, tc_tmem_cols(I.n));
    } else {
      tile = std::max(1, (ept * block) / std::max(1, I.n2));
      while (tile > 1 && diag_tile_smem(I.n2, I.K, tile, mixed) > cap) tile /= 2;
      if (diag_tile_smem(I.n2, I.K, tile, mixed) > cap)
        throw unsupported_error("diagonal-coupling path: one ADO tile exceeds shared memory");
      smem = std::max(smem, diag_tile_smem(I.n2, I.K, tile, mixed));
    }
    I.tile = tile;
    for (int l0 = 0; l0 < I.nh; l0 += tile) tiles.push_back(DiagTile{static_cast<int>(i), l0, std::min(tile, I.nh - l0), 0});
    total = std::max(total, I.elem_off + static_cast<long long>(I.n2) * I.nh);
  }
  P.ds.inst = P.arena.upload(P.inst, s);
  P.ds.tiles = P.arena.upload(tiles, s);
  P.ds.n_tiles = static_cast<int>(tiles.size());
  P.ds.total = total;
  P.ds.smem = smem;
  P.ds.min_blocks = mixed ? min_blocks : 1;
  P.ds.tcore = tcore ? 1 : 0;
  P.ds.tmem_cols = tmem_cols;
  P.ds.sites = sites_tile > 0 ? 1 : 0;
  P.ds.sites_tile = sites_tile;
  P.ds.sites_hreal = (sites_tile > 0 && P.inst[0].h_real) ? 1 : 0;
  P.ds.sites_minb = sites_tile > 0 ? min_blocks : 0;
  P.ds.sites_rt = sites_tile > 0 ? sites_rt : 0;
  P.sites = sites_tile > 0;
  P.tcore = tcore;
  P.block = block;
  P.ept = ept;
  P.min_blocks = P.ds.min_blocks;
  // the site-local-bath kernel loops over tiles with one resident wave (its
  // copies of the next tile overlap the current one); the others take two
  // waves of 2048 threads per SM
  const long long per_sm = sites_tile > 0 ? min_blocks : 2048 / block;
  P.grid = static_cast<int>(std::max<long long>(
      1, std::min<long long>(static_cast<long long>(tiles.size()), static_cast<long long>(n_sm) * per_sm)));
  ck(cudaStreamSynchronize(s), "plan upload");
}

}  // namespace

// ------------------------------------------------------------------ model object
struct heomgb_qme {
  int form = HEOMGB_HILB;
  int max_depth = 0;
  int device = 0;
  int n_sm = 152;
  int n = 0;
  std::vector<cd> H;
  int U = -1;
  std::vector<Bath> baths;
  int precision = HEOMGB_FP64;       // requested
  int sqrt_norm = 0;                 // HEOMGB_NORM_SQRT
  int col_major = 0;                 // HEOMGB_COL_MAJOR: ADOs stored column-major at the boundary
  heomgb_hrchy_filter filter = nullptr;  // hierarchy filter (alloc_hrchy_space's filter_flag)
  void* filter_user = nullptr;
  double2* tx = nullptr;             // col_major transposes of calc_diff (in scratch)
  double2* ty = nullptr;
  int precision_eff = HEOMGB_FP64;   // in use: a MIXED request falls back to FP64 under the range guard
  double range_growth = 0.0;         // range guard inputs (see build_model)
  double range_cancel = 0.0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t user_stream = nullptr;
  bool user_stream_set = false;
  bool ready = false;
  int live_solvers = 0;      // qme_solvers holding device pointers of this model
  // derived
  int K = 0, n_hrchy = 0, path = PATH_DIAG;
  RhsModel dm{};
  DiagInst dinst{};          // diagonal-coupling instance (PATH_DIAG), device pointers into arena
  DiagPlan diff_plan;        // tiles for calc_diff
  heomgb_mlp* term = nullptr;  // learned terminator (not owned); null = plain truncation
  const float2* term_cke = nullptr;  // its set-up tables (TermModel::cke, sgn), in term_arena
  const float* term_sgn = nullptr;
  TermBuffers diff_tb;       // terminator buffers for calc_diff
  DeviceArena term_arena;
  DeviceArena arena;
  DeviceArena scratch;       // calc_diff host-API buffers
  double2* sx = nullptr;
  double2* sy = nullptr;
  cudaStream_t stream() const { return user_stream_set ? user_stream : own_stream; }
  long long main_size() const { return static_cast<long long>(n) * n * n_hrchy; }
};

struct heomgb_solver {
  int kind = HEOMGB_RK4;
};

struct heomgb_qme_solver {
  heomgb_qme* q = nullptr;             // first (or only) model
  std::vector<heomgb_qme*> qmes;       // all models of a batch (one entry otherwise)
  DiagPlan plan;                       // tiles of the diagonal-coupling kernel (autotuned)
  heomgb_mlp* term = nullptr;          // learned terminator of the model, if any
  TermBuffers tb;                      // its per-solver inference buffers
  int kind = HEOMGB_RK4;
  cudaStream_t stream = nullptr;
  bool mixed = false;
  bool separate = false;
  bool col_major = false;              // models store their ADOs column-major
  long long N = 0;
  DeviceArena arena;
  double2* otmp = nullptr;             // boundary transposes of col_major models
  double2* S[2] = {nullptr, nullptr};
  void* Yb[2] = {nullptr, nullptr};
  void* Ytmp[2] = {nullptr, nullptr};
  double2* acc = nullptr;
  void* K[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  DpCtl* ctl = nullptr;
  DpCtl* ctl_host = nullptr;  // pinned mirror
  double* partials = nullptr;
  int grid = 1, block = 32;
  cudaGraphExec_t g_small = nullptr, g_big = nullptr;
  int n_small = 0, n_big = 0;           // steps (fixed) or attempts (DP) per graph
  int nodes_small = 0, nodes_big = 0;
  double dt_save = -1.0;
  long long n_rhs = 0, n_attempts = 0, n_accepted = 0;
  // device time spent inside graph replays of the last solve (CUDA events on
  // the solver stream around every replay batch), and the kernels replayed
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double busy_ms = 0.0;
  bool busy_open = false;  // events of a replay batch recorded, not yet collected
  long long replayed_kernels = 0;
  // resident Dormand-Prince interval (k_dp_resident): one cooperative launch
  // per output interval instead of graph replays of the stage kernels
  bool resident = false;
  int res_grid = 0, res_apc = 0, res_block = 0, res_ept = 2;
  size_t res_smem = 0;
  unsigned long long* res_bar = nullptr;
  double* res_partials = nullptr;
  // instance-resident fixed-step intervals of a batch (k_fixed_local): one launch per
  // output interval, bins of whole instances per CTA, no grid barrier
  bool local = false;
  int loc_grid = 0, loc_block = 0;
  size_t loc_smem = 0;
  DeviceArena loc_arena;
  const int* loc_bin_ptr = nullptr;
  const int* loc_bin_inst = nullptr;
  float stage_ms = 0.f;     // the autotuned stage kernel's time per launch (0: not timed)
  float res_step_ms = 0.f;  // the resident fixed-step plan's time per step (0: not timed)
  // batch solvers run on a stream of their own (sub-batches of one batch run
  // concurrently), ordered after the model stream's pending work at each solve
  cudaStream_t own_stream = nullptr;
  cudaEvent_t user_ready = nullptr;
  ~heomgb_qme_solver() {
    if (g_small) cudaGraphExecDestroy(g_small);
    if (g_big) cudaGraphExecDestroy(g_big);
    if (ctl_host) cudaFreeHost(ctl_host);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (user_ready) cudaEventDestroy(user_ready);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
};

namespace {

void require(bool c, const char* msg) {
  if (!c) throw arg_error(msg);
}

// ------------------------------------------------------------------ set_param
// ------------------------------------------------------------------ Redfield set-up
// Eigen-decomposition of a Hermitian matrix by cyclic Jacobi rotations:
// U^dagger A U = diag(w); U row-major, column k the k-th eigenvector.  Each
// rotation makes a_pq real with a phase factor on column q, then applies the
// real 2x2 rotation that zeroes it.
void hermitian_eigen(std::vector<cd> A, int n, std::vector<double>& w, std::vector<cd>& U) {
  U.assign(static_cast<size_t>(n) * n, cd(0.0, 0.0));
  for (int i = 0; i < n; ++i) U[static_cast<size_t>(i) * n + i] = cd(1.0, 0.0);
  auto at = [&](std::vector<cd>& M, int r, int c) -> cd& { return M[static_cast<size_t>(r) * n + c]; };
  double total = 0.0;
  for (const cd& x : A) total += std::norm(x);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += std::norm(at(A, p, q));
    if (off <= 1e-32 * total) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const cd apq = at(A, p, q);
        const double mag = std::abs(apq);
        if (mag == 0.0) continue;
        const cd phase = apq / mag;
        const double diff = at(A, q, q).real() - at(A, p, p).real();
        const double theta = diff / (2.0 * mag);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        const cd pc = std::conj(phase);
        for (int k = 0; k < n; ++k) {  // columns p, q of A and U
          const cd ap = at(A, k, p), aq = at(A, k, q);
          at(A, k, p) = c * ap - sn * pc * aq;
          at(A, k, q) = sn * ap + c * pc * aq;
          const cd up = at(U, k, p), uq = at(U, k, q);
          at(U, k, p) = c * up - sn * pc * uq;
          at(U, k, q) = sn * up + c * pc * uq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q of A
          const cd ap = at(A, p, k), aq = at(A, q, k);
          at(A, p, k) = c * ap - sn * phase * aq;
          at(A, q, k) = sn * ap + c * phase * aq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = at(A, i, i).real();
}

// x with M x = b (k x k, row-major), Gaussian elimination with partial pivoting.
std::vector<cd> solve_dense(std::vector<cd> M, int k, std::vector<cd> b) {
  for (int i = 0; i < k; ++i) {
    int piv = i;
    for (int r = i + 1; r < k; ++r)
      if (std::abs(M[static_cast<size_t>(r) * k + i]) > std::abs(M[static_cast<size_t>(piv) * k + i])) piv = r;
    if (M[static_cast<size_t>(piv) * k + i] == cd(0.0, 0.0)) throw arg_error("Redfield: singular gamma - i omega");
    if (piv != i) {
      for (int c = 0; c < k; ++c) std::swap(M[static_cast<size_t>(i) * k + c], M[static_cast<size_t>(piv) * k + c]);
      std::swap(b[i], b[piv]);
    }
    for (int r = i + 1; r < k; ++r) {
      const cd f = M[static_cast<size_t>(r) * k + i] / M[static_cast<size_t>(i) * k + i];
      if (f == cd(0.0, 0.0)) continue;
      for (int c = i; c < k; ++c) M[static_cast<size_t>(r) * k + c] -= f * M[static_cast<size_t>(i) * k + c];
      b[r] -= f * b[i];
    }
  }
  for (int i = k - 1; i >= 0; --i) {
    cd acc = b[i];
    for (int c = i + 1; c < k; ++c) acc -= M[static_cast<size_t>(i) * k + c] * b[c];
    b[i] = acc / M[static_cast<size_t>(i) * k + i];
  }
  return b;
}

// Redfield operators of every bath (redfield.h:32-41, 101-173): in the
// eigenbasis of H, Lambda_ij = V_ij C(w_j - w_i) with the bath correlation
// C(omega) = sigma^T (S + iA) (gamma - i omega)^-1 phi_0 + s_delta (the full
// gamma, off-diagonal entries included); back-transformed, concatenated.
void redfield_lambda(const heomgb_qme* q, std::vector<cd>& lam, std::vector<cd>& lamd) {
  const int n = q->n, n2 = n * n;
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b)
      if (std::abs(q->H[static_cast<size_t>(a) * n + b] - std::conj(q->H[static_cast<size_t>(b) * n + a])) >
          1e-12 * (1.0 + std::abs(q->H[static_cast<size_t>(a) * n + b])))
        throw unsupported_error("Redfield models need a Hermitian H");
  std::vector<double> w;
  std::vector<cd> U;
  hermitian_eigen(q->H, n, w, U);
  lam.assign(static_cast<size_t>(q->U) * n2, cd(0.0, 0.0));
  lamd.assign(static_cast<size_t>(q->U) * n2, cd(0.0, 0.0));
  const cd I(0.0, 1.0);
  for (int u = 0; u < q->U; ++u) {
    const Bath& bt = q->baths[u];
    const int L = bt.len;
    std::vector<cd> stc(L, cd(0.0, 0.0));  // sigma^T (S + iA)
    for (int j = 0; j < L; ++j)
      for (int k = 0; k < L; ++k)
        stc[k] += bt.sigma[j] * (bt.S[static_cast<size_t>(j) * L + k] + I * bt.A[static_cast<size_t>(j) * L + k]);
    auto corr = [&](double omega) {
      std::vector<cd> M(bt.gamma.begin(), bt.gamma.end());
      for (int k = 0; k < L; ++k) M[static_cast<size_t>(k) * L + k] -= I * omega;
      const std::vector<cd> x = L > 0 ? solve_dense(M, L, bt.phi0) : std::vector<cd>();
      cd acc = bt.sdelta;
      for (int k = 0; k < L; ++k) acc += stc[k] * x[k];
      return acc;
    };
    // Vv = U^dagger V U, then Lambda_v = Vv o C(w_j - w_i), Lambda = U Lambda_v U^dagger
    std::vector<cd> T(n2, cd(0.0, 0.0)), Vv(n2, cd(0.0, 0.0)), Lv(n2), T2(n2, cd(0.0, 0.0));
    for (int a = 0; a < n; ++a)
      for (int j = 0; j < n; ++j)
        for (int b = 0; b < n; ++b) T[a * n + j] += bt.V[static_cast<size_t>(a) * n + b] * U[static_cast<size_t>(b) * n + j];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int a = 0; a < n; ++a) Vv[i * n + j] += std::conj(U[static_cast<size_t>(a) * n + i]) * T[a * n + j];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) Lv[i * n + j] = Vv[i * n + j] * corr(w[j] - w[i]);
    for (int a = 0; a < n; ++a)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) T2[a * n + j] += U[static_cast<size_t>(a) * n + i] * Lv[i * n + j];
    cd* Lu = lam.data() + static_cast<size_t>(u) * n2;
    cd* LDu = lamd.data() + static_cast<size_t>(u) * n2;
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        cd acc(0.0, 0.0);
        for (int j = 0; j < n; ++j) acc += T2[a * n + j] * std::conj(U[static_cast<size_t>(b) * n + j]);
        Lu[a * n + b] = acc;
      }
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) LDu[a * n + b] = std::conj(Lu[b * n + a]);
  }
}

bool is_redfield(int form) { return form == HEOMGB_REDFIELD_HILB || form == HEOMGB_REDFIELD_LIOU; }

// Hierarchy filter (alloc_hrchy_space with filter_flag, hrchy_space.cc:
// 182-191).  In the breadth-first build every multi-index is spawned by its
// canonical parent n - 1_k, k its last nonzero mode; a candidate the filter
// rejects never enters and spawns nothing.  So an ADO survives when its parent
// survives and the filter accepts it, and the survivors keep their relative
// order.  Walking the full tables in rank order calls the filter on exactly
// the candidates, in the order, that the reference's build does.  The tables
// are then compacted and the +-1 links remapped (void where a neighbour is gone).
void filter_hierarchy(heomgb_qme* q, int K, int nh_full, cudaStream_t s, int*& nidx, int*& p1, int*& m1, int& nh) {
  std::vector<int> n_h(static_cast<size_t>(nh_full) * K), p1_h(static_cast<size_t>(nh_full + 1) * K),
      m1_h(static_cast<size_t>(nh_full + 1) * K);
  ck(cudaMemcpyAsync(n_h.data(), nidx, sizeof(int) * n_h.size(), cudaMemcpyDeviceToHost, s), "tables out");
  ck(cudaMemcpyAsync(p1_h.data(), p1, sizeof(int) * p1_h.size(), cudaMemcpyDeviceToHost, s), "tables out");
  ck(cudaMemcpyAsync(m1_h.data(), m1, sizeof(int) * m1_h.size(), cudaMemcpyDeviceToHost, s), "tables out");
  ck(cudaStreamSynchronize(s), "tables sync");
  std::vector<int> rank(nh_full, -1);
  int cnt = 0;
  rank[0] = cnt++;
  for (int l = 1; l < nh_full; ++l) {
    const int* row = n_h.data() + static_cast<size_t>(l) * K;
    int kmax = K - 1, depth = 0;
    while (row[kmax] == 0) --kmax;
    for (int k = 0; k < K; ++k) depth += row[k];
    const int parent = m1_h[static_cast<size_t>(l) * K + kmax];
    if (rank[parent] < 0) continue;
    if (q->filter(row, K, depth, q->filter_user)) rank[l] = cnt++;
  }
  nh = cnt;
  std::vector<int> n_c(static_cast<size_t>(nh) * K), p1_c(static_cast<size_t>(nh + 1) * K, nh),
      m1_c(static_cast<size_t>(nh + 1) * K, nh);
  for (int l = 0; l < nh_full; ++l) {
    const int r = rank[l];
    if (r < 0) continue;
    for (int k = 0; k < K; ++k) {
      const size_t src = static_cast<size_t>(l) * K + k, dst = static_cast<size_t>(r) * K + k;
      n_c[dst] = n_h[src];
      const int a = p1_h[src], b = m1_h[src];
      p1_c[dst] = a < nh_full && rank[a] >= 0 ? rank[a] : nh;
      m1_c[dst] = b < nh_full && rank[b] >= 0 ? rank[b] : nh;
    }
  }
  nidx = q->arena.upload(n_c, s);
  p1 = q->arena.upload(p1_c, s);
  m1 = q->arena.upload(m1_c, s);
  ck(cudaStreamSynchronize(s), "filtered tables");
}

void build_model(heomgb_qme* q) {
  if (q->n <= 0) throw state_error("set_param: Hamiltonian not set");
  if (q->U < 0) throw state_error("set_param: alloc_noises not called");
  for (int u = 0; u < q->U; ++u)
    if (!q->baths[u].set) throw state_error("set_param: noise " + std::to_string(u) + " not set");
  if (q->live_solvers > 0) throw state_error("set_param: destroy the qme_solvers of this model first");
  ck(cudaSetDevice(q->device), "cudaSetDevice");
  q->arena.release();
  q->term_arena.release();
  q->term = nullptr;  // a rebuilt model starts with plain truncation
  q->diff_tb = TermBuffers{};
  q->ready = false;
  cudaStream_t s = q->stream();
  const int n = q->n, n2 = n * n, U = q->U;
  // linear mode index lk (heom.h:65-74) and per-mode coefficients
  std::vector<int> bath_ptr(U + 1, 0);
  std::vector<cd> sigma, sv, av, gdiag, sdelta;
  for (int u = 0; u < U; ++u) {
    const Bath& b = q->baths[u];
    bath_ptr[u + 1] = bath_ptr[u] + b.len;
    for (int k = 0; k < b.len; ++k) {
      sigma.push_back(b.sigma[k]);
      gdiag.push_back(b.gamma[static_cast<size_t>(k) * b.len + k]);
      // s = S*phi_0, a = A*phi_0 (heom.h:124-138): zero entries skipped, j ascending
      cd s_{0.0, 0.0}, a_{0.0, 0.0};
      for (int j = 0; j < b.len; ++j) {
        const cd Sv = b.S[static_cast<size_t>(k) * b.len + j], Av = b.A[static_cast<size_t>(k) * b.len + j];
        if (Sv != cd(0.0, 0.0)) s_ += Sv * b.phi0[j];
        if (Av != cd(0.0, 0.0)) a_ += Av * b.phi0[j];
      }
      sv.push_back(s_);
      av.push_back(a_);
    }
    sdelta.push_back(b.sdelta);
  }
  const int K = bath_ptr[U];
  // Range guard of the mixed form.  Two properties of the bath expansion
  // decide whether FP32 stage inputs keep rho_0 within ~1e-6 of FP64:
  //   growth:       log10 of how far deep ADOs outgrow rho_0 under the integer
  //                 normalisation, max_k N log10((|s_k| + |a_k|) / |Re gamma_kk|);
  //   cancellation: log10 of sum_k |s_k| / |sum_k s_k| over the modes of one
  //                 bath (large near a Matsubara pole, where the Drude and
  //                 Matsubara coefficients nearly cancel), max over baths.
  // FP32 arithmetic loses rho_0 when the coefficients cancel strongly
  // (cancellation > 0.8), when deep ADOs are huge (growth > 7.5), or when both
  // are moderate (growth > 2 and cancellation > 0.2); such models keep FP64
  // arithmetic.  Measured on a 1024-instance spin-boson/chain sweep (lambda
  // 0.05..5, beta 0.1..10, depth 4..14, RK4 dt 0.005 to t = 20): every
  // instance outside these regions whose FP64 rho_0 stayed physical kept
  // max |delta rho_0| below 5e-7 against FP64.  Storing the coefficients as
  // FP32 hi + lo pairs does not help: emulated, the rounding of the FP32
  // products of cancelling terms dominates.
  {
    double growth = -1e300, cancel = 0.0;
    for (int u = 0; u < U; ++u) {
      double sum_abs = 0.0;
      cd sum(0.0, 0.0);
      for (int k = bath_ptr[u]; k < bath_ptr[u + 1]; ++k) {
        const double r = (std::abs(sv[k]) + std::abs(av[k])) / std::max(std::abs(gdiag[k].real()), 1e-300);
        if (r > 0.0) growth = std::max(growth, q->max_depth * std::log10(r));
        sum_abs += std::abs(sv[k]);
        sum += sv[k];
      }
      if (sum_abs > 0.0) cancel = std::max(cancel, std::abs(sum) > 0.0 ? std::log10(sum_abs / std::abs(sum)) : 300.0);
    }
    q->range_growth = growth < -1e299 ? 0.0 : growth;
    q->range_cancel = cancel;
    const double g = q->range_growth, c = q->range_cancel;
    const bool keep64 = c > 0.8 || g > 7.5 || (g > 2.0 && c > 0.2);
    q->precision_eff = (q->precision == HEOMGB_MIXED && !keep64) ? HEOMGB_MIXED : HEOMGB_FP64;
  }
  const long long count = binom_sat(static_cast<long long>(K) + q->max_depth, q->max_depth);
  if (count > INT_MAX - 1) throw arg_error("hierarchy too large: more than 2^31-2 ADOs");
  if (static_cast<long long>(n2) * count > (1LL << 40)) throw arg_error("state vector too large");
  q->K = K;
  const int nh_full = static_cast<int>(count);

  // hierarchy tables on the device (hrchy_space.cc:137-231)
  DeviceArena full_tables;  // the unfiltered tables when a filter compacts them
  DeviceArena& ta = q->filter ? full_tables : q->arena;
  int* nidx = static_cast<int*>(ta.alloc(sizeof(int) * std::max<size_t>(1, static_cast<size_t>(nh_full) * K)));
  int* p1 = static_cast<int*>(ta.alloc(sizeof(int) * std::max<size_t>(1, static_cast<size_t>(nh_full + 1) * K)));
  int* m1 = static_cast<int*>(ta.alloc(sizeof(int) * std::max<size_t>(1, static_cast<size_t>(nh_full + 1) * K)));
  if (K > 0) {
    const int bd = K + q->max_depth + 2;
    std::vector<long long> bt(static_cast<size_t>(bd) * bd);
    for (int a = 0; a < bd; ++a)
      for (int b = 0; b < bd; ++b) bt[static_cast<size_t>(a) * bd + b] = binom_sat(a, b);
    DeviceArena tmp;
    long long* dbt = tmp.upload(bt, s);
    ck(launch_hrchy_build(K, q->max_depth, nh_full, dbt, bd, nidx, p1, m1, s), "hierarchy build");
    ck(cudaStreamSynchronize(s), "hierarchy build sync");
  }
  int nh = nh_full;
  if (q->filter && K > 0) filter_hierarchy(q, K, nh_full, s, nidx, p1, m1, nh);
  q->n_hrchy = nh;

  RhsModel& m = q->dm;
  m = RhsModel{};
  m.n = n;
  m.n2 = n2;
  m.K = K;
  m.U = U;
  m.n_hrchy = nh;
  m.p1 = p1;
  m.m1 = m1;
  m.nidx = nidx;
  // per-ADO damping sum_k n_k gamma_kk (heom.h:94-104)
  double2* ngd = static_cast<double2*>(q->arena.alloc(sizeof(double2) * nh));
  float2* ngd_f = static_cast<float2*>(q->arena.alloc(sizeof(float2) * nh));
  if (K > 0) {
    DeviceArena tmp;
    double2* dg = tmp.upload(to_d2(gdiag), s);
    ck(launch_ngd(K, nh, nidx, dg, ngd, ngd_f, s), "ngamma");
    ck(cudaStreamSynchronize(s), "ngamma sync");
  } else {
    ck(cudaMemsetAsync(ngd, 0, sizeof(double2) * nh, s), "memset");
    ck(cudaMemsetAsync(ngd_f, 0, sizeof(float2) * nh, s), "memset");
  }
  m.ngd = ngd;
  m.ngd_f = ngd_f;

  // constants
  bool h_real = true;
  for (const cd& v : q->H) h_real = h_real && v.imag() == 0.0;
  m.h_real = h_real ? 1 : 0;
  m.sqrt_norm = q->sqrt_norm;
  m.H = q->arena.upload(to_d2(q->H), s);
  m.H_f = q->arena.upload(to_f2(q->H), s);
  std::vector<cd> Vall;
  bool diag = true;
  for (int u = 0; u < U; ++u) {
    const Bath& b = q->baths[u];
    Vall.insert(Vall.end(), b.V.begin(), b.V.end());
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c)
        if (r != c && b.V[static_cast<size_t>(r) * n + c] != cd(0.0, 0.0)) diag = false;
  }
  m.V = q->arena.upload(to_d2(Vall), s);
  m.V_f = q->arena.upload(to_f2(Vall), s);
  m.bath_ptr = q->arena.upload(bath_ptr, s);
  m.sigma = q->arena.upload(to_d2(sigma), s);
  m.s = q->arena.upload(to_d2(sv), s);
  m.a = q->arena.upload(to_d2(av), s);
  m.sdelta = q->arena.upload(to_d2(sdelta), s);
  m.gdiag = q->arena.upload(to_d2(gdiag), s);
  m.sigma_f = q->arena.upload(to_f2(sigma), s);
  m.s_f = q->arena.upload(to_f2(sv), s);
  m.a_f = q->arena.upload(to_f2(av), s);
  m.sdelta_f = q->arena.upload(to_f2(sdelta), s);

  if (is_redfield(q->form)) {
    // redfield_hilb and redfield_liou apply the same operator; one kernel serves both
    q->path = PATH_REDFIELD;
    if (rhs_smem_bytes(m, PATH_REDFIELD, false) > 200 * 1024)
      throw unsupported_error("Redfield path supports n_level <= 66");
    std::vector<cd> lam, lamd;
    redfield_lambda(q, lam, lamd);
    m.lam = q->arena.upload(to_d2(lam), s);
    m.lam_f = q->arena.upload(to_f2(lam), s);
    m.lamd = q->arena.upload(to_d2(lamd), s);
    m.lamd_f = q->arena.upload(to_f2(lamd), s);
  } else if (q->form == HEOMGB_HILB) {
    q->path = diag ? PATH_DIAG : PATH_GENERAL;
  } else {
    q->path = PATH_LIOU;
  }
  if (q->path == PATH_DIAG) {
    // per-element active modes of the elementwise bath terms
    std::vector<int> pp(n2 + 1, 0), pm(n2 + 1, 0), pmode, mmode;
    std::vector<cd> cp, cmn, csd(n2, cd(0.0, 0.0));
    const cd I(0.0, 1.0);
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        const int e = a * n + b;
        for (int u = 0; u < U; ++u) {
          const Bath& B = q->baths[u];
          const cd va = B.V[static_cast<size_t>(a) * n + a], vb = B.V[static_cast<size_t>(b) * n + b];
          const cd cphi = I * (va - vb), cpsi = va + vb;
          csd[e] += B.sdelta * (va - vb) * (va - vb);
          for (int k = bath_ptr[u]; k < bath_ptr[u + 1]; ++k) {
            const cd c1 = cphi * sigma[k];
            if (c1 != cd(0.0, 0.0)) {
              pmode.push_back(k);
              cp.push_back(c1);
            }
            const cd c2 = cphi * sv[k] - cpsi * av[k];
            if (c2 != cd(0.0, 0.0)) {
              mmode.push_back(k);
              cmn.push_back(c2);
            }
          }
        }
        pp[e + 1] = static_cast<int>(pmode.size());
        pm[e + 1] = static_cast<int>(mmode.size());
      }
    int max_terms = 0;
    for (int e = 0; e < n2; ++e) max_terms = std::max({max_terms, pp[e + 1] - pp[e], pm[e + 1] - pm[e]});
    m.plus_ptr = q->arena.upload(pp, s);
    m.plus_mode = q->arena.upload(pmode, s);
    m.minus_ptr = q->arena.upload(pm, s);
    m.minus_mode = q->arena.upload(mmode, s);
    m.c_plus = q->arena.upload(to_d2(cp), s);
    m.c_minus = q->arena.upload(to_d2(cmn), s);
    m.c_plus_f = q->arena.upload(to_f2(cp), s);
    m.c_minus_f = q->arena.upload(to_f2(cmn), s);
    m.c_sd = q->arena.upload(to_d2(csd), s);
    m.c_sd_f = q->arena.upload(to_f2(csd), s);
    DiagInst& di = q->dinst;
    di = DiagInst{};
    di.n = n;
    di.n2 = n2;
    di.K = K;
    di.nh = nh;
    di.h_real = m.h_real;
    {
      bool sym = m.h_real != 0;
      for (int a = 0; a < n && sym; ++a)
        for (int b = 0; b < a && sym; ++b) sym = q->H[static_cast<size_t>(a) * n + b] == q->H[static_cast<size_t>(b) * n + a];
      di.h_sym = sym ? 1 : 0;
    }
    di.sqrt_norm = m.sqrt_norm;
    di.max_terms = max_terms;
    di.elem_off = 0;
    di.p1 = m.p1;
    di.m1 = m.m1;
    di.nidx = m.nidx;
    di.ngd = m.ngd;
    di.ngd_f = m.ngd_f;
    di.H = m.H;
    di.H_f = m.H_f;
    di.plus_ptr = m.plus_ptr;
    di.plus_mode = m.plus_mode;
    di.minus_ptr = m.minus_ptr;
    di.minus_mode = m.minus_mode;
    di.c_plus = m.c_plus;
    di.c_minus = m.c_minus;
    di.c_plus_f = m.c_plus_f;
    di.c_minus_f = m.c_minus_f;
    di.c_sd = m.c_sd;
    di.c_sd_f = m.c_sd_f;
    int* plus_any = static_cast<int*>(q->arena.alloc(sizeof(int) * std::max(nh, 1)));
    if (K > 0)
      ck(launch_plus_any(K, nh, m.p1, plus_any, s), "plus_any");
    else
      ck(cudaMemsetAsync(plus_any, 0, sizeof(int) * std::max(nh, 1), s), "memset");
    di.plus_any = plus_any;
    // the FP64 coefficients scaled by every occupation (the FP64 kernels' per-term products, tabulated)
    di.occ_rows = q->max_depth + 1;
    const int n_plus = static_cast<int>(cp.size()), n_minus = static_cast<int>(cmn.size());
    double2* cmn_n = static_cast<double2*>(q->arena.alloc(sizeof(double2) * std::max<size_t>(1, static_cast<size_t>(n_minus) * di.occ_rows)));
    ck(launch_scaled_coef(n_minus, di.occ_rows, m.c_minus, cmn_n, false, m.sqrt_norm != 0, s), "scaled coefficients");
    di.c_minus_n = cmn_n;
    di.c_plus_n = nullptr;
    if (m.sqrt_norm) {
      double2* cp_n = static_cast<double2*>(q->arena.alloc(sizeof(double2) * std::max<size_t>(1, static_cast<size_t>(n_plus) * di.occ_rows)));
      ck(launch_scaled_coef(n_plus, di.occ_rows, m.c_plus, cp_n, true, true, s), "scaled coefficients");
      di.c_plus_n = cp_n;
    }
    // site-local baths (every V_u diagonal with a single nonzero entry, at site
    // s_u): the -1 coefficients of an element in the row, column or diagonal
    // of s_u, formed as the per-element table above forms them, and the
    // per-ADO records of occupied modes (k_rhs_sites)
    {
      std::vector<int> usite(U, -1);
      bool site_local = U > 0 && K > 0;
      for (int u = 0; u < U && site_local; ++u) {
        int cnt = 0;
        for (int a = 0; a < n; ++a)
          if (q->baths[u].V[static_cast<size_t>(a) * n + a] != cd(0.0, 0.0)) {
            ++cnt;
            usite[u] = a;
          }
        site_local = cnt == 1;
      }
      if (site_local) {
        std::vector<int> msite(K, 0);
        std::vector<cd> cm3(3 * static_cast<size_t>(K));
        for (int u = 0; u < U; ++u) {
          const cd v = q->baths[u].V[static_cast<size_t>(usite[u]) * n + usite[u]], zero(0.0, 0.0);
          const cd vas[3] = {v, zero, v}, vbs[3] = {zero, v, v};  // row, column, diagonal of the site
          for (int k = bath_ptr[u]; k < bath_ptr[u + 1]; ++k) {
            msite[k] = usite[u];
            for (int c = 0; c < 3; ++c) {
              const cd cphi = I * (vas[c] - vbs[c]), cpsi = vas[c] + vbs[c];
              cm3[3 * static_cast<size_t>(k) + c] = cphi * sv[k] - cpsi * av[k];
            }
          }
        }
        // the +1 coefficient i (v_a - v_b) sigma_k for the row and column cases, and
        // the modes of every site in increasing k
        std::vector<cd> cp2(2 * static_cast<size_t>(K));
        std::vector<int> sptr(n + 1, 0), smodes;
        for (int u = 0; u < U; ++u) {
          const cd v = q->baths[u].V[static_cast<size_t>(usite[u]) * n + usite[u]], zero(0.0, 0.0);
          for (int k = bath_ptr[u]; k < bath_ptr[u + 1]; ++k) {
            cp2[2 * static_cast<size_t>(k)] = I * (v - zero) * sigma[k];
            cp2[2 * static_cast<size_t>(k) + 1] = I * (zero - v) * sigma[k];
          }
        }
        for (int site = 0; site < n; ++site) {
          for (int k = 0; k < K; ++k)
            if (msite[k] == site) smodes.push_back(k);
          sptr[site + 1] = static_cast<int>(smodes.size());
        }
        di.site_local = 1;
        di.site_w = std::max(1, std::min(K, q->max_depth));
        const int* dms = q->arena.upload(msite, s);
        di.site_cm3 = q->arena.upload(to_f2(cm3), s);
        di.site_cp2 = q->arena.upload(to_f2(cp2), s);
        di.site_cm3_d = q->arena.upload(to_d2(cm3), s);
        di.site_cp2_d = q->arena.upload(to_d2(cp2), s);
        di.site_ptr = q->arena.upload(sptr, s);
        di.site_modes = q->arena.upload(smodes, s);
        int4* rec = static_cast<int4*>(q->arena.alloc(sizeof(int4) * static_cast<size_t>(nh) * (1 + di.site_w)));
        di.site_rec = rec;
        ck(launch_site_records(di, dms, rec, s), "site records");
        ck(cudaStreamSynchronize(s), "site records sync");
      }
    }
    build_plan(q->diff_plan, {di}, 128, 4, 1, q->precision_eff == HEOMGB_MIXED, q->n_sm, s);
  } else if (q->path == PATH_GENERAL) {
    if (rhs_smem_bytes(m, PATH_GENERAL, false) > 200 * 1024)
      throw unsupported_error("general-V Hilbert path supports n_level <= 50");
  } else {
    if (rhs_smem_bytes(m, PATH_LIOU, false) > 200 * 1024)
      throw unsupported_error("Liouville path supports n_level <= 56");
    // superoperators (heom_liou.h:71-99)
    const cd I(0.0, 1.0), one(1.0, 0.0);
    Lil L;
    kron_x_1(q->H, n, I, L);
    kron_1_x_T(q->H, n, -I, L);
    Lil R0;
    lil_axpy(one, L, R0);
    std::vector<int> phi_ptr, phi_idx, psi_ptr, psi_idx;
    std::vector<cd> phi_val, psi_val;
    std::vector<Lil> Xi(U);
    for (int u = 0; u < U; ++u) {
      Lil Phi, Psi;
      kron_x_1(q->baths[u].V, n, I, Phi);
      kron_1_x_T(q->baths[u].V, n, -I, Phi);
      lil_optimize(Phi);
      kron_x_1(q->baths[u].V, n, one, Psi);
      kron_1_x_T(q->baths[u].V, n, one, Psi);
      lil_optimize(Psi);
      Xi[u] = lil_gemm(-q->baths[u].sdelta, Phi, Phi);
      Csr cph = to_csr(Phi, n2), cps = to_csr(Psi, n2);
      const int off_ph = static_cast<int>(phi_idx.size()), off_ps = static_cast<int>(psi_idx.size());
      for (int r = 0; r <= n2; ++r) {
        phi_ptr.push_back(off_ph + cph.ptr[r]);
        psi_ptr.push_back(off_ps + cps.ptr[r]);
      }
      phi_idx.insert(phi_idx.end(), cph.idx.begin(), cph.idx.end());
      phi_val.insert(phi_val.end(), cph.val.begin(), cph.val.end());
      psi_idx.insert(psi_idx.end(), cps.idx.begin(), cps.idx.end());
      psi_val.insert(psi_val.end(), cps.val.begin(), cps.val.end());
    }
    for (int u = 0; u < U; ++u) lil_axpy(one, Xi[u], R0);
    Csr cr0 = to_csr(R0, n2);
    m.r0_ptr = q->arena.upload(cr0.ptr, s);
    m.r0_idx = q->arena.upload(cr0.idx, s);
    m.r0_val = q->arena.upload(to_d2(cr0.val), s);
    m.r0_val_f = q->arena.upload(to_f2(cr0.val), s);
    m.phi_ptr = q->arena.upload(phi_ptr, s);
    m.phi_idx = q->arena.upload(phi_idx, s);
    m.phi_val = q->arena.upload(to_d2(phi_val), s);
    m.phi_val_f = q->arena.upload(to_f2(phi_val), s);
    m.psi_ptr = q->arena.upload(psi_ptr, s);
    m.psi_idx = q->arena.upload(psi_idx, s);
    m.psi_val = q->arena.upload(to_d2(psi_val), s);
    m.psi_val_f = q->arena.upload(to_f2(psi_val), s);
  }
  ck(cudaStreamSynchronize(s), "set_param sync");
  q->ready = true;
}

void need_ready(const heomgb_qme* q) {
  if (!q) throw arg_error("null qme");
  if (!q->ready) throw state_error("set_param has not completed");
}

Stage base_stage() {
  Stage st;
  std::memset(&st, 0, sizeof(st));
  return st;
}

// Inference buffers of the terminator for the tier-N ADOs of q (the last
// C(K+N-1, N) ADOs in the breadth-first order).
void alloc_term(DeviceArena& A, const heomgb_qme* q, TermBuffers& tb) {
  int din = 0, h = 0, dout = 0;
  mlp_dims(q->term, &din, &h, &dout);
  const int K = q->K, N = q->max_depth;
  const long long n_tier = N == 0 ? 1 : binom_sat(static_cast<long long>(K) + N - 1, N);
  tb = TermBuffers{};
  tb.n_tier = static_cast<int>(n_tier);
  tb.first = q->n_hrchy - tb.n_tier;
  tb.n2 = q->n * q->n;
  tb.K = K;
  const size_t R = static_cast<size_t>(tb.n_tier) * K;
  tb.X = static_cast<float*>(A.alloc(sizeof(float) * R * din));
  tb.A1 = static_cast<float*>(A.alloc(sizeof(float) * R * h));
  tb.A2 = static_cast<float*>(A.alloc(sizeof(float) * R * h));
  tb.Y = static_cast<float*>(A.alloc(sizeof(float) * R * dout));
  tb.scale = static_cast<float*>(A.alloc(sizeof(float) * tb.n_tier));
  tb.P = static_cast<float2*>(A.alloc(sizeof(float2) * R * tb.n2));
}

TermModel term_model(const heomgb_qme* q) {
  TermModel tm;
  tm.n = q->n;
  tm.K = q->K;
  tm.U = q->U;
  tm.nidx = q->dm.nidx;
  tm.ngd = q->dm.ngd;
  tm.gdiag = q->dm.gdiag;
  tm.s = q->dm.s;
  tm.a = q->dm.a;
  tm.sigma = q->dm.sigma;
  tm.V = q->dm.V;
  tm.bath_ptr = q->dm.bath_ptr;
  tm.cke = q->term_cke;
  tm.sgn = q->term_sgn;
  return tm;
}

void run_diff_rm(heomgb_qme* q, double2* drho, const double2* rho, const double* alpha, const double* beta);

// calc_diff in the model's storage order: a col_major model sees its ADOs
// transposed into row-major scratch and the result transposed back.
void run_diff(heomgb_qme* q, double2* drho, const double2* rho, const double* alpha, const double* beta) {
  if (!q->col_major) {
    run_diff_rm(q, drho, rho, alpha, beta);
    return;
  }
  cudaStream_t s = q->stream();
  if (!q->tx) {
    const size_t bytes = sizeof(double2) * q->main_size();
    q->tx = static_cast<double2*>(q->scratch.alloc(bytes));
    q->ty = static_cast<double2*>(q->scratch.alloc(bytes));
  }
  const bool beta_zero = !beta || (beta[0] == 0.0 && beta[1] == 0.0);
  ck(launch_transpose_ados(rho, q->tx, q->n, q->n_hrchy, s), "transpose in");
  if (!beta_zero) ck(launch_transpose_ados(drho, q->ty, q->n, q->n_hrchy, s), "transpose in");
  run_diff_rm(q, q->ty, q->tx, alpha, beta);
  ck(launch_transpose_ados(q->ty, drho, q->n, q->n_hrchy, s), "transpose out");
}

void run_diff_rm(heomgb_qme* q, double2* drho, const double2* rho, const double* alpha, const double* beta) {
  Stage st = base_stage();
  st.kind = EPI_DIFF;
  st.y_sel = 0;
  st.y_fixed = rho;
  st.out = drho;
  st.alpha = make_double2(alpha ? alpha[0] : 1.0, alpha ? alpha[1] : 0.0);
  st.beta = make_double2(beta ? beta[0] : 0.0, beta ? beta[1] : 0.0);
  st.beta_zero = (st.beta.x == 0.0 && st.beta.y == 0.0) ? 1 : 0;
  const bool diag = q->path == PATH_DIAG;
  if (q->term) {
    TermInput in;
    in.y_fixed = rho;
    ck(term_enqueue(q->term, q->diff_tb, term_model(q), in, false, q->stream()), "terminator");
  }
  const int block = diag ? q->diff_plan.block : rhs_block_size(q->dm, q->path);
  const int grid = diag ? q->diff_plan.grid : rhs_grid_size(q->dm, q->path, block, q->n_sm);
  ck(launch_rhs(q->dm, diag ? &q->diff_plan.ds : nullptr, st, q->path, q->precision_eff == HEOMGB_MIXED, true, grid,
                block, q->stream()),
     "calc_diff");
}

// ------------------------------------------------------------------ solvers
void autotune(heomgb_qme_solver* qs);
void plan_resident(heomgb_qme_solver* qs);
void plan_local(heomgb_qme_solver* qs);

// The resident kernel of the solver's scheme.
int resident_scheme(const heomgb_qme_solver* qs) {
  return qs->kind == HEOMGB_RK4 ? kResidentRk4 : qs->kind == HEOMGB_LSRK4 ? kResidentLs : kResidentDp;
}

// The resident kernel variant of the solver: the scheme in the mixed form,
// k_rk4_resident64 for fixed-step RK4 in the FP64 form, -1 where none exists.
int resident_variant(const heomgb_qme_solver* qs) {
  const int scheme = resident_scheme(qs);
  if (qs->mixed) return scheme;
  if (scheme == kResidentRk4) return kResidentRk4F64;
  // the FP64 Dormand-Prince interval reads the site-local records
  if (scheme == kResidentDp && qs->q->dinst.site_local && qs->q->dinst.site_rec) return kResidentDpF64;
  return -1;
}

// Arguments of the resident kernels for the solver's buffers and its tuned shape.
ResidentArgs resident_args(heomgb_qme_solver* qs) {
  ResidentArgs a{};
  a.inst = qs->q->dinst;
  a.ctl = qs->ctl;
  for (int i = 0; i < 2; ++i) {
    a.S[i] = qs->S[i];
    a.Yb[i] = static_cast<float2*>(qs->Yb[i]);
    a.Ytmp[i] = static_cast<float2*>(qs->Ytmp[i]);
  }
  a.partials = qs->res_partials;
  a.bar = qs->res_bar;
  a.n_total = qs->N;
  a.max_attempts = 2000000LL;
  a.n_steps = 0;
  a.dt_step = a.dt_last = 0.0;
  a.ados_per_cta = qs->res_apc;
  // Fault injection for the tests of the bounded waits: HEOMGB_FAULT_SKIP_ARRIVAL=<cta>
  // makes that CTA skip its grid-barrier arrivals, HEOMGB_FAULT_SPIN_LIMIT=<polls>
  // shortens every wait; the waits then run out, the CTAs leave and the solve
  // reports HEOMGB_ERR_CUDA.  Neither is set in normal use.
  a.skip_arrive_cta = -1;
  a.spin_limit = 1LL << 24;
  if (const char* env = std::getenv("HEOMGB_FAULT_SKIP_ARRIVAL")) a.skip_arrive_cta = std::atoi(env);
  if (const char* env = std::getenv("HEOMGB_FAULT_SPIN_LIMIT"))
    a.spin_limit = std::max(1LL, std::min(1LL << 24, std::atoll(env)));
  return a;
}
Stage solver_stage(heomgb_qme_solver* qs);

void alloc_solver(heomgb_qme_solver* qs) {
  heomgb_qme* q = qs->q;
  long long N = 0;
  for (heomgb_qme* m : qs->qmes) N += m->main_size();
  qs->N = N;
  qs->mixed = q->precision_eff == HEOMGB_MIXED;
  qs->col_major = q->col_major != 0;
  qs->separate = qs->mixed;
  const size_t bd = sizeof(double2) * N;
  const size_t bb = (qs->mixed ? sizeof(float2) : sizeof(double2)) * N;
  auto& A = qs->arena;
  const int nstate = qs->kind == HEOMGB_RK4 ? 1 : 2;
  for (int i = 0; i < nstate; ++i) {
    qs->S[i] = static_cast<double2*>(A.alloc(bd));
    qs->Yb[i] = qs->separate ? A.alloc(bb) : static_cast<void*>(qs->S[i]);
  }
  if (qs->kind == HEOMGB_RK4 || qs->kind == HEOMGB_RKDP) {
    qs->Ytmp[0] = A.alloc(bb);
    qs->Ytmp[1] = A.alloc(bb);
  }
  if (qs->kind == HEOMGB_RK4 || qs->kind == HEOMGB_LSRK4) qs->acc = static_cast<double2*>(A.alloc(bd));
  if (qs->col_major) qs->otmp = static_cast<double2*>(A.alloc(bd));
  if (qs->kind == HEOMGB_RKDP)
    for (int i = 0; i < 6; ++i) qs->K[i] = A.alloc(bb);
  qs->ctl = static_cast<DpCtl*>(A.alloc(sizeof(DpCtl)));
  ck(cudaMemsetAsync(qs->ctl, 0, sizeof(DpCtl), qs->stream), "memset ctl");
  ck(cudaMallocHost(reinterpret_cast<void**>(&qs->ctl_host), sizeof(DpCtl)), "cudaMallocHost");
  ck(cudaEventCreate(&qs->ev0), "event create");
  ck(cudaEventCreate(&qs->ev1), "event create");
  qs->term = q->term;
  if (qs->term) {
    if (qs->qmes.size() != 1) throw unsupported_error("the learned terminator is not available in batches");
    alloc_term(qs->arena, q, qs->tb);
  }
  if (q->path == PATH_DIAG) {
    autotune(qs);
    qs->block = qs->plan.block;
    qs->grid = qs->plan.grid;
  } else {
    qs->block = rhs_block_size(q->dm, q->path);
    qs->grid = rhs_grid_size(q->dm, q->path, qs->block, q->n_sm);
  }
  qs->partials = static_cast<double*>(A.alloc(sizeof(double) * std::max(qs->grid, 1)));
  plan_resident(qs);
  plan_local(qs);
}

// Tile shape search for the diagonal-coupling kernel: CTA size x elements per
// thread (which sets ADOs per tile), timed on right-hand-side launches over
// the solver's own buffers; the fastest shape is kept for the captured graphs.
void autotune(heomgb_qme_solver* qs) {
  const NvtxRange range("heomgb plan: tile search");
  heomgb_qme* q = qs->q;
  std::vector<DiagInst> insts;
  long long off = 0;
  for (heomgb_qme* m : qs->qmes) {
    DiagInst I = m->dinst;
    I.term_p = qs->term ? qs->tb.P : nullptr;
    I.term_first = qs->term ? qs->tb.first : 0;
    I.elem_off = off;
    off += m->main_size();
    insts.push_back(I);
  }
  // Timed on a representative stage of the solver itself (its epilogue
  // traffic shapes the best tile as much as the right-hand side does) over
  // zeroed buffers with the controller idle (dt = 0): RK4 stage 2, an LSRK4
  // middle stage, or Dormand-Prince stage 4.
  const size_t bd = sizeof(double2) * qs->N, bb = (qs->separate ? sizeof(float2) : sizeof(double2)) * qs->N;
  for (double2* p : {qs->S[0], qs->S[1], qs->acc})
    if (p) ck(cudaMemsetAsync(p, 0, bd, qs->stream), "memset");
  for (void* p : {qs->Yb[0], qs->Yb[1], qs->Ytmp[0], qs->Ytmp[1], qs->K[0], qs->K[1], qs->K[2], qs->K[3]})
    if (p) ck(cudaMemsetAsync(p, 0, bb, qs->stream), "memset");
  Stage st = solver_stage(qs);
  if (qs->kind == HEOMGB_RK4) {
    st.kind = EPI_RK4_2;
    st.y_fixed = qs->Ytmp[0];
    st.Ynext = qs->Ytmp[1];
  } else if (qs->kind == HEOMGB_LSRK4) {
    st.kind = EPI_LS;
    st.ls_in = 1;
    st.ls_first = 0;
    st.coef = 0.75;
    st.y_fixed = qs->Yb[1];
  } else {
    st.kind = EPI_DP;
    st.dp_stage = 3;
    st.y_fixed = qs->Ytmp[0];
    st.Ynext = qs->Ytmp[1];
  }
  st.y_sel = 0;
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "event");
  ck(cudaEventCreate(&e1), "event");
  float best = 1e30f;
  int best_b = 128, best_e = 4, best_m = 1;
  // HEOMGB_TILE=<block>x<elements per thread>[x<min blocks>] pins the shape
  // (reproducible profiles: a profiler's replay distorts the timings the
  // search relies on)
  int pin_b = 0, pin_e = 0, pin_m = 1;
  bool pin_tc = false;
  int pin_sb = 0, pin_st = 0, pin_sm = 0, pin_sr = 0;  // HEOMGB_TILE=sites:<block>x<tile>x<CTAs per SM>[x<rows>]
  if (const char* env = std::getenv("HEOMGB_TILE")) {
    if (std::string(env) == "tc") {
      pin_tc = true;
    } else if (std::string(env).rfind("sites:", 0) == 0) {
      const int got = std::sscanf(env + 6, "%dx%dx%dx%d", &pin_sb, &pin_st, &pin_sm, &pin_sr);
      if (got == 3) pin_sr = (pin_sm == 2 && pin_sb <= 256) ? 4 : 2;
      if (got < 3 || pin_sb % 32 || pin_st < 1 || pin_st > 16 || !sites_variant(pin_sr, pin_sm, pin_sb))
        throw arg_error("HEOMGB_TILE=sites:<block>x<1..16 ADOs per tile>x<CTAs per SM>[x<rows 4|2>]: 4 rows with "
                        "2 CTAs of <= 256 threads; 2 rows with 3 or 4 CTAs of <= 256 or 2 CTAs of 288..384");
    } else {
      const int got = std::sscanf(env, "%dx%dx%d", &pin_b, &pin_e, &pin_m);
      if (got < 2 || (pin_b != 64 && pin_b != 128 && pin_b != 256) || pin_e < 1 || pin_e > 8 ||
          (pin_m != 1 && pin_m != 3 && pin_m != 4))
        throw arg_error("HEOMGB_TILE must be tc or <64|128|256>x<1..8>[x<1|3|4>]");
    }
  }
  // the tensor-core commutator joins the search where every instance is
  // eligible; HEOMGB_TCORE=0 keeps it out
  bool tc_ok = qs->mixed;
  for (const DiagInst& I : insts) tc_ok = tc_ok && tcore_eligible(I, qs->mixed);
  if (const char* env = std::getenv("HEOMGB_TCORE"))
    if (std::string(env) == "0") tc_ok = false;
  if (pin_tc && !tc_ok) throw unsupported_error("HEOMGB_TILE=tc: the tensor-core commutator does not apply");
  bool best_tc = false;
  // one warm-up launch, then the best of two timed groups of three launches
  // (a single group let run-to-run noise pick shapes a few percent slower)
  auto time_plan = [&](int b) {
    const bool in_double = !qs->separate;
    ck(launch_rhs(q->dm, &qs->plan.ds, st, PATH_DIAG, qs->mixed, in_double, qs->plan.grid, b, qs->stream), "tune");
    float best_ms = 1e30f;
    for (int g = 0; g < 2; ++g) {
      ck(cudaEventRecord(e0, qs->stream), "event");
      for (int r = 0; r < 3; ++r)
        ck(launch_rhs(q->dm, &qs->plan.ds, st, PATH_DIAG, qs->mixed, in_double, qs->plan.grid, b, qs->stream),
           "tune");
      ck(cudaEventRecord(e1, qs->stream), "event");
      ck(cudaEventSynchronize(e1), "event sync");
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, e0, e1), "event time");
      best_ms = std::min(best_ms, ms);
    }
    return best_ms;
  };
  // HEOMGB_TUNE_LOG=1 prints every timed candidate to stderr
  const bool tune_log = std::getenv("HEOMGB_TUNE_LOG") && std::string(std::getenv("HEOMGB_TUNE_LOG")) == "1";
  auto log_shape = [&](const char* kind, int b, int x, int m, float ms) {
    if (tune_log) std::fprintf(stderr, "heomgb tune: %s block %d x %d min_blocks %d: %.4f ms per launch\n", kind, b, x, m, ms / 3.f);
  };
  int best_tc_m = 3, best_tc_b = 256;
  if (tc_ok && (pin_tc || !pin_b)) {
    for (int b : {128, 256})
    for (int m : {3, 2}) {  // register caps 80 and 128
      build_plan(qs->plan, insts, b, 1, m, qs->mixed, q->n_sm, qs->stream, true);
      const float ms = time_plan(b);
      log_shape("tensor cores", b, 1, m, ms);
      // the stage flags a tensor-core wait that ran out; such a plan is not kept
      DpCtl probe;
      ck(cudaMemcpyAsync(&probe, qs->ctl, sizeof(DpCtl), cudaMemcpyDeviceToHost, qs->stream), "ctl read");
      ck(cudaStreamSynchronize(qs->stream), "ctl sync");
      if (probe.status == 2) {
        ck(cudaMemsetAsync(&qs->ctl->status, 0, sizeof(int), qs->stream), "ctl reset");
        if (pin_tc) throw cuda_error("tensor-core stage did not complete");
      } else if (ms < best) {
        best = ms;
        best_tc = true;
        best_tc_m = m;
        best_tc_b = b;
      }
    }
  }
  // the site-local-bath kernel joins the search for one eligible model whose
  // stage input is the FP32 copy; HEOMGB_SITES=0 keeps it out
  bool sites_ok = qs->separate && insts.size() == 1 && sites_eligible(insts[0], qs->mixed);
  if (const char* env = std::getenv("HEOMGB_SITES"))
    if (std::string(env) == "0") sites_ok = false;
  if (pin_sb && !sites_ok) throw unsupported_error("HEOMGB_TILE=sites: the site-local-bath kernel does not apply");
  bool best_sites = false;
  int best_sb = 256, best_st = 1, best_sm = 2, best_sr = 4;
  if (sites_ok && !pin_tc && (pin_sb || !pin_b)) {
    // a thread owns an R x 4 block of an ADO (R = 4 or 2 rows): n^2 / (4 R) per ADO
    struct SV {
      int rt, minb;
      std::vector<int> blocks;
    };
    std::vector<SV> variants = {{4, 2, {128, 192, 224, 256}}, {2, 3, {128, 192, 224, 256}},
                                {2, 4, {128, 192, 224, 256}}, {2, 2, {288, 320, 352, 384}}};
    if (pin_sb) variants = {{pin_sr, pin_sm, {pin_sb}}};
    for (const SV& v : variants)
      for (int b : v.blocks) {
        const int per_ado = (insts[0].n / v.rt) * (insts[0].n / 4);
        for (int t = 1; t <= 16; ++t) {
          if (pin_sb && t != pin_st) continue;
          const int nq = t * per_ado;
          // one register block per thread, and at least 85 % of the threads busy
          if (nq > b || (!pin_sb && nq < 0.85 * b)) continue;
          if (sites_smem(insts[0].n, insts[0].K, t, insts[0].site_w) * v.minb > 220 * 1024) continue;
          try {
            build_plan(qs->plan, insts, b, 1, v.minb, qs->mixed, q->n_sm, qs->stream, false, t, v.rt);
          } catch (const unsupported_error&) {
            continue;
          }
          const float ms = pin_sb ? 0.f : time_plan(b);
          if (tune_log)
            std::fprintf(stderr, "heomgb tune: sites rows %d block %d tile %d min_blocks %d: %.4f ms per launch\n",
                         v.rt, b, t, v.minb, ms / 3.f);
          if (pin_sb || ms < best) {
            best = ms;
            best_sites = true;
            best_sb = b;
            best_st = t;
            best_sm = v.minb;
            best_sr = v.rt;
          }
        }
      }
  }
  if (pin_sb && !best_sites) throw unsupported_error("HEOMGB_TILE=sites: the pinned shape does not fit");
  const int blocks[3] = {64, 128, 256}, epts[4] = {1, 2, 4, 8};
  const int n_minb = qs->mixed ? 3 : 1, minbs[3] = {1, 3, 4};
  for (int b : blocks)
    for (int e : epts)
      for (int mi = 0; mi < n_minb; ++mi) {
      const int m = minbs[mi];
      if (pin_tc || pin_sb || (pin_b && (b != pin_b || e != pin_e || m != pin_m))) continue;
      try {
        build_plan(qs->plan, insts, b, e, m, qs->mixed, q->n_sm, qs->stream);
      } catch (const unsupported_error&) {
        continue;
      }
      if (pin_b) {
        best_b = b;
        best_e = e;
        best_m = m;
        break;
      }
      const float ms = time_plan(b);
      log_shape("diag (x = elements per thread)", b, e, m, ms);
      if (ms < best) {
        best = ms;
        best_b = b;
        best_e = e;
        best_m = m;
        best_tc = false;
        best_sites = false;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  qs->stage_ms = best < 1e29f ? best / 3.f : 0.f;
  if (best_sites)
    build_plan(qs->plan, insts, best_sb, 1, best_sm, qs->mixed, q->n_sm, qs->stream, false, best_st, best_sr);
  else if (best_tc)
    build_plan(qs->plan, insts, best_tc_b, 1, best_tc_m, qs->mixed, q->n_sm, qs->stream, true);
  else
    build_plan(qs->plan, insts, best_b, best_e, best_m, qs->mixed, q->n_sm, qs->stream);
}

// The resident interval (Dormand-Prince, fixed-step RK4 or LSRK4; fixed-step
// RK4 also in the FP64 form) applies to one model on the diagonal-coupling
// path without a terminator, when a co-resident grid holds its state in
// shared memory.  Fewer ADOs per CTA shorten each stage, more
// CTAs lengthen each grid barrier, so the grid is tuned: every co-resident
// shape (1 to 8 CTAs per SM, 1 or 2 elements per thread) runs one
// Dormand-Prince attempt or one fixed step over the solver's zeroed buffers and the fastest is
// kept.  HEOMGB_RESIDENT=0 keeps the stage kernels; HEOMGB_RESIDENT_PER_SM
// and HEOMGB_RESIDENT_EPT pin the shape.
void plan_resident(heomgb_qme_solver* qs) {
  const NvtxRange range("heomgb plan: resident interval");
  heomgb_qme* q = qs->q;
  qs->resident = false;
  const int scheme = resident_scheme(qs);
  const int variant = resident_variant(qs);
  if (variant < 0 || q->path != PATH_DIAG || qs->qmes.size() != 1 || qs->term) return;
  if (q->dinst.max_terms > kResidentTerms / 2) return;  // the per-element term table holds 4 + 4
  if (const char* env = std::getenv("HEOMGB_RESIDENT"))
    if (std::string(env) == "0") return;
  int coop = 0;
  ck(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, q->device), "device attribute");
  if (!coop) return;
  const DiagInst& I = q->dinst;
  const bool hreal = I.h_real != 0;
  int pin = 0;
  if (const char* env = std::getenv("HEOMGB_RESIDENT_PER_SM")) pin = std::atoi(env);
  int pin_ept = 0;
  if (const char* env = std::getenv("HEOMGB_RESIDENT_EPT")) pin_ept = std::atoi(env);
  struct Shape {
    int grid, apc, block, ept;
    size_t smem;
  };
  std::vector<Shape> shapes;
  for (int ept = 1; ept <= kResidentMaxEpt; ++ept) {
    if (pin_ept && ept != pin_ept) continue;
    int last_grid = -1;
    for (int per_sm = 8; per_sm >= 1; --per_sm) {
      if (pin && per_sm != pin) continue;
      const int target = per_sm * q->n_sm;
      const int apc = (I.nh + target - 1) / target;
      const int grid = (I.nh + apc - 1) / apc;
      if (grid == last_grid) continue;
      const size_t smem = variant == kResidentDpF64 ? resident_dp64_smem(I, apc) : resident_smem(I.n2, apc, variant);
      if (smem > 200 * 1024) continue;
      const int E = apc * I.n2;  // ept elements per thread
      const int block = std::max(64, ((E + ept - 1) / ept + 31) / 32 * 32);
      if (block > kResidentMaxBlock) continue;
      const int nb = resident_blocks_per_sm(variant, hreal, ept, I.n, block, smem);
      if (nb < 1 || static_cast<long long>(nb) * q->n_sm < grid) continue;
      shapes.push_back(Shape{grid, apc, block, ept, smem});
      last_grid = grid;
    }
  }
  if (shapes.empty()) return;
  qs->res_bar = static_cast<unsigned long long*>(qs->arena.alloc(kResidentBarWords * sizeof(unsigned long long)));
  int max_grid = 0;
  for (const Shape& sh : shapes) max_grid = std::max(max_grid, sh.grid);
  qs->res_partials = static_cast<double*>(qs->arena.alloc(sizeof(double) * max_grid));
  size_t best = 0;
  if (shapes.size() > 1) {
    const size_t bd = sizeof(double2) * qs->N, bb = sizeof(float2) * qs->N;
    for (int i = 0; i < 2; ++i) {
      if (qs->S[i]) ck(cudaMemsetAsync(qs->S[i], 0, bd, qs->stream), "memset");
      if (qs->Yb[i]) ck(cudaMemsetAsync(qs->Yb[i], 0, bb, qs->stream), "memset");
    }
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    float best_ms = 1e30f;
    for (size_t i = 0; i < shapes.size(); ++i) {
      qs->res_grid = shapes[i].grid;
      qs->res_apc = shapes[i].apc;
      qs->res_block = shapes[i].block;
      qs->res_ept = shapes[i].ept;
      qs->res_smem = shapes[i].smem;
      float ms_i = 1e30f;
      for (int r = 0; r < 4; ++r) {  // one warm-up, best of three
        // one attempt (zero state, zero error, accepted, t_bound reached) or one RK4 step
        ck(launch_ctl_init(qs->ctl, 0.0, 1e-3, 1e-3, 1e-8, 1e-8, 0, qs->stream), "ctl init");
        ck(cudaMemsetAsync(qs->res_bar, 0, kResidentBarWords * sizeof(unsigned long long), qs->stream), "memset");
        ResidentArgs a = resident_args(qs);
        a.n_steps = scheme == kResidentDp ? 0 : 3;  // fixed steps: four, as the instance-resident plan times
        a.dt_step = a.dt_last = 1e-3;
        ck(cudaEventRecord(e0, qs->stream), "event");
        ck(launch_resident(a, variant, hreal, qs->res_ept, qs->res_grid, qs->res_block, qs->res_smem, qs->stream),
           "resident tune");
        ck(cudaEventRecord(e1, qs->stream), "event");
        ck(cudaEventSynchronize(e1), "event sync");
        float ms = 0.f;
        ck(cudaEventElapsedTime(&ms, e0, e1), "event time");
        if (r > 0) ms_i = std::min(ms_i, ms);
      }
      unsigned long long flag = 0;
      ck(cudaMemcpy(&flag, qs->res_bar + 16, sizeof(flag), cudaMemcpyDeviceToHost), "barrier read");
      if (flag) throw cuda_error("resident Dormand-Prince interval: a grid barrier wait ran out");
      if (ms_i < best_ms) {
        best_ms = ms_i;
        best = i;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    qs->res_step_ms = scheme == kResidentDp ? 0.f : best_ms / 4.f;
  }
  qs->res_grid = shapes[best].grid;
  qs->res_apc = shapes[best].apc;
  qs->res_block = shapes[best].block;
  qs->res_ept = shapes[best].ept;
  qs->res_smem = shapes[best].smem;
  qs->resident = true;
}

// Instance-resident fixed-step intervals (k_fixed_local) apply to RK4 and
// LSRK4 on the diagonal-coupling path without a terminator when every instance fits one
// CTA's shared memory.  Instances are packed into bins (largest first, each
// into the least-loaded bin with room: at most kLocalMaxInst instances and
// the shared-memory cap), for 1, 2 or 4 bins per SM and 128, 256 or 512
// threads per CTA; every shape runs four steps over the solver's zeroed
// buffers and the fastest is kept.  It replaces the cooperative resident
// plan (timed the same way) or, without one, the graphs of stage kernels
// (four launches of the autotuned stage kernel) only where it is faster.
// HEOMGB_LOCAL=0 keeps the other paths, HEOMGB_LOCAL=1 takes the fastest
// shape without the comparison.
void plan_local(heomgb_qme_solver* qs) {
  const NvtxRange range("heomgb plan: instance-resident bins");
  heomgb_qme* q = qs->q;
  qs->local = false;
  if ((qs->kind != HEOMGB_RK4 && qs->kind != HEOMGB_LSRK4) || q->path != PATH_DIAG || qs->term || qs->plan.tcore)
    return;
  const int scheme = resident_scheme(qs);
  if (qs->resident && qs->res_step_ms <= 0.f) return;  // an untimed (pinned) resident plan stays
  bool force = false;
  if (const char* env = std::getenv("HEOMGB_LOCAL")) {
    if (std::string(env) == "0") return;
    force = std::string(env) == "1";
  }
  const std::vector<DiagInst>& insts = qs->plan.inst;
  if (insts.empty()) return;
  for (const DiagInst& I : insts)
    if (I.n2 > kLocalMaxN2 || I.nh > kLocalMaxAdo || I.term_p) return;
  const bool mixed = qs->mixed;
  auto inst_smem = [&](const DiagInst& I) { return local_bin_smem(&I.n2, &I.nh, 1, mixed); };
  std::vector<int> order(insts.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = static_cast<int>(i);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return static_cast<long long>(insts[x].n2) * insts[x].nh > static_cast<long long>(insts[y].n2) * insts[y].nh;
  });
  struct Shape {
    int grid, block;
    size_t smem;
    std::vector<int> ptr, list;
  };
  std::vector<Shape> shapes;
  for (int per_sm : {1, 2, 4}) {
    const size_t cap = (200u * 1024u) / per_sm;
    const int want = static_cast<int>(std::min<size_t>(insts.size(), static_cast<size_t>(per_sm) * q->n_sm));
    std::vector<long long> load(want, 0);
    std::vector<size_t> used(want, 0);
    std::vector<std::vector<int>> bins(want);
    bool fits = true;
    for (int i : order) {
      const size_t si = inst_smem(insts[i]);
      if (si > cap) {
        fits = false;
        break;
      }
      int pick_b = -1;
      for (size_t b = 0; b < bins.size(); ++b)
        if (used[b] + si <= cap && static_cast<int>(bins[b].size()) < kLocalMaxInst &&
            (pick_b < 0 || load[b] < load[pick_b]))
          pick_b = static_cast<int>(b);
      if (pick_b < 0) {  // every bin is full: open another (it runs in a later wave)
        bins.emplace_back();
        load.push_back(0);
        used.push_back(0);
        pick_b = static_cast<int>(bins.size()) - 1;
      }
      bins[pick_b].push_back(i);
      load[pick_b] += static_cast<long long>(insts[i].n2) * insts[i].nh;
      used[pick_b] += si;
    }
    if (!fits) continue;
    Shape sh;
    sh.smem = 16;
    sh.ptr.push_back(0);
    // the heaviest bins first, so that later waves (if any) hold the light ones
    std::vector<int> bo(bins.size());
    for (size_t b = 0; b < bo.size(); ++b) bo[b] = static_cast<int>(b);
    std::stable_sort(bo.begin(), bo.end(), [&](int x, int y) { return load[x] > load[y]; });
    for (int b : bo) {
      if (bins[b].empty()) continue;
      for (int i : bins[b]) sh.list.push_back(i);
      sh.ptr.push_back(static_cast<int>(sh.list.size()));
      sh.smem = std::max(sh.smem, used[b]);
    }
    sh.grid = static_cast<int>(sh.ptr.size()) - 1;
    for (int block : {128, 256, 512}) {
      if (local_blocks_per_sm(mixed, scheme, block, sh.smem) < 1) continue;
      sh.block = block;
      shapes.push_back(sh);
    }
  }
  if (shapes.empty()) return;
  const size_t bd = sizeof(double2) * qs->N;
  for (double2* p : {qs->S[0], qs->acc})
    if (p) ck(cudaMemsetAsync(p, 0, bd, qs->stream), "memset");
  if (mixed) ck(cudaMemsetAsync(qs->Yb[0], 0, sizeof(float2) * qs->N, qs->stream), "memset");
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "event");
  ck(cudaEventCreate(&e1), "event");
  float best_ms = 1e30f;
  size_t best = 0;
  for (size_t i = 0; i < shapes.size(); ++i) {
    DeviceArena tab;
    LocalArgs a{};
    a.inst = qs->plan.ds.inst;
    a.bin_ptr = tab.upload(shapes[i].ptr, qs->stream);
    a.bin_inst = tab.upload(shapes[i].list, qs->stream);
    a.S = qs->S[0];
    a.acc = qs->acc;
    a.Yf = mixed ? static_cast<float2*>(qs->Yb[0]) : nullptr;
    a.n_steps = 3;  // four steps
    a.dt_step = a.dt_last = 1e-3;
    float ms_i = 1e30f;
    for (int r = 0; r < 4; ++r) {  // one warm-up, best of three
      ck(cudaEventRecord(e0, qs->stream), "event");
      ck(launch_local(a, mixed, scheme, shapes[i].grid, shapes[i].block, shapes[i].smem, qs->stream), "local tune");
      ck(cudaEventRecord(e1, qs->stream), "event");
      ck(cudaEventSynchronize(e1), "event sync");
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, e0, e1), "event time");
      if (r > 0) ms_i = std::min(ms_i, ms);
    }
    if (ms_i < best_ms) {
      best_ms = ms_i;
      best = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // against the cooperative resident plan where there is one, else the stage kernels
  const float rival = qs->resident ? qs->res_step_ms : 4.f * qs->stage_ms;
  if (!force && !(best_ms / 4.f < rival)) return;
  qs->resident = false;
  const Shape& sh = shapes[best];
  qs->loc_arena.release();
  qs->loc_bin_ptr = qs->loc_arena.upload(sh.ptr, qs->stream);
  qs->loc_bin_inst = qs->loc_arena.upload(sh.list, qs->stream);
  ck(cudaStreamSynchronize(qs->stream), "local plan upload");
  qs->loc_grid = sh.grid;
  qs->loc_block = sh.block;
  qs->loc_smem = sh.smem;
  qs->local = true;
}

Stage solver_stage(heomgb_qme_solver* qs) {
  Stage st = base_stage();
  st.ctl = qs->ctl;
  st.S[0] = qs->S[0];
  st.S[1] = qs->S[1];
  st.Yb[0] = qs->Yb[0];
  st.Yb[1] = qs->Yb[1];
  st.acc = qs->acc;
  for (int i = 0; i < 6; ++i) st.K[i] = qs->K[i];
  st.bulk_separate = qs->separate ? 1 : 0;
  st.partials = qs->partials;
  return st;
}

void launch_stage(heomgb_qme_solver* qs, const Stage& st) {
  if (qs->term) {
    TermInput in;
    in.y_fixed = st.y_fixed;
    in.yb[0] = st.Yb[0];
    in.yb[1] = st.Yb[1];
    in.y_sel = st.y_sel;
    in.ctl = st.ctl;
    ck(term_enqueue(qs->term, qs->tb, term_model(qs->q), in, qs->mixed, qs->stream), "terminator");
  }
  const bool diag = qs->q->path == PATH_DIAG;
  ck(launch_rhs(qs->q->dm, diag ? &qs->plan.ds : nullptr, st, qs->q->path, qs->mixed, false, qs->grid, qs->block,
                qs->stream),
     "stage launch");
}

// One step (RK4/LSRK4) or one attempt (DP5) as a sequence of fused launches.
int enqueue_unit(heomgb_qme_solver* qs) {
  Stage st = solver_stage(qs);
  if (qs->kind == HEOMGB_RK4) {
    const int kinds[4] = {EPI_RK4_1, EPI_RK4_2, EPI_RK4_3, EPI_RK4_4};
    const void* in[4] = {qs->Yb[0], qs->Ytmp[0], qs->Ytmp[1], qs->Ytmp[0]};
    void* nxt[4] = {qs->Ytmp[0], qs->Ytmp[1], qs->Ytmp[0], nullptr};
    for (int s = 0; s < 4; ++s) {
      st.kind = kinds[s];
      st.y_sel = 0;
      st.y_fixed = in[s];
      st.Ynext = nxt[s];
      launch_stage(qs, st);
    }
    return 4;
  }
  if (qs->kind == HEOMGB_LSRK4) {  // B = 1/3, 3/4, 2/3, 1/4 (lsrk4.h:39-46)
    const double B[4] = {1.0 / 3.0, 3.0 / 4.0, 2.0 / 3.0, 1.0 / 4.0};
    for (int s = 0; s < 4; ++s) {
      st.kind = EPI_LS;
      st.ls_in = s & 1;
      st.ls_first = s == 0;
      st.coef = B[s];
      st.y_sel = 0;
      st.y_fixed = qs->Yb[s & 1];
      launch_stage(qs, st);
    }
    return 4;
  }
  for (int s = 0; s < 6; ++s) {
    st.kind = EPI_DP;
    st.dp_stage = s;
    if (s == 0) {
      st.y_sel = 1;
    } else {
      st.y_sel = 0;
      st.y_fixed = qs->Ytmp[(s - 1) & 1];
    }
    st.Ynext = s < 5 ? qs->Ytmp[s & 1] : nullptr;
    launch_stage(qs, st);
  }
  st.kind = EPI_DP7;
  st.y_sel = 2;
  st.Ynext = nullptr;
  launch_stage(qs, st);
  return 7;
}

cudaGraphExec_t capture_units(heomgb_qme_solver* qs, int units, int* nodes) {
  cudaGraph_t g = nullptr;
  ck(cudaStreamBeginCapture(qs->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  int launched = 0;
  const long long before = LaunchCounter::mine();
  try {
    for (int i = 0; i < units; ++i) enqueue_unit(qs);
  } catch (...) {
    cudaStreamEndCapture(qs->stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  launched = static_cast<int>(LaunchCounter::mine() - before);  // kernels per replay, terminator included
  g_launches += -static_cast<long long>(launched);  // captured launches are counted when the graph replays
  ck(cudaStreamEndCapture(qs->stream, &g), "end capture");
  cudaGraphExec_t ex = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  ck(e, "graph instantiate");
  *nodes = launched;
  return ex;
}

void ensure_graphs(heomgb_qme_solver* qs) {
  if (qs->g_small) return;
  if (qs->kind == HEOMGB_RKDP) {
    qs->n_small = 4;
    qs->n_big = 32;
  } else {
    qs->n_small = 1;
    qs->n_big = 50;
  }
  qs->g_small = capture_units(qs, qs->n_small, &qs->nodes_small);
  qs->g_big = capture_units(qs, qs->n_big, &qs->nodes_big);
}

void replay(heomgb_qme_solver* qs, bool big) {
  const NvtxRange range(big ? "heomgb replay: 50 steps / 32 attempts" : "heomgb replay: 1 step / 4 attempts");
  ck(cudaGraphLaunch(big ? qs->g_big : qs->g_small, qs->stream), "graph launch");
  const int nodes = big ? qs->nodes_big : qs->nodes_small;
  g_launches += nodes;
  qs->replayed_kernels += nodes;
}

// Busy-time bracket around a batch of replays; collected after a stream sync.
void busy_begin(heomgb_qme_solver* qs) { ck(cudaEventRecord(qs->ev0, qs->stream), "event record"); }
void busy_end(heomgb_qme_solver* qs) {
  ck(cudaEventRecord(qs->ev1, qs->stream), "event record");
  qs->busy_open = true;
}
void busy_collect(heomgb_qme_solver* qs) {
  if (!qs->busy_open) return;
  float ms = 0.f;
  ck(cudaEventElapsedTime(&ms, qs->ev0, qs->ev1), "event elapsed");
  qs->busy_ms += ms;
  qs->busy_open = false;
}

void state_to_bulk(heomgb_qme_solver* qs, int idx) {
  if (qs->separate)
    ck(launch_to_bulk(qs->S[idx], static_cast<float2*>(qs->Yb[idx]), qs->N, qs->stream), "to bulk");
}

double need_kw(const heomgb_kwargs* kw, int has, double v, const char* key) {
  if (!kw || !has) throw arg_error(std::string("missing kwarg \"") + key + "\"");
  return v;
}

// fixed_step_size_solver::solve_1 (fixed_step_size_solver.h:29-52): the host
// replays the reference's time loop to get the step sequence (m steps of dt,
// then the clamped last step), and the device runs it as graph replays.
void solve_fixed(heomgb_qme_solver* qs, double t0, double t1, const heomgb_kwargs* kw) {
  const NvtxRange range("heomgb interval: fixed steps");
  const double dt = need_kw(kw, kw ? kw->has_dt : 0, kw ? kw->dt : 0, "dt");
  long long m = 0;
  double t = t0, d = dt, last = dt;
  const long long cap = 1LL << 40;
  while (true) {
    if (t + d - t1 > -std::numeric_limits<double>::epsilon()) {
      last = t1 - t;
      break;
    }
    t += d;
    if (++m > cap) throw numeric_error("fixed-step loop does not terminate");
  }
  if (qs->local) {  // the whole interval as one launch of instance-resident bins (k_fixed_local)
    LocalArgs a{};
    a.inst = qs->plan.ds.inst;
    a.bin_ptr = qs->loc_bin_ptr;
    a.bin_inst = qs->loc_bin_inst;
    a.S = qs->S[0];
    a.acc = qs->acc;
    a.Yf = qs->mixed ? static_cast<float2*>(qs->Yb[0]) : nullptr;
    a.n_steps = m;
    a.dt_step = dt;
    a.dt_last = last;
    busy_begin(qs);
    ck(launch_local(a, qs->mixed, resident_scheme(qs), qs->loc_grid, qs->loc_block, qs->loc_smem, qs->stream),
       "instance-resident interval");
    busy_end(qs);
    qs->replayed_kernels += 1;
    qs->n_rhs += 4 * (m + 1);
    qs->n_attempts += m + 1;
    qs->n_accepted += m + 1;
    return;
  }
  if (qs->resident) {  // the whole interval as one resident launch (k_rk4_resident / k_ls_resident)
    ck(cudaMemsetAsync(qs->res_bar, 0, kResidentBarWords * sizeof(unsigned long long), qs->stream), "barrier reset");
    ResidentArgs a = resident_args(qs);
    a.n_steps = m;
    a.dt_step = dt;
    a.dt_last = last;
    busy_begin(qs);
    const cudaError_t le = launch_resident(a, resident_variant(qs), qs->q->dinst.h_real != 0, qs->res_ept,
                                           qs->res_grid, qs->res_block, qs->res_smem, qs->stream);
    if (le != cudaErrorCooperativeLaunchTooLarge) {
      ck(le, "resident interval");
      busy_end(qs);
      qs->replayed_kernels += 1;
      unsigned long long flag = 0;
      ck(cudaMemcpyAsync(&flag, qs->res_bar + 16, sizeof(flag), cudaMemcpyDeviceToHost, qs->stream),
         "barrier read");
      ck(cudaStreamSynchronize(qs->stream), "solve sync");
      busy_collect(qs);
      if (flag) throw cuda_error("resident fixed-step interval: a grid barrier wait ran out");
      qs->n_rhs += 4 * (m + 1);
      qs->n_attempts += m + 1;
      qs->n_accepted += m + 1;
      return;
    }
    // the device cannot hold the grid now: this and later intervals take the graphs
    cudaGetLastError();
    busy_end(qs);
    ck(cudaStreamSynchronize(qs->stream), "solve sync");
    busy_collect(qs);
    qs->resident = false;
  }
  ensure_graphs(qs);
  ck(launch_ctl_init(qs->ctl, t0, dt, t1, 0.0, 0.0, 0, qs->stream), "ctl init");
  busy_begin(qs);
  for (long long i = 0; i < m / qs->n_big; ++i) replay(qs, true);
  for (long long i = 0; i < m % qs->n_big; ++i) replay(qs, false);
  ck(launch_ctl_set_fixed(qs->ctl, last, qs->stream), "ctl dt");
  replay(qs, false);
  busy_end(qs);
  if (qs->plan.tcore) {  // a tensor-core stage that gave up flags the controller
    ck(cudaMemcpyAsync(qs->ctl_host, qs->ctl, sizeof(DpCtl), cudaMemcpyDeviceToHost, qs->stream), "ctl read");
    ck(cudaStreamSynchronize(qs->stream), "ctl sync");
    if (qs->ctl_host->status == 2) throw cuda_error("tensor-core stage did not complete");
  }
  qs->n_rhs += 4 * (m + 1);
  qs->n_attempts += m + 1;
  qs->n_accepted += m + 1;
}

// adaptive_step_size_solver::solve_1 + rkdp::solve_adaptive_step as one
// resident launch (k_dp_resident).
int solve_adaptive(heomgb_qme_solver* qs, double t0, double t1, const heomgb_kwargs* kw, int cur);

int solve_resident(heomgb_qme_solver* qs, double t0, double t1, const heomgb_kwargs* kw, int cur) {
  const NvtxRange range("heomgb interval: resident Dormand-Prince");
  if (qs->dt_save == -1.0) qs->dt_save = need_kw(kw, kw ? kw->has_dt : 0, kw ? kw->dt : 0, "dt");
  const double atol = need_kw(kw, kw ? kw->has_atol : 0, kw ? kw->atol : 0, "atol");
  const double rtol = need_kw(kw, kw ? kw->has_rtol : 0, kw ? kw->rtol : 0, "rtol");
  double dt = qs->dt_save;
  if (t0 + dt > t1) dt = t1 - t0;
  ck(launch_ctl_init(qs->ctl, t0, dt, t1, atol, rtol, cur, qs->stream), "ctl init");
  ck(cudaMemsetAsync(qs->res_bar, 0, kResidentBarWords * sizeof(unsigned long long), qs->stream), "barrier reset");
  busy_begin(qs);
  const cudaError_t le = launch_resident(resident_args(qs), resident_variant(qs), qs->q->dinst.h_real != 0, qs->res_ept,
                                         qs->res_grid, qs->res_block, qs->res_smem, qs->stream);
  if (le == cudaErrorCooperativeLaunchTooLarge) {
    // the device cannot hold the grid now (another context holds SMs or
    // shared memory): this and later intervals take the stage kernels
    cudaGetLastError();
    busy_end(qs);
    ck(cudaStreamSynchronize(qs->stream), "solve sync");
    busy_collect(qs);
    qs->resident = false;
    return solve_adaptive(qs, t0, t1, kw, cur);
  }
  ck(le, "resident interval");
  busy_end(qs);
  qs->replayed_kernels += 1;
  unsigned long long flag = 0;
  ck(cudaMemcpyAsync(qs->ctl_host, qs->ctl, sizeof(DpCtl), cudaMemcpyDeviceToHost, qs->stream), "ctl read");
  ck(cudaMemcpyAsync(&flag, qs->res_bar + 16, sizeof(flag), cudaMemcpyDeviceToHost, qs->stream), "barrier read");
  ck(cudaStreamSynchronize(qs->stream), "solve sync");
  busy_collect(qs);
  if (flag) throw cuda_error("resident Dormand-Prince interval: a grid barrier wait ran out");
  if (qs->ctl_host->status == 3) throw numeric_error("Dormand-Prince attempt cap reached");
  if (qs->ctl_host->status) throw numeric_error("non-finite step size in Dormand-Prince control");
  qs->dt_save = qs->ctl_host->dt;
  qs->n_attempts += qs->ctl_host->attempts;
  qs->n_accepted += qs->ctl_host->accepted;
  qs->n_rhs += 7 * qs->ctl_host->attempts;
  return qs->ctl_host->cur;
}

// adaptive_step_size_solver::solve_1 + rkdp::solve_adaptive_step
// (adaptive_step_size_solver.h:32-56, rkdp.h:81-179) with the controller on
// the device; the host only polls the `done` flag between graph replays.
int solve_adaptive(heomgb_qme_solver* qs, double t0, double t1, const heomgb_kwargs* kw, int cur) {
  const NvtxRange range("heomgb interval: Dormand-Prince graphs");
  if (qs->dt_save == -1.0) qs->dt_save = need_kw(kw, kw ? kw->has_dt : 0, kw ? kw->dt : 0, "dt");
  const double atol = need_kw(kw, kw ? kw->has_atol : 0, kw ? kw->atol : 0, "atol");
  const double rtol = need_kw(kw, kw ? kw->has_rtol : 0, kw ? kw->rtol : 0, "rtol");
  double dt = qs->dt_save;
  if (t0 + dt > t1) dt = t1 - t0;
  ensure_graphs(qs);
  ck(launch_ctl_init(qs->ctl, t0, dt, t1, atol, rtol, cur, qs->stream), "ctl init");
  long long launched = 0;
  bool big = false;
  const long long cap = 2000000LL;
  while (true) {
    busy_begin(qs);
    replay(qs, big);
    busy_end(qs);
    launched += big ? qs->n_big : qs->n_small;
    ck(cudaMemcpyAsync(qs->ctl_host, qs->ctl, sizeof(DpCtl), cudaMemcpyDeviceToHost, qs->stream), "ctl read");
    ck(cudaStreamSynchronize(qs->stream), "solve sync");
    busy_collect(qs);
    if (qs->ctl_host->done) break;
    big = true;
    if (launched > cap) throw numeric_error("Dormand-Prince attempt cap reached");
  }
  if (qs->ctl_host->status == 2) throw cuda_error("tensor-core stage did not complete");
  if (qs->ctl_host->status) throw numeric_error("non-finite step size in Dormand-Prince control");
  qs->dt_save = qs->ctl_host->dt;
  qs->n_attempts += qs->ctl_host->attempts;
  qs->n_accepted += qs->ctl_host->accepted;
  qs->n_rhs += 7 * qs->ctl_host->attempts;
  return qs->ctl_host->cur;
}

// Per-instance ADO transposes of a concatenated (batch) state.
void transpose_instances(heomgb_qme_solver* qs, const double2* in, double2* out) {
  long long off = 0;
  for (heomgb_qme* m : qs->qmes) {
    ck(launch_transpose_ados(in + off, out + off, m->n, m->n_hrchy, qs->stream), "transpose");
    off += m->main_size();
  }
}

void solve_impl(heomgb_qme_solver* qs, void* rho, bool host, const double* t_list, int n_t, heomgb_callback cb,
                void* user, const heomgb_kwargs* kw) {
  const NvtxRange range("heomgb solve");
  if (!qs) throw arg_error("null qme_solver");
  for (heomgb_qme* m : qs->qmes) need_ready(m);
  if (!rho) throw arg_error("null rho");
  if (n_t < 1 || !t_list) throw arg_error("t_list must hold at least one time");
  ck(cudaSetDevice(qs->q->device), "cudaSetDevice");
  if (qs->own_stream) {  // after the work the caller queued on the model stream (e.g. filling rho)
    ck(cudaEventRecord(qs->user_ready, qs->q->stream()), "event record");
    ck(cudaStreamWaitEvent(qs->stream, qs->user_ready, 0), "stream wait");
  }
  qs->n_rhs = qs->n_attempts = qs->n_accepted = 0;
  qs->busy_ms = 0.0;
  qs->replayed_kernels = 0;
  qs->busy_open = false;
  const size_t bytes = sizeof(double2) * qs->N;
  const cudaMemcpyKind in_kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind out_kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  // solver_base::solve (solver_base.h:64-79)
  for (int i = 0; i < n_t - 1; ++i) {
    if (cb) {
      if (!host) ck(cudaStreamSynchronize(qs->stream), "sync before callback");
      cb(t_list[i], user);
    }
    if (qs->col_major) {  // the caller's ADOs are column-major: transpose at the boundary
      ck(cudaMemcpyAsync(qs->otmp, rho, bytes, in_kind, qs->stream), "state in");
      transpose_instances(qs, qs->otmp, qs->S[0]);
    } else {
      ck(cudaMemcpyAsync(qs->S[0], rho, bytes, in_kind, qs->stream), "state in");
    }
    state_to_bulk(qs, 0);
    int cur = 0;
    if (qs->kind == HEOMGB_RKDP)
      cur = qs->resident ? solve_resident(qs, t_list[i], t_list[i + 1], kw, 0)
                         : solve_adaptive(qs, t_list[i], t_list[i + 1], kw, 0);
    else
      solve_fixed(qs, t_list[i], t_list[i + 1], kw);
    if (qs->col_major) {
      transpose_instances(qs, qs->S[cur], qs->otmp);
      ck(cudaMemcpyAsync(rho, qs->otmp, bytes, out_kind, qs->stream), "state out");
    } else {
      ck(cudaMemcpyAsync(rho, qs->S[cur], bytes, out_kind, qs->stream), "state out");
    }
    ck(cudaStreamSynchronize(qs->stream), "interval sync");
    busy_collect(qs);
    if (qs->term && mlp_take_error(qs->term, qs->stream))
      throw cuda_error("terminator inference: a tensor-core GEMM did not complete");
  }
  if (cb) cb(t_list[n_t - 1], user);
}

}  // namespace

namespace heomgb {

void set_error_message(const std::string& msg) { g_err = msg; }
}  // namespace heomgb

// ======================================================================= C ABI
extern "C" {

const char* heomgb_last_error(void) { return g_err.c_str(); }
const char* heomgb_version(void) { return "0.1.0"; }
int heomgb_abi_version(void) { return 1; }
long long heomgb_launch_count(void) { return g_launches.total.load(); }

heomgb_status heomgb_qme_create(heomgb_form form, int max_depth, int n_inner_threads, int n_outer_threads,
                                heomgb_qme** out) {
  (void)n_inner_threads;
  (void)n_outer_threads;
  return guard([&] {
    require(out != nullptr, "null out");
    require(form == HEOMGB_HILB || form == HEOMGB_LIOU || form == HEOMGB_ADO || is_redfield(form), "unknown form");
    require(max_depth >= 0, "max_depth must be >= 0");
    auto q = std::make_unique<heomgb_qme>();
    q->form = form;
    q->max_depth = is_redfield(form) ? 0 : max_depth;  // Redfield: one n x n state, no hierarchy
    ck(cudaGetDevice(&q->device), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&q->n_sm, cudaDevAttrMultiProcessorCount, q->device), "device attribute");
    ck(cudaStreamCreateWithFlags(&q->own_stream, cudaStreamNonBlocking), "stream create");
    *out = q.release();
  });
}

heomgb_status heomgb_qme_destroy(heomgb_qme* q) {
  if (!q) return HEOMGB_OK;
  if (q->live_solvers > 0) return fail(HEOMGB_ERR_STATE, "destroy the qme_solvers of this model first");
  cudaSetDevice(q->device);
  if (q->own_stream) cudaStreamSynchronize(q->own_stream);
  if (q->user_stream_set) cudaStreamSynchronize(q->user_stream);
  q->arena.release();
  q->term_arena.release();
  q->scratch.release();
  if (q->own_stream) cudaStreamDestroy(q->own_stream);
  delete q;
  return HEOMGB_OK;
}

heomgb_status heomgb_qme_set_hamiltonian(heomgb_qme* q, int n_level, const double* H) {
  return guard([&] {
    require(q && H, "null argument");
    require(n_level > 0, "n_level must be > 0");
    q->n = n_level;
    q->H.resize(static_cast<size_t>(n_level) * n_level);
    for (size_t i = 0; i < q->H.size(); ++i) q->H[i] = C(H, i);
    q->ready = false;
  });
}

heomgb_status heomgb_qme_alloc_noises(heomgb_qme* q, int n_noise) {
  return guard([&] {
    require(q != nullptr, "null qme");
    require(n_noise >= 0, "n_noise must be >= 0");
    q->U = n_noise;
    q->baths.assign(n_noise, Bath{});
    q->ready = false;
  });
}

heomgb_status heomgb_qme_set_noise(heomgb_qme* q, int u, const double* V, int len_gamma, const double* gamma,
                                   const double* phi_0, const double* sigma, const double* S, const double* A,
                                   const double* s_delta) {
  return guard([&] {
    require(q != nullptr, "null qme");
    if (q->U < 0) throw state_error("alloc_noises must precede set_noise");
    require(u >= 0 && u < q->U, "bath index out of range");
    require(q->n > 0, "set the Hamiltonian (n_level) before the noises");
    require(len_gamma >= 0, "len_gamma must be >= 0");
    require(V && s_delta, "null V or s_delta");
    require(len_gamma == 0 || (gamma && phi_0 && sigma && S && A), "null noise array");
    Bath b;
    b.set = true;
    b.len = len_gamma;
    const size_t n2 = static_cast<size_t>(q->n) * q->n, L = len_gamma, L2 = L * L;
    b.V.resize(n2);
    for (size_t i = 0; i < n2; ++i) b.V[i] = C(V, i);
    b.gamma.resize(L2);
    b.S.resize(L2);
    b.A.resize(L2);
    for (size_t i = 0; i < L2; ++i) {
      b.gamma[i] = C(gamma, i);
      b.S[i] = C(S, i);
      b.A[i] = C(A, i);
    }
    b.phi0.resize(L);
    b.sigma.resize(L);
    for (size_t i = 0; i < L; ++i) {
      b.phi0[i] = C(phi_0, i);
      b.sigma[i] = C(sigma, i);
    }
    b.sdelta = C(s_delta, 0);
    q->baths[u] = std::move(b);
    q->ready = false;
  });
}

heomgb_status heomgb_qme_set_precision(heomgb_qme* q, heomgb_precision p) {
  return guard([&] {
    require(q != nullptr, "null qme");
    require(p == HEOMGB_FP64 || p == HEOMGB_MIXED, "unknown precision");
    q->precision = p;
  });
}

heomgb_status heomgb_qme_set_hrchy_filter(heomgb_qme* q, heomgb_hrchy_filter filter, void* user) {
  return guard([&] {
    require(q != nullptr, "null qme");
    if (q->live_solvers > 0) throw state_error("set_hrchy_filter: destroy the qme_solvers of this model first");
    q->filter = filter;
    q->filter_user = user;
  });
}

heomgb_status heomgb_qme_set_order(heomgb_qme* q, heomgb_order order) {
  return guard([&] {
    require(q != nullptr, "null qme");
    require(order == HEOMGB_ROW_MAJOR || order == HEOMGB_COL_MAJOR, "unknown order");
    if (q->live_solvers > 0) throw state_error("set_order: destroy the qme_solvers of this model first");
    q->col_major = order == HEOMGB_COL_MAJOR ? 1 : 0;
  });
}

heomgb_status heomgb_qme_set_normalization(heomgb_qme* q, heomgb_normalization norm) {
  return guard([&] {
    require(q != nullptr, "null qme");
    require(norm == HEOMGB_NORM_INTEGER || norm == HEOMGB_NORM_SQRT, "unknown normalisation");
    if (q->live_solvers > 0) throw state_error("set_normalization: destroy the qme_solvers of this model first");
    q->sqrt_norm = norm == HEOMGB_NORM_SQRT ? 1 : 0;
  });
}

heomgb_status heomgb_qme_get_precision(const heomgb_qme* q, int* requested, int* effective, double* growth_log10,
                                       double* cancel_log10) {
  return guard([&] {
    need_ready(q);
    if (requested) *requested = q->precision;
    if (effective) *effective = q->precision_eff;
    if (growth_log10) *growth_log10 = q->range_growth;
    if (cancel_log10) *cancel_log10 = q->range_cancel;
  });
}

heomgb_status heomgb_qme_set_stream(heomgb_qme* q, void* cuda_stream) {
  return guard([&] {
    require(q != nullptr, "null qme");
    q->user_stream = static_cast<cudaStream_t>(cuda_stream);
    q->user_stream_set = cuda_stream != nullptr;
  });
}

heomgb_status heomgb_qme_set_param(heomgb_qme* q) {
  return guard([&] {
    const NvtxRange range("heomgb set_param");
    require(q != nullptr, "null qme");
    build_model(q);
  });
}

heomgb_status heomgb_qme_set_terminator(heomgb_qme* q, heomgb_mlp* mlp) {
  return guard([&] {
    need_ready(q);
    if (q->live_solvers > 0) throw state_error("set_terminator: destroy the qme_solvers of this model first");
    if (mlp) {
      if (q->path != PATH_DIAG) throw unsupported_error("the learned terminator needs diagonal couplings V (heom_hilb)");
      if (q->sqrt_norm) throw unsupported_error("the learned terminator is trained for the integer normalisation");
      if (q->filter) throw unsupported_error("the learned terminator needs the complete truncated tier (no filter)");
      int din = 0, h = 0, dout = 0;
      mlp_dims(mlp, &din, &h, &dout);
      const int n2 = q->n * q->n;
      if (din != 4 * n2 + q->K || dout != 2 * n2)
        throw arg_error("terminator MLP must map 4*n_level^2 + n_dim inputs to 2*n_level^2 outputs");
    }
    ck(cudaSetDevice(q->device), "cudaSetDevice");
    q->term_arena.release();
    q->diff_tb = TermBuffers{};
    q->term = mlp;
    DiagInst di = q->dinst;
    q->term_cke = nullptr;
    q->term_sgn = nullptr;
    if (mlp) {
      alloc_term(q->term_arena, q, q->diff_tb);
      di.term_p = q->diff_tb.P;
      di.term_first = q->diff_tb.first;
      // per mode k and element e: -i s_k (v_a - v_b) + a_k (v_a + v_b), sign(Re(v_a - v_b))
      const int n = q->n, n2 = n * n, K = q->K;
      std::vector<cd> sv, av;
      std::vector<int> bath_of;
      for (int u = 0; u < q->U; ++u) {
        const Bath& B = q->baths[u];
        for (int k = 0; k < B.len; ++k) {
          cd sk(0.0, 0.0), ak(0.0, 0.0);  // s = S phi_0, a = A phi_0 as the model forms them
          for (int j = 0; j < B.len; ++j) {
            const cd Sv = B.S[static_cast<size_t>(k) * B.len + j], Av = B.A[static_cast<size_t>(k) * B.len + j];
            if (Sv != cd(0.0, 0.0)) sk += Sv * B.phi0[j];
            if (Av != cd(0.0, 0.0)) ak += Av * B.phi0[j];
          }
          sv.push_back(sk);
          av.push_back(ak);
          bath_of.push_back(u);
        }
      }
      std::vector<cd> cke(static_cast<size_t>(K) * n2);
      std::vector<float> sgn(static_cast<size_t>(K) * n2);
      const cd I(0.0, 1.0);
      for (int k = 0; k < K; ++k) {
        const Bath& B = q->baths[bath_of[k]];
        for (int a = 0; a < n; ++a)
          for (int b = 0; b < n; ++b) {
            const cd va = B.V[static_cast<size_t>(a) * n + a], vb = B.V[static_cast<size_t>(b) * n + b];
            cke[static_cast<size_t>(k) * n2 + a * n + b] = -I * sv[k] * (va - vb) + av[k] * (va + vb);
            const double dv = (va - vb).real();
            sgn[static_cast<size_t>(k) * n2 + a * n + b] = dv > 0.0 ? 1.f : (dv < 0.0 ? -1.f : 0.f);
          }
      }
      q->term_cke = q->term_arena.upload(to_f2(cke), q->stream());
      q->term_sgn = q->term_arena.upload(sgn, q->stream());
      ck(cudaStreamSynchronize(q->stream()), "terminator tables");
    }
    build_plan(q->diff_plan, {di}, q->diff_plan.block, q->diff_plan.ept, q->diff_plan.min_blocks,
               q->precision_eff == HEOMGB_MIXED, q->n_sm,
               q->stream());
  });
}

heomgb_status heomgb_qme_get_n_hrchy(const heomgb_qme* q, int* n_hrchy) {
  return guard([&] {
    need_ready(q);
    require(n_hrchy != nullptr, "null out");
    *n_hrchy = q->n_hrchy;
  });
}

heomgb_status heomgb_qme_get_n_dim(const heomgb_qme* q, int* n_dim) {
  return guard([&] {
    need_ready(q);
    require(n_dim != nullptr, "null out");
    *n_dim = q->K;
  });
}

heomgb_status heomgb_qme_main_size(const heomgb_qme* q, long long* size) {
  return guard([&] {
    need_ready(q);
    require(size != nullptr, "null out");
    *size = q->main_size();
  });
}

heomgb_status heomgb_qme_get_hrchy(const heomgb_qme* q, int* n, int* ptr_p1, int* ptr_m1) {
  return guard([&] {
    need_ready(q);
    ck(cudaSetDevice(q->device), "cudaSetDevice");
    const size_t K = q->K, nh = q->n_hrchy;
    cudaStream_t s = q->stream();
    if (K == 0) return;
    if (n) ck(cudaMemcpyAsync(n, q->dm.nidx, sizeof(int) * nh * K, cudaMemcpyDeviceToHost, s), "copy n");
    if (ptr_p1) ck(cudaMemcpyAsync(ptr_p1, q->dm.p1, sizeof(int) * (nh + 1) * K, cudaMemcpyDeviceToHost, s), "copy p1");
    if (ptr_m1) ck(cudaMemcpyAsync(ptr_m1, q->dm.m1, sizeof(int) * (nh + 1) * K, cudaMemcpyDeviceToHost, s), "copy m1");
    ck(cudaStreamSynchronize(s), "hierarchy copy sync");
  });
}

heomgb_status heomgb_qme_calc_diff(heomgb_qme* q, double* drho, const double* rho, const double* alpha,
                                   const double* beta) {
  return guard([&] {
    need_ready(q);
    require(drho && rho, "null rho/drho");
    require(drho != rho, "drho and rho must not alias");
    ck(cudaSetDevice(q->device), "cudaSetDevice");
    cudaStream_t s = q->stream();
    const size_t bytes = sizeof(double2) * q->main_size();
    if (!q->sx) {
      q->sx = static_cast<double2*>(q->scratch.alloc(bytes));
      q->sy = static_cast<double2*>(q->scratch.alloc(bytes));
    }
    const bool beta_zero = !beta || (beta[0] == 0.0 && beta[1] == 0.0);
    ck(cudaMemcpyAsync(q->sx, rho, bytes, cudaMemcpyHostToDevice, s), "rho in");
    if (!beta_zero) ck(cudaMemcpyAsync(q->sy, drho, bytes, cudaMemcpyHostToDevice, s), "drho in");
    run_diff(q, q->sy, q->sx, alpha, beta);
    ck(cudaMemcpyAsync(drho, q->sy, bytes, cudaMemcpyDeviceToHost, s), "drho out");
    ck(cudaStreamSynchronize(s), "calc_diff sync");
  });
}

heomgb_status heomgb_qme_calc_diff_device(heomgb_qme* q, void* drho, const void* rho, const double* alpha,
                                          const double* beta) {
  return guard([&] {
    need_ready(q);
    require(drho && rho, "null rho/drho");
    require(drho != rho, "drho and rho must not alias");
    ck(cudaSetDevice(q->device), "cudaSetDevice");
    run_diff(q, static_cast<double2*>(drho), static_cast<const double2*>(rho), alpha, beta);
  });
}

heomgb_status heomgb_solver_create(heomgb_solver_kind kind, heomgb_solver** out) {
  return guard([&] {
    require(out != nullptr, "null out");
    require(kind == HEOMGB_RK4 || kind == HEOMGB_LSRK4 || kind == HEOMGB_RKDP, "unknown solver");
    auto s = std::make_unique<heomgb_solver>();
    s->kind = kind;
    *out = s.release();
  });
}

heomgb_status heomgb_solver_destroy(heomgb_solver* s) {
  delete s;
  return HEOMGB_OK;
}

heomgb_status heomgb_qme_solver_create(heomgb_qme* q, heomgb_solver* s, heomgb_qme_solver** out) {
  return guard([&] {
    need_ready(q);
    require(s && out, "null argument");
    ck(cudaSetDevice(q->device), "cudaSetDevice");
    auto qs = std::make_unique<heomgb_qme_solver>();
    qs->q = q;
    qs->qmes = {q};
    qs->kind = s->kind;
    qs->stream = q->stream();
    alloc_solver(qs.get());
    ck(cudaStreamSynchronize(qs->stream), "solver init sync");
    q->live_solvers += 1;
    *out = qs.release();
  });
}

heomgb_status heomgb_batch_solver_create(heomgb_qme* const* qmes, int count, heomgb_solver* s,
                                         heomgb_qme_solver** out) {
  return guard([&] {
    require(qmes && s && out && count >= 1, "null argument or empty batch");
    require(s->kind == HEOMGB_RK4 || s->kind == HEOMGB_LSRK4,
            "batches step all instances with one dt: rk4 or lsrk4 only");
    heomgb_qme* q0 = qmes[0];
    for (int i = 0; i < count; ++i) {
      need_ready(qmes[i]);
      if (qmes[i]->path != PATH_DIAG)
        throw unsupported_error("batches need heom_hilb models with diagonal couplings V");
      if (qmes[i]->precision_eff != q0->precision_eff)
        throw arg_error("batch models must share one effective precision (heomgb_qme_get_precision)");
      if (qmes[i]->col_major != q0->col_major) throw arg_error("batch models must share one storage order");
      if (qmes[i]->device != q0->device) throw arg_error("batch models must live on one device");
    }
    ck(cudaSetDevice(q0->device), "cudaSetDevice");
    auto qs = std::make_unique<heomgb_qme_solver>();
    qs->q = q0;
    qs->qmes.assign(qmes, qmes + count);
    qs->kind = s->kind;
    ck(cudaStreamSynchronize(q0->stream()), "model stream sync");
    ck(cudaStreamCreateWithFlags(&qs->own_stream, cudaStreamNonBlocking), "stream create");
    ck(cudaEventCreateWithFlags(&qs->user_ready, cudaEventDisableTiming), "event create");
    qs->stream = qs->own_stream;
    alloc_solver(qs.get());
    ck(cudaStreamSynchronize(qs->stream), "solver init sync");
    for (heomgb_qme* m : qs->qmes) m->live_solvers += 1;
    *out = qs.release();
  });
}

heomgb_status heomgb_qme_solver_destroy(heomgb_qme_solver* qs) {
  if (!qs) return HEOMGB_OK;
  cudaSetDevice(qs->q->device);
  cudaStreamSynchronize(qs->stream);
  for (heomgb_qme* m : qs->qmes) m->live_solvers -= 1;
  delete qs;
  return HEOMGB_OK;
}

heomgb_status heomgb_qme_solver_main_size(const heomgb_qme_solver* qs, long long* size) {
  return guard([&] {
    require(qs && size, "null argument");
    *size = qs->N;
  });
}

heomgb_status heomgb_qme_solver_tuning(const heomgb_qme_solver* qs, int* block, int* elems_per_thread,
                                       int* n_tiles, int* min_blocks) {
  return guard([&] {
    require(qs != nullptr, "null qme_solver");
    const bool diag = qs->q->path == PATH_DIAG;
    if (block) *block = qs->block;
    if (elems_per_thread) *elems_per_thread = diag ? qs->plan.ept : 0;
    if (n_tiles) *n_tiles = diag ? qs->plan.ds.n_tiles : 0;
    if (min_blocks) *min_blocks = diag ? qs->plan.min_blocks : 0;
  });
}

heomgb_status heomgb_qme_solver_resident(const heomgb_qme_solver* qs, int* on, int* grid, int* ados_per_cta) {
  return guard([&] {
    require(qs != nullptr && on != nullptr, "null argument");
    *on = qs->resident ? 1 : 0;
    if (grid) *grid = qs->resident ? qs->res_grid : 0;
    if (ados_per_cta) *ados_per_cta = qs->resident ? qs->res_apc : 0;
  });
}

heomgb_status heomgb_qme_solver_local(const heomgb_qme_solver* qs, int* on, int* bins, int* block) {
  return guard([&] {
    require(qs != nullptr && on != nullptr, "null argument");
    *on = qs->local ? 1 : 0;
    if (bins) *bins = qs->local ? qs->loc_grid : 0;
    if (block) *block = qs->local ? qs->loc_block : 0;
  });
}

heomgb_status heomgb_qme_solver_site_kernel(const heomgb_qme_solver* qs, int* on, int* ados_per_tile) {
  return guard([&] {
    require(qs != nullptr && on != nullptr, "null argument");
    const bool sites = qs->q->path == PATH_DIAG && qs->plan.sites;
    *on = sites ? 1 : 0;
    if (ados_per_tile) *ados_per_tile = sites ? qs->plan.ds.sites_tile : 0;
  });
}

heomgb_status heomgb_qme_solver_tensor_cores(const heomgb_qme_solver* qs, int* on) {
  return guard([&] {
    require(qs != nullptr && on != nullptr, "null argument");
    *on = (qs->q->path == PATH_DIAG && qs->plan.tcore) ? 1 : 0;
  });
}

heomgb_status heomgb_qme_solver_solve(heomgb_qme_solver* qs, double* rho, const double* t_list, int n_t,
                                      heomgb_callback cb, void* user, const heomgb_kwargs* kwargs) {
  return guard([&] { solve_impl(qs, rho, true, t_list, n_t, cb, user, kwargs); });
}

heomgb_status heomgb_qme_solver_solve_device(heomgb_qme_solver* qs, void* rho, const double* t_list, int n_t,
                                             heomgb_callback cb, void* user, const heomgb_kwargs* kwargs) {
  return guard([&] { solve_impl(qs, rho, false, t_list, n_t, cb, user, kwargs); });
}

heomgb_status heomgb_qme_solver_stats(const heomgb_qme_solver* qs, long long* n_rhs, long long* n_attempts,
                                      long long* n_accepted, double* dt_save) {
  return guard([&] {
    require(qs != nullptr, "null qme_solver");
    if (n_rhs) *n_rhs = qs->n_rhs;
    if (n_attempts) *n_attempts = qs->n_attempts;
    if (n_accepted) *n_accepted = qs->n_accepted;
    if (dt_save) *dt_save = qs->dt_save;
  });
}

heomgb_status heomgb_probe_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  return guard([&] {
    require(fp64_tflops && fp32_tflops, "null out");
    int dev = 0, n_sm = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    cudaStream_t s = nullptr;
    ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream create");
    const cudaError_t e = probe_fma_peaks(n_sm, fp64_tflops, fp32_tflops, s);
    cudaStreamDestroy(s);
    ck(e, "fma probe");
  });
}

size_t heomgb_errnrm1_scratch(long long n) { return static_cast<size_t>(errnrm1_grid(n > 0 ? n : 1)) + 2; }

heomgb_status heomgb_qme_solver_timing(const heomgb_qme_solver* qs, double* busy_ms, long long* kernels) {
  return guard([&] {
    require(qs != nullptr, "null qme_solver");
    if (busy_ms) *busy_ms = qs->busy_ms;
    if (kernels) *kernels = qs->replayed_kernels;
  });
}

heomgb_status heomgb_errnrm1_device(const void* e, const void* x1, const void* x2, double atol, double rtol,
                                    long long n, double* scratch, double* result, void* cuda_stream) {
  return guard([&] {
    require(e && x1 && x2 && scratch && result, "null argument");
    require(n > 0, "n must be > 0");
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    const int grid = errnrm1_grid(n);
    double* out = scratch + grid;
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + grid + 1);
    ck(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s), "memset counter");
    ck(launch_errnrm1(static_cast<const double2*>(e), static_cast<const double2*>(x1),
                      static_cast<const double2*>(x2), atol, rtol, n, scratch, out, counter, grid, s),
       "errnrm1");
    ck(cudaMemcpyAsync(result, out, sizeof(double), cudaMemcpyDeviceToHost, s), "errnrm1 result");
    ck(cudaStreamSynchronize(s), "errnrm1 sync");
  });
}

}  // extern "C"
