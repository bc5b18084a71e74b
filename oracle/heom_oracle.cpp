// Test infrastructure: CPU restatement of the reference's HEOM propagation path.
//
// THIS IS THE ORACLE, NOT THE PRODUCT.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline arm load it, and only as the checker or as the
// timed CPU baseline.  Its agreement with the reference's own code (compiled
// by `make -C oracle ref` from the reference tree) is pinned by the committed
// golden fixtures in tests/golden/ (tests/test_oracle_golden.py).
//
// What it restates, step by step (file:line in the reference tree):
//   alloc_hrchy_space BFS order and +-1 tables      src/hrchy_space.cc:137-231
//   heom::set_param (lk, ngamma_diag, s=S*phi0, a=A*phi0;
//     off-diagonal gamma is cleared before use, so it never contributes)
//                                                  include/heom.h:57-139
//   heom_hilb::calc_diff_impl                       include/heom_hilb.h:70-215
//   rk4 / lsrk4 / rkdp steps                        include/solver/rk4.h:40-65,
//                                                  lsrk4.h:32-47, rkdp.h:81-179
//   fixed / adaptive step loops, solve()            fixed_step_size_solver.h:29-52,
//                                                  adaptive_step_size_solver.h:32-56,
//                                                  solver_base.h:64-79
//   errnrm1                                         linalg_engine_eigen.h.j2:360-379
// heom_liou / heom_ado apply the same operator through superoperators
// (heom_liou.h:66-258, heom_ado.h:62-202); the restatement evaluates their
// common Hilbert-space form for every `form`.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "heom_case.h"

namespace {

struct cx {
  double re, im;
};
inline cx operator+(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
inline cx operator-(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
inline cx operator*(cx a, cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cx operator*(double s, cx a) { return {s * a.re, s * a.im}; }
inline bool is_zero(cx a) { return a.re == 0.0 && a.im == 0.0; }
inline double cabs(cx a) { return std::hypot(a.re, a.im); }
const cx I_UNIT{0.0, 1.0};

thread_local std::string g_err;

// ---------------------------------------------------------------- hierarchy
struct Hierarchy {
  int K = 0, depth = 0, count = 0;
  std::vector<int> n;       // count*K
  std::vector<int> p1, m1;  // (count+1)*K, sentinel = count
};

using Filter = int (*)(const int*, int, int, void*);

// Breadth-first enumeration: a multi-index only spawns children by raising
// modes at or after the one it was created by, so each index is made once;
// the FIFO queue yields tier order (src/hrchy_space.cc:160-198).  With a
// filter, a candidate enters only if the filter accepts it (filter_flag,
// src/hrchy_space.cc:182-191), so a rejected index also drops the subtree it
// would have spawned.
Hierarchy build_hierarchy(int K, int depth, Filter filter = nullptr, void* user = nullptr) {
  Hierarchy h;
  h.K = K;
  h.depth = depth;
  std::map<std::vector<int>, int> index_of;
  std::queue<std::pair<std::vector<int>, int>> pending;
  pending.push({std::vector<int>(K, 0), 0});
  while (!pending.empty()) {
    auto [idx, first_mode] = pending.front();
    pending.pop();
    index_of[idx] = h.count++;
    h.n.insert(h.n.end(), idx.begin(), idx.end());
    int tier = 0;
    for (int v : idx) tier += v;
    if (tier + 1 > depth) continue;
    for (int k = first_mode; k < K; ++k) {
      ++idx[k];
      if (!filter || filter(idx.data(), K, tier + 1, user)) pending.push({idx, k});
      --idx[k];
    }
  }
  // Neighbour tables with the sentinel row (src/hrchy_space.cc:200-229).
  const int sentinel = h.count;
  h.p1.assign(static_cast<size_t>(h.count + 1) * K, sentinel);
  h.m1.assign(static_cast<size_t>(h.count + 1) * K, sentinel);
  std::vector<int> idx(K);
  for (int l = 0; l < h.count; ++l) {
    std::copy(h.n.begin() + static_cast<size_t>(l) * K, h.n.begin() + static_cast<size_t>(l + 1) * K, idx.begin());
    for (int k = 0; k < K; ++k) {
      ++idx[k];
      auto it = index_of.find(idx);
      if (it != index_of.end()) h.p1[static_cast<size_t>(l) * K + k] = it->second;
      idx[k] -= 2;
      if (idx[k] >= 0) {
        it = index_of.find(idx);
        if (it != index_of.end()) h.m1[static_cast<size_t>(l) * K + k] = it->second;
      }
      ++idx[k];
    }
  }
  return h;
}

// ---------------------------------------------------------------- model
struct Model {
  int n = 0, n2 = 0, U = 0, K = 0;
  std::vector<cx> H, V;        // n*n, U*n*n
  std::vector<int> bath_of;    // K: bath u of linear mode k
  std::vector<cx> sigma, s, a; // K
  std::vector<cx> s_delta;     // U
  std::vector<cx> ngamma;      // count
  bool sqrt_norm = false;      // LIBHEOM_SQRT_NORMALIZATION
  Hierarchy hs;
};

cx C(const double* p, size_t i) { return {p[2 * i], p[2 * i + 1]}; }

Model make_model(const heom_case* c) {
  Model m;
  m.n = c->n_level;
  m.n2 = m.n * m.n;
  m.U = c->n_noise;
  m.sqrt_norm = c->sqrt_normalization != 0;
  if (m.n <= 0 || m.U < 0 || c->max_depth < 0) throw std::invalid_argument("bad sizes");
  m.H.resize(m.n2);
  for (int i = 0; i < m.n2; ++i) m.H[i] = C(c->H, i);
  m.V.resize(static_cast<size_t>(m.U) * m.n2);
  for (size_t i = 0; i < m.V.size(); ++i) m.V[i] = C(c->V, i);
  std::vector<cx> gdiag;
  size_t off1 = 0, off2 = 0;
  for (int u = 0; u < m.U; ++u) {
    const int L = c->len_gamma[u];
    for (int k = 0; k < L; ++k) {
      m.bath_of.push_back(u);
      m.sigma.push_back(C(c->sigma, off1 + k));
      gdiag.push_back(C(c->gamma, off2 + static_cast<size_t>(k) * L + k));
      // s = S*phi_0 and a = A*phi_0 (heom.h:124-138), zero entries skipped.
      cx sv{0, 0}, av{0, 0};
      for (int j = 0; j < L; ++j) {
        const cx Sv = C(c->S, off2 + static_cast<size_t>(k) * L + j);
        const cx Av = C(c->A, off2 + static_cast<size_t>(k) * L + j);
        const cx ph = C(c->phi_0, off1 + j);
        if (!is_zero(Sv)) sv = sv + Sv * ph;
        if (!is_zero(Av)) av = av + Av * ph;
      }
      m.s.push_back(sv);
      m.a.push_back(av);
    }
    m.s_delta.push_back(C(c->s_delta, u));
    off1 += L;
    off2 += static_cast<size_t>(L) * L;
  }
  m.K = static_cast<int>(m.bath_of.size());
  m.hs = build_hierarchy(m.K, c->max_depth, c->hrchy_filter, c->filter_user);
  // ngamma_diag[l] = sum_k n_k gamma_kk, accumulated mode by mode (heom.h:94-104).
  m.ngamma.assign(m.hs.count, cx{0, 0});
  for (int l = 0; l < m.hs.count; ++l) {
    cx acc{0, 0};
    for (int k = 0; k < m.K; ++k) acc = acc + static_cast<double>(m.hs.n[static_cast<size_t>(l) * m.K + k]) * gdiag[k];
    m.ngamma[l] = acc;
  }
  return m;
}

// out_l = in_l^T for every n x n block (row-major <-> column-major storage).
void transpose_ados(const cx* in, cx* out, int n, int count) {
  const size_t n2 = static_cast<size_t>(n) * n;
  for (int l = 0; l < count; ++l)
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) out[l * n2 + static_cast<size_t>(j) * n + i] = in[l * n2 + static_cast<size_t>(i) * n + j];
}

// ---------------------------------------------------------------- RHS
// out_l = beta*out_l - alpha*D_l, with D_l the operator of heom_hilb.h:96-212.
void calc_diff(const Model& m, const cx* rho, cx* out, cx alpha, cx beta) {
  const int n = m.n, n2 = m.n2, K = m.K, count = m.hs.count;
#pragma omp parallel
  {
    std::vector<cx> D(n2), Phi(n2), Psi(n2), T(n2);
#pragma omp for schedule(static)
    for (int l = 0; l < count; ++l) {
      const cx* r = rho + static_cast<size_t>(l) * n2;
      // i[H, rho] + ngamma*rho
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          cx acc{0, 0};
          for (int k = 0; k < n; ++k) acc = acc + m.H[i * n + k] * r[k * n + j] - r[i * n + k] * m.H[k * n + j];
          D[i * n + j] = I_UNIT * acc + m.ngamma[l] * r[i * n + j];
        }
      for (int u = 0; u < m.U; ++u) {
        const cx* V = m.V.data() + static_cast<size_t>(u) * n2;
        // s_delta [V, [V, rho]]
        if (!is_zero(m.s_delta[u])) {
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
              cx acc{0, 0};
              for (int k = 0; k < n; ++k) acc = acc + V[i * n + k] * r[k * n + j] - r[i * n + k] * V[k * n + j];
              T[i * n + j] = acc;
            }
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
              cx acc{0, 0};
              for (int k = 0; k < n; ++k) acc = acc + V[i * n + k] * T[k * n + j] - T[i * n + k] * V[k * n + j];
              D[i * n + j] = D[i * n + j] + m.s_delta[u] * acc;
            }
        }
        // Phi = sum sigma_k rho_{n+1_k} + n_k s_k rho_{n-1_k};  Psi = -sum n_k a_k rho_{n-1_k}
        // (heom_hilb.h:170-196; with the square-root normalisation the +1 term
        // carries sqrt(n_k+1) and the -1 terms sqrt(n_k) instead of n_k)
        std::fill(Phi.begin(), Phi.end(), cx{0, 0});
        std::fill(Psi.begin(), Psi.end(), cx{0, 0});
        for (int k = 0; k < K; ++k) {
          if (m.bath_of[k] != u) continue;
          const int p = m.hs.p1[static_cast<size_t>(l) * K + k];
          if (p != count) {
            const cx* rp = rho + static_cast<size_t>(p) * n2;
            const double nk = m.hs.n[static_cast<size_t>(l) * K + k];
            const cx cp = m.sqrt_norm ? std::sqrt(nk + 1.0) * m.sigma[k] : m.sigma[k];
            for (int e = 0; e < n2; ++e) Phi[e] = Phi[e] + cp * rp[e];
          }
        }
        for (int k = 0; k < K; ++k) {
          if (m.bath_of[k] != u) continue;
          const int q = m.hs.m1[static_cast<size_t>(l) * K + k];
          if (q != count) {
            const double nk = m.hs.n[static_cast<size_t>(l) * K + k];
            const cx* rq = rho + static_cast<size_t>(q) * n2;
            const double f = m.sqrt_norm ? std::sqrt(nk) : nk;
            const cx cs = f * m.s[k], ca = -1.0 * (f * m.a[k]);
            for (int e = 0; e < n2; ++e) {
              Phi[e] = Phi[e] + cs * rq[e];
              Psi[e] = Psi[e] + ca * rq[e];
            }
          }
        }
        // i[V, Phi] + {V, Psi}
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            cx c1{0, 0}, c2{0, 0};
            for (int k = 0; k < n; ++k) {
              c1 = c1 + V[i * n + k] * Phi[k * n + j] - Phi[i * n + k] * V[k * n + j];
              c2 = c2 + V[i * n + k] * Psi[k * n + j] + Psi[i * n + k] * V[k * n + j];
            }
            D[i * n + j] = D[i * n + j] + I_UNIT * c1 + c2;
          }
      }
      cx* o = out + static_cast<size_t>(l) * n2;
      const bool beta0 = is_zero(beta);
      for (int e = 0; e < n2; ++e) o[e] = (beta0 ? cx{0, 0} : beta * o[e]) - alpha * D[e];
    }
  }
}

// ---------------------------------------------------------------- integrators
void axpy(cx a, const cx* x, cx* y, size_t n) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < static_cast<long long>(n); ++i) y[i] = y[i] + a * x[i];
}
void copyv(const cx* x, cx* y, size_t n) { std::memcpy(y, x, n * sizeof(cx)); }

double errnrm1(const cx* e, const cx* x1, const cx* x2, double atol, double rtol, size_t n) {
  double acc = 0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
  for (long long i = 0; i < static_cast<long long>(n); ++i) {
    const double q = cabs(e[i]) / (atol + rtol * std::max(cabs(x1[i]), cabs(x2[i])));
    acc += q * q;
  }
  return std::sqrt(acc) / std::sqrt(static_cast<double>(n));
}

struct Stats {
  long long rhs = 0, attempts = 0, accepted = 0;
};

struct Integrator {
  const Model& m;
  size_t N;
  std::vector<cx> buf;
  int kind;
  double dt_save = -1;
  Stats st;
  Integrator(const Model& mm, int k) : m(mm), N(static_cast<size_t>(mm.n2) * mm.hs.count), kind(k) {
    buf.assign(N * (k == 0 ? 4 : k == 1 ? 1 : 9), cx{0, 0});
  }
  void f(cx* out, const cx* in, double dt, double beta) {
    calc_diff(m, in, out, cx{dt, 0}, cx{beta, 0});
    ++st.rhs;
  }
  // rk4.h:40-65
  void rk4_step(cx* rho, double dt) {
    cx *rn = buf.data(), *k1 = rn + N, *k2 = k1 + N, *k3 = k2 + N;
    copyv(rho, rn, N);
    f(k1, rn, dt, 0);
    axpy({0.5, 0}, k1, rn, N);
    f(k2, rn, dt, 0);
    copyv(rho, rn, N);
    axpy({0.5, 0}, k2, rn, N);
    f(k3, rn, dt, 0);
    copyv(rho, rn, N);
    axpy({1, 0}, k3, rn, N);
    axpy({1, 0}, k3, k2, N);
    f(k3, rn, dt, 0);
    axpy({1.0 / 6.0, 0}, k1, rho, N);
    axpy({2.0 / 6.0, 0}, k2, rho, N);
    axpy({1.0 / 6.0, 0}, k3, rho, N);
  }
  // lsrk4.h:32-47
  void lsrk4_step(cx* rho, double dt) {
    cx* b = buf.data();
    const double B[4] = {1.0 / 3.0, 3.0 / 4.0, 2.0 / 3.0, 1.0 / 4.0};
    for (int s = 0; s < 4; ++s) {
      f(b, rho, dt, s == 0 ? 0.0 : -1.0);
      axpy({B[s], 0}, b, rho, N);
    }
  }
  // fixed_step_size_solver.h:29-52
  void fixed(cx* rho, double t0, double t1, double dt) {
    double t = t0;
    bool last = false;
    while (true) {
      if (t + dt - t1 > -std::numeric_limits<double>::epsilon()) {
        dt = t1 - t;
        last = true;
      }
      if (kind == 0)
        rk4_step(rho, dt);
      else
        lsrk4_step(rho, dt);
      ++st.attempts;
      ++st.accepted;
      t += dt;
      if (last) break;
    }
  }
  // rkdp.h:81-179
  void dp_step(cx* rho, double& t, double t_bound, double& dt, double atol, double rtol) {
    static const double A[6][5] = {{0, 0, 0, 0, 0},
                                   {1.0 / 5, 0, 0, 0, 0},
                                   {3.0 / 40, 9.0 / 40, 0, 0, 0},
                                   {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0},
                                   {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0},
                                   {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656}};
    static const double B[6] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84};
    static const double E[7] = {-71.0 / 57600, 0, 71.0 / 16695, -71.0 / 1920, 17253.0 / 339200, -22.0 / 525, 1.0 / 40};
    cx *rn = buf.data(), *rold = rn + N, *k[7];
    for (int i = 0; i < 7; ++i) k[i] = rold + N * (i + 1);
    copyv(rho, rold, N);
    int count = 0;
    bool accepted = false;
    while (!accepted) {
      if (++count > 1000) {
        t = t_bound;
        break;
      }
      if (t + dt > t_bound) dt = t_bound - t;
      for (int i = 0; i < 6; ++i) {
        copyv(rho, rn, N);
        for (int j = 0; j < i; ++j) axpy({A[i][j], 0}, k[j], rn, N);
        f(k[i], rn, dt, 0);
      }
      for (int i = 0; i < 6; ++i) axpy({B[i], 0}, k[i], rho, N);
      f(k[6], rho, dt, 0);
#pragma omp parallel for schedule(static)
      for (long long e = 0; e < static_cast<long long>(N); ++e) k[0][e] = E[0] * k[0][e];
      for (int i = 1; i < 7; ++i) axpy({E[i], 0}, k[i], k[0], N);
      const double err = errnrm1(k[0], rho, rold, atol, rtol, N);
      ++st.attempts;
      const double fac = std::pow(err, -0.2);
      if (err < 1.0) {
        t += dt;
        dt *= 0.9 * std::min(10.0, fac);
        accepted = true;
        ++st.accepted;
      } else {
        dt *= 0.9 * std::max(0.2, fac);
        if (dt < 1e-16) dt = 1e-16;
        copyv(rold, rho, N);
      }
    }
  }
  // adaptive_step_size_solver.h:32-56
  void adaptive(cx* rho, double t0, double t1, double dt, double atol, double rtol) {
    if (dt_save == -1) dt_save = dt;
    double t = t0, d = dt_save;
    while (true) {
      dp_step(rho, t, t1, d, atol, rtol);
      if (t >= t1) break;
    }
    dt_save = d;
  }
};

void check_case(const heom_case* c) {
  if (!c || !c->H || c->n_level <= 0) throw std::invalid_argument("invalid case");
}

}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int oracle_hrchy_filtered(int n_dim, int max_depth, Filter filter, void* user, int* n_hrchy, int* n_tab, int* p1_tab,
                          int* m1_tab) {
  try {
    Hierarchy h = build_hierarchy(n_dim, max_depth, filter, user);
    *n_hrchy = h.count;
    if (n_tab) std::copy(h.n.begin(), h.n.end(), n_tab);
    if (p1_tab) std::copy(h.p1.begin(), h.p1.end(), p1_tab);
    if (m1_tab) std::copy(h.m1.begin(), h.m1.end(), m1_tab);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int oracle_hrchy(int n_dim, int max_depth, int* n_hrchy, int* n_tab, int* p1_tab, int* m1_tab) {
  try {
    Hierarchy h = build_hierarchy(n_dim, max_depth);
    *n_hrchy = h.count;
    if (n_tab) std::copy(h.n.begin(), h.n.end(), n_tab);
    if (p1_tab) std::copy(h.p1.begin(), h.p1.end(), p1_tab);
    if (m1_tab) std::copy(h.m1.begin(), h.m1.end(), m1_tab);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int oracle_n_hrchy(const heom_case* c, int* n_hrchy) {
  try {
    check_case(c);
    int K = 0;
    for (int u = 0; u < c->n_noise; ++u) K += c->len_gamma[u];
    *n_hrchy = build_hierarchy(K, c->max_depth, c->hrchy_filter, c->filter_user).count;
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int oracle_calc_diff(const heom_case* c, int form, const double* rho, double* drho, const double* alpha,
                     const double* beta, int n_threads) {
  try {
    check_case(c);
    (void)form;
    oracle_set_threads(n_threads);
    Model m = make_model(c);
    if (c->col_major) {
      // the col_major order stores every ADO column-major; the operator is the same
      const size_t N = static_cast<size_t>(m.hs.count) * m.n2;
      std::vector<cx> x(N), y(N);
      transpose_ados(reinterpret_cast<const cx*>(rho), x.data(), m.n, m.hs.count);
      transpose_ados(reinterpret_cast<const cx*>(drho), y.data(), m.n, m.hs.count);
      calc_diff(m, x.data(), y.data(), cx{alpha[0], alpha[1]}, cx{beta[0], beta[1]});
      transpose_ados(y.data(), reinterpret_cast<cx*>(drho), m.n, m.hs.count);
      return 0;
    }
    calc_diff(m, reinterpret_cast<const cx*>(rho), reinterpret_cast<cx*>(drho), cx{alpha[0], alpha[1]},
              cx{beta[0], beta[1]});
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// stats (optional, 3 entries): RHS evaluations, step attempts, accepted steps.
int oracle_solve(const heom_case* c, int form, int solver, double* rho, const double* t_list, int n_t, double dt,
                 double atol, double rtol, double* rho_t, int n_threads, long long* stats) {
  try {
    check_case(c);
    (void)form;
    if (solver < 0 || solver > 2) throw std::invalid_argument("unknown solver");
    oracle_set_threads(n_threads);
    Model m = make_model(c);
    Integrator in(m, solver);
    const size_t N = in.N;
    std::vector<cx> work;
    cx* r = reinterpret_cast<cx*>(rho);
    if (c->col_major) {  // integrate the row-major transpose; the error norm is layout-free
      work.resize(N);
      transpose_ados(r, work.data(), m.n, m.hs.count);
      r = work.data();
    }
    auto snap = [&](int i) {
      if (!rho_t) return;
      cx* dst = reinterpret_cast<cx*>(rho_t) + N * i;
      if (c->col_major)
        transpose_ados(r, dst, m.n, m.hs.count);
      else
        std::memcpy(dst, r, N * sizeof(cx));
    };
    // solver_base::solve: callback at t_i, then one interval (solver_base.h:64-79).
    for (int i = 0; i < n_t - 1; ++i) {
      snap(i);
      if (solver == 2)
        in.adaptive(r, t_list[i], t_list[i + 1], dt, atol, rtol);
      else
        in.fixed(r, t_list[i], t_list[i + 1], dt);
    }
    if (n_t > 0) snap(n_t - 1);
    if (c->col_major) transpose_ados(r, reinterpret_cast<cx*>(rho), m.n, m.hs.count);
    if (stats) {
      stats[0] = in.st.rhs;
      stats[1] = in.st.attempts;
      stats[2] = in.st.accepted;
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"
