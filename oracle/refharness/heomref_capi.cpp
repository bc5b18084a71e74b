// Test infrastructure (oracle build only; never part of the product).
//
// C entry points around the reference's UNMODIFIED model, hierarchy and
// integrator code (heom_hilb.h, heom_liou.h, heom_ado.h, hrchy_space.cc,
// solver/rk4.h, solver/lsrk4.h, solver/rkdp.h, qme_solver.h), compiled from
// the reference tree by oracle/Makefile with the `loops` engine standing in
// for Eigen.  Used only to generate and check golden fixtures.
#include <any>
#include <cstring>
#include <exception>
#include <iostream>
#include <memory>
#include <string>

#include "harness_engine.h"
#include "linalg_engine/linalg_engine_nil.h"

#include "heom_hilb.h"
#include "heom_liou.h"
#include "heom_ado.h"
#include "hrchy_space.h"
#include "redfield_hilb.h"
#include "redfield_liou.h"
#include "qme_solver.h"
#include "solver/lsrk4.h"
#include "solver/rk4.h"
#include "solver/rkdp.h"

#include "../heom_case.h"

namespace libheom {
// Defined in hrchy_space.cc:68-71 but not declared in its header.
long long calc_hrchy_element_count(int level, int dim);
}

using namespace libheom;
using cplx = complex128;

namespace {

thread_local std::string g_err;

cplx C(const double* p, size_t i) { return cplx(p[2 * i], p[2 * i + 1]); }

// Logical (row, col) entries through the reference's own push(), which stores
// them as data[row][col] (row_major) or data[col][row] (col_major).
template <order_t order>
void fill_lil(lil_matrix<dynamic, cplx, order, nil>& m, int rows, int cols, const double* src) {
  m.set_shape(rows, cols);
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) {
      const cplx v = C(src, static_cast<size_t>(r) * cols + c);
      if (v != cplx(0.0, 0.0)) m.push(r, c, v);
    }
}

template <class Q>
void fill_params(Q& q, const heom_case* c) {
  const int n = c->n_level;
  q.n_level = n;
  q.n_level_2 = n * n;
  fill_lil(q.H, n, n, c->H);
  q.alloc_noises(c->n_noise);
  size_t off1 = 0, off2 = 0;
  for (int u = 0; u < c->n_noise; ++u) {
    const int L = c->len_gamma[u];
    fill_lil(q.V[u], n, n, c->V + 2 * static_cast<size_t>(u) * n * n);
    q.len_gamma[u] = L;
    fill_lil(q.gamma[u], L, L, c->gamma + 2 * off2);
    fill_lil(q.S[u], L, L, c->S + 2 * off2);
    fill_lil(q.A[u], L, L, c->A + 2 * off2);
    q.phi_0[u].resize(L);
    q.sigma[u].resize(L);
    for (int k = 0; k < L; ++k) {
      q.phi_0[u][k] = C(c->phi_0, off1 + k);
      q.sigma[u][k] = C(c->sigma, off1 + k);
    }
    q.s_delta[u] = C(c->s_delta, u);
    off1 += L;
    off2 += static_cast<size_t>(L) * L;
  }
}

using hilb_t = heom_hilb<dynamic, cplx, dense_matrix, row_major, loops>;
using liou_t = heom_liou<dynamic, cplx, sparse_matrix, row_major, row_major, loops>;
using ado_t = heom_ado<dynamic, cplx, sparse_matrix, row_major, row_major, loops>;
// col_major: heom_hilb only (the harness's set-up algebra covers the gemv
// heom::set_param needs in that order, not the Liouville-space kron products)
using hilb_c_t = heom_hilb<dynamic, cplx, dense_matrix, col_major, loops>;
using rf_hilb_t = redfield_hilb<dynamic, cplx, dense_matrix, row_major, loops>;
using rf_liou_t = redfield_liou<dynamic, cplx, sparse_matrix, row_major, row_major, loops>;

void check_normalisation(const heom_case* c) {
#ifdef LIBHEOM_SQRT_NORMALIZATION
  const int built_sqrt = 1;
#else
  const int built_sqrt = 0;
#endif
  // the normalisation is the reference's compile-time switch: one build per choice
  if (c->sqrt_normalization != built_sqrt)
    throw std::invalid_argument("this reference build has the other normalisation");
}

std::unique_ptr<qme_base<cplx, col_major, loops>> make_qme_c(int form, const heom_case* c, int threads, loops* eng,
                                                             int* n_hrchy) {
  check_normalisation(c);
  if (form != 0) throw std::invalid_argument("col_major: heom_hilb only in this harness");
  auto q = std::make_unique<hilb_c_t>(c->max_depth, 1, threads);
  fill_params(*q, c);
  q->set_param(eng);
  *n_hrchy = q->get_n_hrchy();
  return q;
}

std::unique_ptr<qme_base<cplx, row_major, loops>> make_qme(int form, const heom_case* c, int threads,
                                                             loops* eng, int* n_hrchy) {
  check_normalisation(c);
  if (c->col_major) throw std::invalid_argument("make_qme: row_major model expected");
  if (form == 0) {
    auto q = std::make_unique<hilb_t>(c->max_depth, 1, threads);
    fill_params(*q, c);
    q->set_param(eng);
    *n_hrchy = q->get_n_hrchy();
    return q;
  } else if (form == 1) {
    auto q = std::make_unique<liou_t>(c->max_depth, 1, threads);
    fill_params(*q, c);
    q->set_param(eng);
    *n_hrchy = q->get_n_hrchy();
    return q;
  } else if (form == 2) {
    auto q = std::make_unique<ado_t>(c->max_depth, 1, threads);
    fill_params(*q, c);
    q->set_param(eng);
    *n_hrchy = q->get_n_hrchy();
    return q;
  } else if (form == 3) {  // redfield_hilb (redfield_hilb.h:18-91): no hierarchy
    auto q = std::make_unique<rf_hilb_t>();
    fill_params(*q, c);
    q->set_param(eng);
    *n_hrchy = 1;
    return q;
  } else if (form == 4) {  // redfield_liou (redfield_liou.h:18-104)
    auto q = std::make_unique<rf_liou_t>();
    fill_params(*q, c);
    q->set_param(eng);
    *n_hrchy = 1;
    return q;
  }
  throw std::invalid_argument("unknown form");
}

template <class Q>
void diff_with(Q* q, loops* eng, const double* rho, double* drho, const double* alpha, const double* beta) {
  const int size = q->main_size();
  const int tsize = std::max(1, q->temp_size());
  std::vector<cplx> x(size), y(size), temp(tsize);
  std::memcpy(x.data(), rho, sizeof(cplx) * size);
  std::memcpy(y.data(), drho, sizeof(cplx) * size);
  q->calc_diff_impl(eng, y.data(), x.data(), cplx(alpha[0], alpha[1]), cplx(beta[0], beta[1]), temp.data());
  std::memcpy(drho, y.data(), sizeof(cplx) * size);
}

template <order_t order>
void solve_with(qme_base<cplx, order, loops>* q, loops* eng, int solver, double* rho, const double* t_list, int n_t,
                double dt, double atol, double rtol, double* rho_t) {
  const int size = q->main_size();
  std::unique_ptr<solver_base<cplx, order, loops>> s;
  if (solver == 0)
    s = std::make_unique<rk4<cplx, order, loops>>();
  else if (solver == 1)
    s = std::make_unique<lsrk4<cplx, order, loops>>();
  else if (solver == 2)
    s = std::make_unique<rkdp<cplx, order, loops>>();
  else
    throw std::invalid_argument("unknown solver");
  qme_solver<cplx, order, loops> qs(eng, q, s.get());
  kwargs_t kw;
  kw["dt"] = dt;
  kw["atol"] = atol;
  kw["rtol"] = rtol;
  cplx* r = reinterpret_cast<cplx*>(rho);
  int idx = 0;
  qs.solve(r, t_list, n_t,
           [&](double) {
             if (rho_t) std::memcpy(rho_t + 2 * static_cast<size_t>(idx) * size, r, sizeof(cplx) * size);
             ++idx;
           },
           kw);
}

}  // namespace

extern "C" {

const char* heomref_last_error() { return g_err.c_str(); }

// Hierarchy tables from the reference's alloc_hrchy_space (hrchy_space.cc:137-231).
// n_tab: n_hrchy*n_dim, p1_tab/m1_tab: (n_hrchy+1)*n_dim; any may be null.
int heomref_hrchy(int n_dim, int max_depth, int* n_hrchy, int* n_tab, int* p1_tab, int* m1_tab) {
  try {
    hrchy_space hs;
    hs.n_dim = n_dim;
    const int count = alloc_hrchy_space(hs, max_depth);
    *n_hrchy = count;
    for (int l = 0; l <= count; ++l)
      for (int k = 0; k < n_dim; ++k) {
        if (n_tab && l < count) n_tab[static_cast<size_t>(l) * n_dim + k] = hs.n[l][k];
        if (p1_tab) p1_tab[static_cast<size_t>(l) * n_dim + k] = hs.ptr_p1[l][k];
        if (m1_tab) m1_tab[static_cast<size_t>(l) * n_dim + k] = hs.ptr_m1[l][k];
      }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// alloc_hrchy_space with a hierarchy filter and filter_flag = true
// (hrchy_space.cc:137-231); heom::set_param never passes one (heom.h:80-91).
int heomref_hrchy_filtered(int n_dim, int max_depth, int (*filter)(const int*, int, int, void*), void* user,
                           int* n_hrchy, int* n_tab, int* p1_tab, int* m1_tab) {
  try {
    hrchy_space hs;
    hs.n_dim = n_dim;
    auto f = [&](std::vector<int> index, int depth) -> bool { return filter(index.data(), n_dim, depth, user) != 0; };
    std::streambuf* keep = std::cerr.rdbuf(nullptr);  // the reference warns on stderr at max_depth
    const int count = alloc_hrchy_space(hs, max_depth, [](int, int) {}, 1024, f, true);
    std::cerr.rdbuf(keep);
    *n_hrchy = count;
    for (int l = 0; l <= count; ++l)
      for (int k = 0; k < n_dim; ++k) {
        if (n_tab && l < count) n_tab[static_cast<size_t>(l) * n_dim + k] = hs.n[l][k];
        if (p1_tab) p1_tab[static_cast<size_t>(l) * n_dim + k] = hs.ptr_p1[l][k];
        if (m1_tab) m1_tab[static_cast<size_t>(l) * n_dim + k] = hs.ptr_m1[l][k];
      }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

long long heomref_element_count(int level, int dim) { return calc_hrchy_element_count(level, dim); }

int heomref_n_hrchy(const heom_case* c, int* n_hrchy) {
  try {
    loops eng;
    make_qme(0, c, 1, &eng, n_hrchy);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// One right-hand-side evaluation: drho = beta*drho - alpha*D(rho)  (heom_hilb.h:70-215).
int heomref_calc_diff(const heom_case* c, int form, const double* rho, double* drho, const double* alpha,
                      const double* beta, int n_threads) {
  try {
    loops eng;
    int nh = 0;
    if (c->col_major) {
      auto q = make_qme_c(form, c, n_threads, &eng, &nh);
      diff_with(q.get(), &eng, rho, drho, alpha, beta);
      return 0;
    }
    auto q = make_qme(form, c, n_threads, &eng, &nh);
    const int size = q->main_size();
    const int tsize = std::max(1, q->temp_size());
    std::vector<cplx> x(size), y(size), temp(tsize);
    std::memcpy(x.data(), rho, sizeof(cplx) * size);
    std::memcpy(y.data(), drho, sizeof(cplx) * size);
    q->calc_diff_impl(&eng, y.data(), x.data(), cplx(alpha[0], alpha[1]), cplx(beta[0], beta[1]), temp.data());
    std::memcpy(drho, y.data(), sizeof(cplx) * size);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Propagation through qme_solver::solve (qme_solver.h:44-52).  rho holds the
// initial state and receives the final one; rho_t (optional) receives the
// state at every output time, as seen by the reference's callback.
int heomref_solve(const heom_case* c, int form, int solver, double* rho, const double* t_list, int n_t,
                  double dt, double atol, double rtol, double* rho_t, int n_threads) {
  try {
    loops eng;
    int nh = 0;
    if (c->col_major) {
      auto q = make_qme_c(form, c, n_threads, &eng, &nh);
      solve_with<col_major>(q.get(), &eng, solver, rho, t_list, n_t, dt, atol, rtol, rho_t);
    } else {
      auto q = make_qme(form, c, n_threads, &eng, &nh);
      solve_with<row_major>(q.get(), &eng, solver, rho, t_list, n_t, dt, atol, rtol, rho_t);
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"
