// heomgb.hpp -- C++17 mirror of libheom's model / solver classes over the C ABI.
//
// The class names, public members and call sequence follow the reference, so
// a caller written against libheom changes only its includes and the template
// arguments:
//
//   libheom::heom_hilb<dynamic,complex128,dense_matrix,row_major,eigen> (heom_hilb.h:18-216)
//   libheom::rk4 / lsrk4 / rkdp<complex128,row_major,eigen>              (solver/*.h)
//   libheom::qme_solver<complex128,row_major,eigen>                      (qme_solver.h:18-53)
// become
//   heomgb::heom_hilb, heomgb::rk4 / lsrk4 / rkdp, heomgb::qme_solver.
//
// Public parameter members (qme_base.h:32-67) are LIL matrices as in the
// reference (`data[row][col] = value`, lil_matrix.h.j2:22-183).  The engine
// argument of set_param / qme_solver is accepted and ignored: the device path
// is the only path.  Errors throw heomgb::error (the reference throws
// std::out_of_range / std::bad_any_cast for kwargs and exits on CUDA errors).
#ifndef HEOMGB_HPP
#define HEOMGB_HPP

#include <any>
#include <complex>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "heomgb.h"

namespace heomgb {

using complex128 = std::complex<double>;
using kwargs_t = std::map<std::string, std::any>;

class error : public std::runtime_error {
 public:
  error(heomgb_status s, const std::string& m) : std::runtime_error(m), status(s) {}
  heomgb_status status;
};

inline void check(heomgb_status s) {
  if (s != HEOMGB_OK) throw error(s, heomgb_last_error());
}

// Sparse LIL matrix with the reference's public surface (set_shape, push, data).
class lil_matrix {
 public:
  std::tuple<int, int> shape{0, 0};
  std::map<int, std::map<int, complex128>> data;
  void set_shape(int rows, int cols) {
    shape = {rows, cols};
    data.clear();
  }
  void push(int row, int col, const complex128& v) { data[row][col] += v; }
  std::vector<complex128> dense(int rows, int cols) const {
    std::vector<complex128> out(static_cast<size_t>(rows) * cols);
    for (const auto& r : data)
      for (const auto& e : r.second)
        if (r.first < rows && e.first < cols) out[static_cast<size_t>(r.first) * cols + e.first] = e.second;
    return out;
  }
};

class qme_base {
 public:
  int n_level = 0;
  int n_level_2 = 0;
  lil_matrix H;
  int n_noise = 0;
  std::unique_ptr<lil_matrix[]> V;
  std::unique_ptr<int[]> len_gamma;
  std::unique_ptr<lil_matrix[]> gamma;
  std::unique_ptr<std::vector<complex128>[]> phi_0;
  std::unique_ptr<std::vector<complex128>[]> sigma;
  std::unique_ptr<lil_matrix[]> S;
  std::unique_ptr<lil_matrix[]> A;
  std::unique_ptr<complex128[]> s_delta;
  heomgb_precision precision = HEOMGB_FP64;
  // the reference's LIBHEOM_SQRT_NORMALIZATION build switch, as a member
  heomgb_normalization normalization = HEOMGB_NORM_INTEGER;
  // the reference's `order` template argument, as a member
  heomgb_order order = HEOMGB_ROW_MAJOR;

  virtual ~qme_base() { release(); }

  void alloc_noises(int n) {
    n_noise = n;
    V.reset(new lil_matrix[n]);
    len_gamma.reset(new int[n]());
    gamma.reset(new lil_matrix[n]);
    phi_0.reset(new std::vector<complex128>[n]);
    sigma.reset(new std::vector<complex128>[n]);
    S.reset(new lil_matrix[n]);
    A.reset(new lil_matrix[n]);
    s_delta.reset(new complex128[n]());
  }

  int main_size() const { return static_cast<int>(size_ll()); }
  heomgb_qme* handle() const { return h_; }

  // calc_diff_impl(obj, drho_dt, rho, alpha, beta, temp) -- heom_hilb.h:70-215 (host arrays)
  void calc_diff_impl(void* /*engine*/, complex128* drho_dt, complex128* rho, complex128 alpha, complex128 beta,
                      void* /*temp*/ = nullptr) {
    const double a[2] = {alpha.real(), alpha.imag()}, b[2] = {beta.real(), beta.imag()};
    check(heomgb_qme_calc_diff(h_, reinterpret_cast<double*>(drho_dt), reinterpret_cast<const double*>(rho), a, b));
  }

 protected:
  heomgb_qme* h_ = nullptr;
  long long size_ll() const {
    long long s = 0;
    if (h_) check(heomgb_qme_main_size(h_, &s));
    return s;
  }
  void release() {
    if (h_) heomgb_qme_destroy(h_);
    h_ = nullptr;
  }
  void build(heomgb_form form, int max_depth, int n_inner, int n_outer) {
    release();
    if (n_level_2 != 0 && n_level_2 != n_level * n_level) throw error(HEOMGB_ERR_INVALID_ARGUMENT, "n_level_2 != n_level^2");
    check(heomgb_qme_create(form, max_depth, n_inner, n_outer, &h_));
    const int n = n_level;
    auto Hd = H.dense(n, n);
    check(heomgb_qme_set_hamiltonian(h_, n, reinterpret_cast<const double*>(Hd.data())));
    check(heomgb_qme_alloc_noises(h_, n_noise));
    for (int u = 0; u < n_noise; ++u) {
      const int L = len_gamma[u];
      auto Vd = V[u].dense(n, n);
      auto gd = gamma[u].dense(L, L), Sd = S[u].dense(L, L), Ad = A[u].dense(L, L);
      std::vector<complex128> ph(phi_0[u]), sg(sigma[u]);
      ph.resize(L);
      sg.resize(L);
      const complex128 sd = s_delta[u];
      check(heomgb_qme_set_noise(h_, u, reinterpret_cast<const double*>(Vd.data()), L,
                                 reinterpret_cast<const double*>(gd.data()), reinterpret_cast<const double*>(ph.data()),
                                 reinterpret_cast<const double*>(sg.data()), reinterpret_cast<const double*>(Sd.data()),
                                 reinterpret_cast<const double*>(Ad.data()), reinterpret_cast<const double*>(&sd)));
    }
    check(heomgb_qme_set_precision(h_, precision));
    check(heomgb_qme_set_normalization(h_, normalization));
    check(heomgb_qme_set_order(h_, order));
    check(heomgb_qme_set_param(h_));
  }
};

template <heomgb_form Form>
class heom_model : public qme_base {
 public:
  // heom_hilb(int max_depth, int n_inner_threads, int n_outer_threads) -- heom_hilb.h:41-43
  heom_model(int max_depth, int n_inner_threads, int n_outer_threads)
      : max_depth_(max_depth), n_inner_(n_inner_threads), n_outer_(n_outer_threads) {}
  void set_param(void* /*engine*/ = nullptr) { build(Form, max_depth_, n_inner_, n_outer_); }
  int get_n_hrchy() const {
    int v = 0;
    check(heomgb_qme_get_n_hrchy(h_, &v));
    return v;
  }

 private:
  int max_depth_, n_inner_, n_outer_;
};

using heom_hilb = heom_model<HEOMGB_HILB>;
using heom_liou = heom_model<HEOMGB_LIOU>;
using heom_ado = heom_model<HEOMGB_ADO>;

// redfield_hilb() / redfield_liou() -- redfield_hilb.h:36-37, redfield_liou.h:38-39
template <heomgb_form Form>
class redfield_model : public qme_base {
 public:
  redfield_model() = default;
  void set_param(void* /*engine*/ = nullptr) { build(Form, 0, 1, 1); }
};
using redfield_hilb = redfield_model<HEOMGB_REDFIELD_HILB>;
using redfield_liou = redfield_model<HEOMGB_REDFIELD_LIOU>;

class solver_base {
 public:
  explicit solver_base(heomgb_solver_kind k) { check(heomgb_solver_create(k, &h_)); }
  virtual ~solver_base() { heomgb_solver_destroy(h_); }
  solver_base(const solver_base&) = delete;
  solver_base& operator=(const solver_base&) = delete;
  heomgb_solver* handle() const { return h_; }

 private:
  heomgb_solver* h_ = nullptr;
};
struct rk4 : solver_base {
  rk4() : solver_base(HEOMGB_RK4) {}
};
struct lsrk4 : solver_base {
  lsrk4() : solver_base(HEOMGB_LSRK4) {}
};
struct rkdp : solver_base {
  rkdp() : solver_base(HEOMGB_RKDP) {}
};

class qme_solver {
 public:
  // qme_solver(engine, qme, solver) -- qme_solver.h:26-35
  qme_solver(void* /*engine*/, qme_base* qme, solver_base* solver) {
    check(heomgb_qme_solver_create(qme->handle(), solver->handle(), &h_));
  }
  ~qme_solver() { heomgb_qme_solver_destroy(h_); }
  qme_solver(const qme_solver&) = delete;
  qme_solver& operator=(const qme_solver&) = delete;

  // solve(rho, t_list, n_t, callback, kwargs) -- qme_solver.h:44-52
  void solve(complex128* rho, const double* t_list, int n_t, std::function<void(double)> callback,
             const kwargs_t& kwargs) {
    heomgb_kwargs kw{};
    read(kwargs, "dt", kw.dt, kw.has_dt);
    read(kwargs, "atol", kw.atol, kw.has_atol);
    read(kwargs, "rtol", kw.rtol, kw.has_rtol);
    check(heomgb_qme_solver_solve(h_, reinterpret_cast<double*>(rho), t_list, n_t, &trampoline, &callback, &kw));
  }

 private:
  heomgb_qme_solver* h_ = nullptr;
  static void trampoline(double t, void* user) {
    auto* f = static_cast<std::function<void(double)>*>(user);
    if (f && *f) (*f)(t);
  }
  // The reference any_casts to real_t<dtype> (double); a wrong type throws bad_any_cast.
  static void read(const kwargs_t& kw, const char* key, double& v, int& has) {
    auto it = kw.find(key);
    if (it == kw.end()) return;
    v = std::any_cast<double>(it->second);
    has = 1;
  }
};

}  // namespace heomgb

#endif  // HEOMGB_HPP
