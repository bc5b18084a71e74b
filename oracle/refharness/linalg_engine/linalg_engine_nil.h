// Test infrastructure (oracle build only; never part of the product).
//
// Set-up-time ("nil") algebra on LIL matrices, written for this harness.  The
// reference generates this header from `include/linalg_engine/
// linalg_engine_nil.h.j2`; the harness supplies its own implementation of the
// few dispatch points the HEOM set-up uses, with the same semantics:
//   gemv  (heom.h:130-137, s = S phi_0)          linalg_engine_nil.h.j2:137-163
//   axpym (heom_liou.h:96-99, heom_ado.h:336-337) linalg_engine_nil.h.j2:38-56
//   gemm  (heom_liou.h:91, Xi = -s_delta Phi^2)   linalg_engine_nil.h.j2:59-96
//   kron_x_1 / kron_1_x_T (heom_liou.h:72-87)     linalg_engine_nil.h.j2:197-299
//   dotu / gevm / lu_solve (redfield.h:32-41,66-73) linalg_engine_nil.h.j2:467-533
// The row-major orders are provided, and the col-major gemv that heom_hilb's
// set-up needs in that order.
#ifndef HEOMREF_SHIM_LINALG_ENGINE_NIL_H
#define HEOMREF_SHIM_LINALG_ENGINE_NIL_H

#include <vector>

#include "env.h"
#include "linalg_engine/linalg_engine.h"
#include "linalg_engine/lil_matrix.h"

namespace libheom {

template <typename dtype>
struct gemv_impl<dynamic, dtype, lil_matrix, row_major, nil> {
  static void func(nil*, dtype alpha, lil_matrix<dynamic, dtype, row_major, nil>& A,
                   dtype* x, dtype beta, dtype* y, int n) {
    for (int r = 0; r < n; ++r) y[r] *= beta;
    for (const auto& row : A.data)
      for (const auto& e : row.second) y[row.first] += alpha * e.second * x[e.first];
  }
};

// col_major LIL stores A(r, c) as data[c][r] (lil_matrix.h.j2:156-163).
template <typename dtype>
struct gemv_impl<dynamic, dtype, lil_matrix, col_major, nil> {
  static void func(nil*, dtype alpha, lil_matrix<dynamic, dtype, col_major, nil>& A,
                   dtype* x, dtype beta, dtype* y, int n) {
    for (int r = 0; r < n; ++r) y[r] *= beta;
    for (const auto& col : A.data)
      for (const auto& e : col.second) y[e.first] += alpha * e.second * x[col.first];
  }
};

template <typename dtype, order_t order>
struct axpym_impl<dynamic, dtype, lil_matrix, order, nil> {
  static void func(nil*, dtype alpha, const lil_matrix<dynamic, dtype, order, nil>& x,
                   lil_matrix<dynamic, dtype, order, nil>& y, int) {
    for (const auto& row : x.data)
      for (const auto& e : row.second) y.data[row.first][e.first] += alpha * e.second;
  }
};

template <typename dtype>
struct gemm_impl<dynamic, dtype, lil_matrix, row_major, nil> {
  static void func(nil*, dtype alpha, lil_matrix<dynamic, dtype, row_major, nil>& A,
                   lil_matrix<dynamic, dtype, row_major, nil>& B, dtype beta,
                   lil_matrix<dynamic, dtype, row_major, nil>& C, int) {
    for (auto& row : C.data)
      for (auto& e : row.second) e.second *= beta;
    for (const auto& arow : A.data) {
      for (const auto& ae : arow.second) {
        auto it = B.data.find(ae.first);
        if (it == B.data.end()) continue;
        for (const auto& be : it->second)
          C.data[arow.first][be.first] += alpha * ae.second * be.second;
      }
    }
    C.optimize();
  }
};

// y = beta*y + alpha*(x (x) 1): entry x(r,c) lands on (r*n+k, c*n+k) for all k.
template <typename dtype>
struct kron_x_1_impl<dynamic, dtype, lil_matrix, row_major, row_major, nil> {
  static void func(nil*, const dtype& alpha, const lil_matrix<dynamic, dtype, row_major, nil>& x,
                   const dtype& beta, lil_matrix<dynamic, dtype, row_major, nil>& y,
                   bool conj = false) {
    if (beta == zero<dtype>()) {
      y.data.clear();
    } else {
      for (auto& row : y.data)
        for (auto& e : row.second) e.second *= beta;
    }
    const int n = std::get<0>(x.shape);
    for (const auto& row : x.data) {
      for (const auto& e : row.second) {
        if (e.second == zero<dtype>()) continue;
        const int r = conj ? e.first : row.first;
        const int c = conj ? row.first : e.first;
        dtype v = conj ? std::conj(e.second) : e.second;
        v *= alpha;
        for (int k = 0; k < n; ++k) y.data[r * n + k][c * n + k] += v;
      }
    }
  }
};

// y = beta*y + alpha*(1 (x) x^T): entry x(r,c) lands on (k*n+c, k*n+r) for all k.
template <typename dtype>
struct kron_1_x_T_impl<dynamic, dtype, lil_matrix, row_major, row_major, nil> {
  static void func(nil*, const dtype& alpha, const lil_matrix<dynamic, dtype, row_major, nil>& x,
                   const dtype& beta, lil_matrix<dynamic, dtype, row_major, nil>& y,
                   bool conj = false) {
    if (beta == zero<dtype>()) {
      y.data.clear();
    } else {
      for (auto& row : y.data)
        for (auto& e : row.second) e.second *= beta;
    }
    const int n = std::get<0>(x.shape);
    for (const auto& row : x.data) {
      for (const auto& e : row.second) {
        if (e.second == zero<dtype>()) continue;
        const int r = conj ? e.first : row.first;
        const int c = conj ? row.first : e.first;
        dtype v = conj ? std::conj(e.second) : e.second;
        v *= alpha;
        for (int k = 0; k < n; ++k) y.data[k * n + c][k * n + r] += v;
      }
    }
  }
};

// dotu (linalg_engine.h:207-217): sum_i x_i y_i (no conjugation).
template <typename dtype>
struct dotu_impl<dynamic, dtype, nil> {
  static dtype func(nil*, dtype* x, dtype* y, int n) {
    dtype acc = zero<dtype>();
    for (int i = 0; i < n; ++i) acc += x[i] * y[i];
    return acc;
  }
};

// gevm (linalg_engine.h:374-394): y = alpha x^T A + beta y.
template <typename dtype>
struct gevm_impl<dynamic, dtype, lil_matrix, row_major, nil> {
  static void func(nil*, dtype alpha, dtype* x, lil_matrix<dynamic, dtype, row_major, nil>& A, dtype beta,
                   dtype* y, int n) {
    std::vector<dtype> out(n, zero<dtype>());
    for (const auto& row : A.data)
      for (const auto& e : row.second) out[e.first] += x[row.first] * e.second;
    for (int i = 0; i < n; ++i) y[i] = (beta == zero<dtype>() ? zero<dtype>() : beta * y[i]) + alpha * out[i];
  }
};

// lu_solve (the reference's nil engine, linalg_engine_nil.h.j2:467-533): x
// with A x = b by Gaussian elimination with partial pivoting (the Redfield
// correlation's (gamma - i omega) x = phi_0).
template <typename dtype>
void lu_solve(const lil_matrix<dynamic, dtype, row_major, nil>& A, const std::vector<dtype>& b,
              std::vector<dtype>& x) {
  const int n = std::get<0>(A.shape);
  std::vector<dtype> m(static_cast<size_t>(n) * n, zero<dtype>());
  for (const auto& row : A.data)
    for (const auto& e : row.second) m[row.first * n + e.first] = e.second;
  x.assign(b.begin(), b.end());
  for (int i = 0; i < n; ++i) {
    int piv = i;
    for (int r = i + 1; r < n; ++r)
      if (std::abs(m[r * n + i]) > std::abs(m[piv * n + i])) piv = r;
    if (piv != i) {
      for (int c = 0; c < n; ++c) std::swap(m[i * n + c], m[piv * n + c]);
      std::swap(x[i], x[piv]);
    }
    for (int r = i + 1; r < n; ++r) {
      if (m[r * n + i] == zero<dtype>()) continue;
      const dtype f = m[r * n + i] / m[i * n + i];
      for (int c = i; c < n; ++c) m[r * n + c] -= f * m[i * n + c];
      x[r] -= f * x[i];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    dtype acc = x[i];
    for (int c = i + 1; c < n; ++c) acc -= m[i * n + c] * x[c];
    x[i] = acc / m[i * n + i];
  }
}

}  // namespace libheom

#endif
