// Test infrastructure (oracle build only; never part of the product).
//
// `loops`: a plain-loop linear-algebra engine that stands in for the
// reference's Eigen engine (unbuildable here: the Eigen submodule is empty).
// It specialises the reference's dispatch points (`linalg_engine.h:136-563`)
// for the dynamic size only:
//   nullify/copy/scal/axpy        linalg_engine_eigen.h.j2:288-343
//   errnrm1                       linalg_engine_eigen.h.j2:360-379
//   gemm (matrix*ptr, ptr*matrix) linalg_engine_eigen.h.j2:381-412
//   gemv (dense and CSR)          linalg_engine_eigen.h.j2:414-433
// plus `dense_matrix` / `sparse_matrix` containers with `import` from LIL
// (dense_matrix_eigen.h.j2:62-80, sparse_matrix_eigen.h.j2:53-75).
// Semantics follow BLAS: a beta of exactly zero never reads the output.
#ifndef HEOMREF_HARNESS_ENGINE_H
#define HEOMREF_HARNESS_ENGINE_H

#include <algorithm>
#include <cmath>
#include <vector>

#include "linalg_engine/linalg_engine.h"
#include "linalg_engine/dense_matrix.h"
#include "linalg_engine/sparse_matrix.h"
#include "linalg_engine/lil_matrix.h"

namespace libheom {

class loops : public linalg_engine_base {
 public:
  loops() : linalg_engine_base() {}
  explicit loops(loops* parent) : linalg_engine_base(parent) {}
  loops* create_child() override { return new loops(this); }
};

template <> struct engine_env_impl<loops> { typedef env_cpu value; };
template <> inline bool is_supported<loops>() { return true; }

template <typename T>
struct nullify_impl<dynamic, T, loops> {
  static void func(loops*, T* x, int n) {
    for (int i = 0; i < n; ++i) x[i] = T();
  }
};

template <typename T>
struct copy_impl<dynamic, T, loops> {
  static void func(loops*, T* x, T* y, int n) {
    for (int i = 0; i < n; ++i) y[i] = x[i];
  }
};

template <typename T>
struct scal_impl<dynamic, T, loops> {
  static void func(loops*, T a, T* y, int n) {
    if (a == zero<T>()) {
      for (int i = 0; i < n; ++i) y[i] = zero<T>();
    } else {
      for (int i = 0; i < n; ++i) y[i] = a * y[i];
    }
  }
};

template <typename T>
struct axpy_impl<dynamic, T, loops> {
  static void func(loops*, T a, T* x, T* y, int n) {
    for (int i = 0; i < n; ++i) y[i] += a * x[i];
  }
};

template <typename R>
struct errnrm1_impl<dynamic, R, loops> {
  static R func(loops*, std::complex<R>* e, std::complex<R>* x1, std::complex<R>* x2, R atol,
                R rtol, int n) {
    R acc = 0;
    for (int i = 0; i < n; ++i) {
      const R m = std::max(std::abs(x1[i]), std::abs(x2[i]));
      const R q = std::abs(e[i]) / (atol + rtol * m);
      acc += q * q;
    }
    return std::sqrt(acc) / std::sqrt(static_cast<R>(n));
  }
};

// Dense square matrix in the requested storage order.
template <typename dtype, order_t order>
class dense_matrix<dynamic, dtype, order, loops> : public matrix_base<dynamic, dtype, order, loops> {
 public:
  int rows = 0, cols = 0;
  std::vector<dtype> data;
  dtype at(int r, int c) const { return order == row_major ? data[r * cols + c] : data[c * rows + r]; }
  void import(lil_matrix<dynamic, dtype, order, nil>& src) {
    rows = std::get<0>(src.shape);
    cols = std::get<1>(src.shape);
    data.assign(static_cast<size_t>(rows) * cols, zero<dtype>());
    const int stride = order == row_major ? cols : rows;
    for (const auto& row : src.data)
      for (const auto& e : row.second) data[static_cast<size_t>(row.first) * stride + e.first] = e.second;
  }
};

// CSR matrix (row-major semantics of the logical matrix).
template <typename dtype, order_t order>
class sparse_matrix<dynamic, dtype, order, loops> : public matrix_base<dynamic, dtype, order, loops> {
 public:
  int rows = 0, cols = 0;
  std::vector<int> ptr, idx;
  std::vector<dtype> val;
  void import(lil_matrix<dynamic, dtype, order, nil>& src) {
    rows = std::get<0>(src.shape);
    cols = std::get<1>(src.shape);
    std::vector<std::vector<std::pair<int, dtype>>> tmp(rows);
    for (const auto& row : src.data)
      for (const auto& e : row.second) {
        const int r = order == row_major ? row.first : e.first;
        const int c = order == row_major ? e.first : row.first;
        tmp[r].push_back({c, e.second});
      }
    ptr.assign(rows + 1, 0);
    idx.clear();
    val.clear();
    for (int r = 0; r < rows; ++r) {
      std::sort(tmp[r].begin(), tmp[r].end(),
                [](const std::pair<int, dtype>& a, const std::pair<int, dtype>& b) { return a.first < b.first; });
      for (auto& p : tmp[r]) {
        idx.push_back(p.first);
        val.push_back(p.second);
      }
      ptr[r + 1] = static_cast<int>(idx.size());
    }
  }
};

template <typename dtype, order_t order>
struct gemm_impl<dynamic, dtype, dense_matrix, order, loops> {
  static int ix(int r, int c, int n) { return order == row_major ? r * n + c : c * n + r; }
  // C = alpha*A*B + beta*C with A the stored matrix.
  static void func(loops*, dtype alpha, dense_matrix<dynamic, dtype, order, loops>& A, dtype* B, dtype beta,
                   dtype* C, int n) {
    std::vector<dtype> out(static_cast<size_t>(n) * n);
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) {
        dtype s = zero<dtype>();
        for (int k = 0; k < n; ++k) s += A.at(r, k) * B[ix(k, c, n)];
        out[ix(r, c, n)] = beta == zero<dtype>() ? alpha * s : alpha * s + beta * C[ix(r, c, n)];
      }
    for (int i = 0; i < n * n; ++i) C[i] = out[i];
  }
  // C = alpha*A*B + beta*C with B the stored matrix.
  static void func(loops*, dtype alpha, dtype* A, dense_matrix<dynamic, dtype, order, loops>& B, dtype beta,
                   dtype* C, int n) {
    std::vector<dtype> out(static_cast<size_t>(n) * n);
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) {
        dtype s = zero<dtype>();
        for (int k = 0; k < n; ++k) s += A[ix(r, k, n)] * B.at(k, c);
        out[ix(r, c, n)] = beta == zero<dtype>() ? alpha * s : alpha * s + beta * C[ix(r, c, n)];
      }
    for (int i = 0; i < n * n; ++i) C[i] = out[i];
  }
};

template <typename dtype, order_t order>
struct gemv_impl<dynamic, dtype, dense_matrix, order, loops> {
  static void func(loops*, dtype alpha, dense_matrix<dynamic, dtype, order, loops>& A, dtype* x, dtype beta,
                   dtype* y, int n) {
    std::vector<dtype> out(n);
    for (int r = 0; r < n; ++r) {
      dtype s = zero<dtype>();
      for (int c = 0; c < n; ++c) s += A.at(r, c) * x[c];
      out[r] = beta == zero<dtype>() ? alpha * s : alpha * s + beta * y[r];
    }
    for (int r = 0; r < n; ++r) y[r] = out[r];
  }
};

template <typename dtype, order_t order>
struct gemv_impl<dynamic, dtype, sparse_matrix, order, loops> {
  static void func(loops*, dtype alpha, sparse_matrix<dynamic, dtype, order, loops>& A, dtype* x, dtype beta,
                   dtype* y, int n) {
    for (int r = 0; r < A.rows; ++r) {
      dtype s = zero<dtype>();
      for (int p = A.ptr[r]; p < A.ptr[r + 1]; ++p) s += A.val[p] * x[A.idx[p]];
      y[r] = beta == zero<dtype>() ? alpha * s : alpha * s + beta * y[r];
    }
  }
};

}  // namespace libheom

#endif
