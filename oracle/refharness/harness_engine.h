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
//   eig / utf / utb (Redfield)    linalg_engine.h:405-483
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
  dtype& ref(int r, int c) { return order == row_major ? data[r * cols + c] : data[c * rows + r]; }
  void set_shape(int r, int c) {
    rows = r;
    cols = c;
    data.assign(static_cast<size_t>(r) * c, zero<dtype>());
  }
  // dense -> LIL (dense_matrix_eigen.h.j2:82-100): logical entries, zeros skipped
  void dump(lil_matrix<dynamic, dtype, order, nil>& dest) {
    dest.set_shape(rows, cols);
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c)
        if (at(r, c) != zero<dtype>()) dest.push(r, c, at(r, c));
  }
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

// eig (linalg_engine.h:405-423), Hermitian A: w ascending, v[i*n + k] = component
// i of eigenvector k (unitary).  Cyclic complex Jacobi: each rotation first
// turns a_pq real with a phase, then applies the real symmetric 2x2 rotation.
template <typename dtype, order_t order>
struct eig_impl<dynamic, dtype, dense_matrix, order, loops> {
  static void func(loops*, dense_matrix<dynamic, dtype, order, loops>& A, real_t<dtype>* w, dtype* v, int n) {
    using R = real_t<dtype>;
    std::vector<dtype> a(static_cast<size_t>(n) * n), u(static_cast<size_t>(n) * n, zero<dtype>());
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) a[r * n + c] = A.at(r, c);
    for (int i = 0; i < n; ++i) u[i * n + i] = one<dtype>();
    R norm = 0;
    for (const dtype& x : a) norm += std::norm(x);
    for (int sweep = 0; sweep < 100; ++sweep) {
      R off = 0;
      for (int p = 0; p < n; ++p)
        for (int q = p + 1; q < n; ++q) off += std::norm(a[p * n + q]);
      if (off <= 1e-32 * norm) break;
      for (int p = 0; p < n; ++p)
        for (int q = p + 1; q < n; ++q) {
          const dtype g = a[p * n + q];
          const R ag = std::abs(g);
          if (ag == 0) continue;
          const dtype ph = g / ag;  // e^{i phi}
          const R app = std::real(a[p * n + p]), aqq = std::real(a[q * n + q]);
          const R th = (aqq - app) / (2 * ag);
          const R t = (th >= 0 ? 1 : -1) / (std::abs(th) + std::sqrt(th * th + 1));
          const R c = 1 / std::sqrt(t * t + 1), s = t * c;
          // G on columns p, q: G_pp = c, G_pq = s, G_qp = -s e^{-i phi}, G_qq = c e^{-i phi}
          const dtype em = std::conj(ph);
          for (int k = 0; k < n; ++k) {  // A <- A G, U <- U G
            for (dtype* m : {a.data(), u.data()}) {
              const dtype xp = m[k * n + p], xq = m[k * n + q];
              m[k * n + p] = c * xp - s * em * xq;
              m[k * n + q] = s * xp + c * em * xq;
            }
          }
          for (int k = 0; k < n; ++k) {  // A <- G^dagger A
            const dtype xp = a[p * n + k], xq = a[q * n + k];
            a[p * n + k] = c * xp - s * ph * xq;
            a[q * n + k] = s * xp + c * ph * xq;
          }
        }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return std::real(a[x * n + x]) < std::real(a[y * n + y]); });
    for (int k = 0; k < n; ++k) {
      w[k] = std::real(a[idx[k] * n + idx[k]]);
      for (int i = 0; i < n; ++i) v[i * n + k] = u[i * n + idx[k]];
    }
  }
};

// utf (linalg_engine.h:434-453): A_v = v^dagger A v, row-major n x n.
template <typename dtype, order_t order>
struct utf_impl<dynamic, dtype, dense_matrix, order, loops> {
  static void func(loops*, dense_matrix<dynamic, dtype, order, loops>& A, dtype* v, dtype* A_v, int n) {
    std::vector<dtype> t(static_cast<size_t>(n) * n, zero<dtype>());
    for (int a = 0; a < n; ++a)
      for (int j = 0; j < n; ++j) {
        dtype acc = zero<dtype>();
        for (int b = 0; b < n; ++b) acc += A.at(a, b) * v[b * n + j];
        t[a * n + j] = acc;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        dtype acc = zero<dtype>();
        for (int a = 0; a < n; ++a) acc += std::conj(v[a * n + i]) * t[a * n + j];
        A_v[i * n + j] = acc;
      }
  }
};

// utb (linalg_engine.h:464-483): A = v A_v v^dagger.
template <typename dtype, order_t order>
struct utb_impl<dynamic, dtype, dense_matrix, order, loops> {
  static void func(loops*, dtype* A_v, dtype* v, dense_matrix<dynamic, dtype, order, loops>& A, int n) {
    std::vector<dtype> t(static_cast<size_t>(n) * n, zero<dtype>());
    for (int a = 0; a < n; ++a)
      for (int j = 0; j < n; ++j) {
        dtype acc = zero<dtype>();
        for (int i = 0; i < n; ++i) acc += v[a * n + i] * A_v[i * n + j];
        t[a * n + j] = acc;
      }
    A.set_shape(n, n);
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        dtype acc = zero<dtype>();
        for (int j = 0; j < n; ++j) acc += t[a * n + j] * std::conj(v[b * n + j]);
        A.ref(a, b) = acc;
      }
  }
};

}  // namespace libheom

#endif
