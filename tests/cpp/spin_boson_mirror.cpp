// Drives the engine through the C++ mirror (include/heomgb.hpp) exactly the
// way a libheom caller drives heom_hilb + rk4 + qme_solver, and writes the
// final state (complex128, row-major) to argv[1].
#include <cmath>
#include <cstdio>
#include <vector>

#include "heomgb.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  using heomgb::complex128;
  const double lam = 0.5, gc = 1.0, beta = 1.0, pi = 3.14159265358979323846;
  const int depth = 6, n_mats = 2, K = 1 + n_mats;
  std::vector<complex128> nu, c;
  nu.push_back(gc);
  c.push_back(lam * gc * complex128(1.0 / std::tan(beta * gc / 2.0), -1.0));
  for (int m = 1; m <= n_mats; ++m) {
    const double v = 2.0 * pi * m / beta;
    nu.push_back(v);
    c.push_back(4.0 * lam * gc * v / (beta * (v * v - gc * gc)));
  }
  heomgb::heom_hilb qme(depth, 1, 1);
  qme.n_level = 2;
  qme.n_level_2 = 4;
  qme.H.set_shape(2, 2);
  qme.H.data[0][1] = 1.0;
  qme.H.data[1][0] = 1.0;
  qme.alloc_noises(1);
  qme.V[0].set_shape(2, 2);
  qme.V[0].data[0][0] = 1.0;
  qme.V[0].data[1][1] = -1.0;
  qme.len_gamma[0] = K;
  qme.gamma[0].set_shape(K, K);
  qme.S[0].set_shape(K, K);
  qme.A[0].set_shape(K, K);
  qme.phi_0[0].assign(K, 1.0);
  qme.sigma[0].assign(K, 1.0);
  for (int k = 0; k < K; ++k) {
    qme.gamma[0].data[k][k] = nu[k];
    qme.S[0].data[k][k] = c[k].real();
    if (c[k].imag() != 0.0) qme.A[0].data[k][k] = c[k].imag();
  }
  qme.s_delta[0] = 0.0;
  qme.set_param();
  heomgb::rk4 solver;
  heomgb::qme_solver qs(nullptr, &qme, &solver);
  std::vector<complex128> rho(qme.main_size());
  rho[0] = 1.0;
  const double t_list[2] = {0.0, 0.5};
  int calls = 0;
  heomgb::kwargs_t kw;
  kw["dt"] = 0.005;
  qs.solve(rho.data(), t_list, 2, [&](double) { ++calls; }, kw);
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 3;
  std::fwrite(rho.data(), sizeof(complex128), rho.size(), f);
  std::fclose(f);
  std::printf("n_hrchy=%d callbacks=%d\n", qme.get_n_hrchy(), calls);
  return calls == 2 ? 0 : 4;
}
