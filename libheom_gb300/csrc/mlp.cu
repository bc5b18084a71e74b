// Learned terminator: a small MLP that predicts the truncated tier N+1 of the
// hierarchy from tier-N ADOs, trained and evaluated with the kernels below.
//
// Network: x (d_in) -> Linear(h) -> GELU -> Linear(h) -> GELU -> Linear(d_out).
// Weights are kept as FP32 masters (Adam) and BF16 copies.  Every product of
// the forward pass, the backward pass (data and weight gradients) and the
// inference is a BF16 tensor-core GEMM (tcgemm.cu: tcgen05.mma, BF16 operands,
// FP32 accumulation in tensor memory); bias, GELU and the GELU derivative run
// in the GEMM's epilogue.
//
// Terminator use: for a tier-N ADO rho_n and mode k, the input is
// [Re rho_n / s, Im rho_n / s, onehot(k), Re A / s, Im A / s] with
// s = max_e |rho_n[e]| (the hierarchy is linear, so the map is learned on the
// unit-scale problem) and A the adiabatic estimate of rho_{n+1_k}; the
// output is an elementwise complex gain C with rho_{n+1_k} ~ C rho_n / sigma_k,
// constrained so that the closure term damps (k_term_scatter).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "heomgb.h"
#include "heomgb_impl.cuh"

namespace heomgb {
void set_error_message(const std::string& msg);
}

using namespace heomgb;

namespace {

// db[o] = sum_b dZ[b, o] (bias gradient; the weight gradients are tensor-core GEMMs)
__global__ void k_bias_grad(const float* __restrict__ dZ, float* __restrict__ db, int B, int dout) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= dout) return;
  float acc = 0.f;
  for (int b = 0; b < B; ++b) acc += dZ[static_cast<size_t>(b) * dout + o];
  db[o] = acc;
}

// Mean-squared error and its gradient d/dY of mean((Y-T)^2); per-CTA partial
// losses are summed on the host.
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY,
                      float* __restrict__ part, long long n) {
  __shared__ float red[256];
  float s = 0.f;
  const float scale = 2.0f / static_cast<float>(n);
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float d = Y[i] - T[i];
    s += d * d;
    dY[i] = scale * d;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Closure ("gain") loss of the terminator head.  Per row the network gives
// (Re C_e, z_e) for the n2 elements; C_e = Re C_e - i sg_e softplus(z_e) with
// sg_e = sign(v_a - v_b) of the mode's bath (0 where the +1 term vanishes).
// Target row: [Re t, Im t, Re r, Im r, sg] (5 n2 floats), t = rho_{n+1_k}/s,
// r = rho_n/(s sigma_k).  Loss = mean over rows of
//   sum_e m_e |C_e r_e - t_e|^2 / (sum_e m_e (|t_e|^2 + 1e-2 |r_e|^2) + 1e-6),
// m_e = |sg_e|: each row's error relative to its own size.
__device__ __forceinline__ float softplus_f(float z) { return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z))); }
__device__ __forceinline__ float sigmoid_f(float z) { return 1.f / (1.f + expf(-z)); }

__global__ void k_gain_loss(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY,
                            float* __restrict__ part, int B, int n2) {
  __shared__ float red[256];
  float acc = 0.f;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    const float* y = Y + static_cast<size_t>(b) * 2 * n2;
    const float* t = T + static_cast<size_t>(b) * 5 * n2;
    float* dy = dY + static_cast<size_t>(b) * 2 * n2;
    float den = 1e-6f;
    for (int e = 0; e < n2; ++e) {
      const float m = fabsf(t[4 * n2 + e]);
      den += m * (t[e] * t[e] + t[n2 + e] * t[n2 + e] + 1e-2f * (t[2 * n2 + e] * t[2 * n2 + e] +
                                                                 t[3 * n2 + e] * t[3 * n2 + e]));
    }
    const float w = 2.f / (static_cast<float>(B) * den);
    float num = 0.f;
    for (int e = 0; e < n2; ++e) {
      const float sg = t[4 * n2 + e], m = fabsf(sg);
      const float cr = y[e], ci = -sg * softplus_f(y[n2 + e]);
      const float rr = t[2 * n2 + e], ri = t[3 * n2 + e];
      const float dr = cr * rr - ci * ri - t[e], di = cr * ri + ci * rr - t[n2 + e];
      num += m * (dr * dr + di * di);
      // conj(d) r = (dr rr + di ri) + i (dr ri - di rr)
      const float re = dr * rr + di * ri, im = dr * ri - di * rr;
      dy[e] = w * m * re;
      dy[n2 + e] = w * m * sg * sigmoid_f(y[n2 + e]) * im;
    }
    acc += num / den;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Adam on the FP32 masters, then refresh the BF16 copies.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ wb, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16(wi);
  }
}

__global__ void k_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    wb[i] = __float2bfloat16(w[i]);
}

void ckm(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

int grid_for(long long n) { return static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024))); }

}  // namespace

struct heomgb_mlp {
  int din = 0, h = 0, dout = 0;
  long long n_params = 0;
  // offsets into the packed parameter vector: W1, b1, W2, b2, W3, b3
  long long off[6] = {0, 0, 0, 0, 0, 0};
  float* w = nullptr;           // FP32 masters
  __nv_bfloat16* wb = nullptr;  // BF16 copies
  float* g = nullptr;           // gradients
  float* m = nullptr;           // Adam moments
  float* v = nullptr;
  long long step = 0;
  int loss_kind = 0;            // 0: mean squared error; 1: terminator closure loss (k_gain_loss)
  int loss_n2 = 0;              // elements per ADO for loss_kind 1 (d_out = 2 loss_n2)
  int cap = 0;                  // batch capacity of the activation buffers
  float *a1 = nullptr, *p1 = nullptr, *a2 = nullptr, *p2 = nullptr, *y = nullptr, *d = nullptr, *d2 = nullptr;
  float* part = nullptr;
  int* err = nullptr;           // set by a tensor-core GEMM whose wait ran out
  cudaStream_t s = nullptr;
  void free_acts() {
    for (float* p : {a1, p1, a2, p2, y, d, d2, part}) cudaFree(p);
    a1 = p1 = a2 = p2 = y = d = d2 = part = nullptr;
    cap = 0;
  }
  void ensure(int B) {
    if (B <= cap) return;
    free_acts();
    const size_t hb = sizeof(float) * static_cast<size_t>(B) * h;
    ckm(cudaMalloc(&a1, hb), "mlp alloc");
    ckm(cudaMalloc(&p1, hb), "mlp alloc");
    ckm(cudaMalloc(&a2, hb), "mlp alloc");
    ckm(cudaMalloc(&p2, hb), "mlp alloc");
    ckm(cudaMalloc(&y, sizeof(float) * static_cast<size_t>(B) * dout), "mlp alloc");
    ckm(cudaMalloc(&d, hb + sizeof(float) * static_cast<size_t>(B) * (dout + din)), "mlp alloc");
    ckm(cudaMalloc(&d2, hb), "mlp alloc");
    ckm(cudaMalloc(&part, sizeof(float) * 1024), "mlp alloc");
    cap = B;
  }
  ~heomgb_mlp() {
    free_acts();
    for (void* p : {static_cast<void*>(w), static_cast<void*>(wb), static_cast<void*>(g), static_cast<void*>(m),
                    static_cast<void*>(v), static_cast<void*>(err)})
      cudaFree(p);
    if (s) cudaStreamDestroy(s);
  }
};

namespace {

template <class F>
heomgb_status mguard(F&& f) {
  try {
    f();
    return HEOMGB_OK;
  } catch (const std::invalid_argument& e) {
    set_error_message(e.what());
    return HEOMGB_ERR_INVALID_ARGUMENT;
  } catch (const std::exception& e) {
    set_error_message(e.what());
    return HEOMGB_ERR_CUDA;
  }
}

GemmOperand op_f32(const float* p, long long sm, long long sk) { return GemmOperand{p, 0, sm, sk}; }
GemmOperand op_bf16(const __nv_bfloat16* p, long long sm, long long sk) { return GemmOperand{p, 1, sm, sk}; }

void gemm(heomgb_mlp* M, GemmOperand a, GemmOperand b, float* c, long long ldc, const float* bias, float* pre,
          int m, int n, int k, int epi, cudaStream_t s) {
  GemmArgs g{};
  g.a = a;
  g.b = b;
  g.c = c;
  g.ldc = ldc;
  g.bias = bias;
  g.pre = pre;
  g.M = m;
  g.N = n;
  g.K = k;
  g.epi = epi;
  g.err = M->err;
  ckm(launch_gemm_bf16(g, s), "tensor-core gemm");
}

// Y[b][o] = act(sum_i X[b][i] W[o][i] + bias[o]) for layer 0..2
void linear_fwd(heomgb_mlp* M, const float* X, int layer, float* Y, float* PRE, int B, bool act, cudaStream_t s) {
  const int din = layer == 0 ? M->din : M->h, dout = layer == 2 ? M->dout : M->h;
  gemm(M, op_f32(X, din, 1), op_bf16(M->wb + M->off[2 * layer], din, 1), Y, dout, M->w + M->off[2 * layer + 1],
       PRE, B, dout, din, act ? GEMM_GELU : GEMM_STORE, s);
}

void check_err(heomgb_mlp* M) {
  int e = 0;
  ckm(cudaMemcpyAsync(&e, M->err, sizeof(int), cudaMemcpyDeviceToHost, M->s), "mlp status");
  ckm(cudaStreamSynchronize(M->s), "mlp sync");
  if (e) {
    ckm(cudaMemsetAsync(M->err, 0, sizeof(int), M->s), "mlp status reset");
    throw std::runtime_error("tensor-core GEMM did not complete (a bounded wait ran out)");
  }
}

void forward(heomgb_mlp* M, const float* X, float* out, int B) {
  M->ensure(B);
  linear_fwd(M, X, 0, M->a1, M->p1, B, true, M->s);
  linear_fwd(M, M->a1, 1, M->a2, M->p2, B, true, M->s);
  linear_fwd(M, M->a2, 2, out, nullptr, B, false, M->s);
}

// Weight and bias gradients of layer `layer` from dZ (B x dout) and its input X (B x din):
// dW[o][i] = sum_b dZ[b][o] X[b][i], db[o] = sum_b dZ[b][o]
void weight_grad(heomgb_mlp* M, const float* dZ, const float* X, int layer, int B) {
  const int din = layer == 0 ? M->din : M->h, dout = layer == 2 ? M->dout : M->h;
  gemm(M, op_f32(dZ, 1, dout), op_f32(X, 1, din), M->g + M->off[2 * layer], din, nullptr, nullptr, dout, din, B,
       GEMM_STORE, M->s);
  k_bias_grad<<<(dout + 127) / 128, 128, 0, M->s>>>(dZ, M->g + M->off[2 * layer + 1], B, dout);
  ++g_launches;
}

// dH[b][i] = (sum_o dZ[b][o] W[o][i]) gelu'(PRE[b][i]) for the hidden layer below `layer`
void data_grad(heomgb_mlp* M, const float* dZ, int layer, const float* PRE, float* dH, int B) {
  const int din = layer == 0 ? M->din : M->h, dout = layer == 2 ? M->dout : M->h;
  gemm(M, op_f32(dZ, dout, 1), op_bf16(M->wb + M->off[2 * layer], 1, din), dH, din, nullptr,
       const_cast<float*>(PRE), B, din, dout, GEMM_GELU_GRAD, M->s);
}

// Forward + backward: fills M->g with the gradient of the loss; returns the loss.
float backward(heomgb_mlp* M, const float* X, const float* T, int B) {
  M->ensure(B);
  forward(M, X, M->y, B);
  const long long ny = static_cast<long long>(B) * M->dout;
  const int gm = grid_for(ny);
  float* dy = M->d;                                   // B*dout
  const int gl = M->loss_kind == 1 ? grid_for(B) : gm;
  if (M->loss_kind == 1)
    k_gain_loss<<<gl, 256, 0, M->s>>>(M->y, T, dy, M->part, B, M->loss_n2);
  else
    k_mse<<<gm, 256, 0, M->s>>>(M->y, T, dy, M->part, ny);
  ++g_launches;
  float* dh1 = M->d + ny;  // B*h scratch after dy
  weight_grad(M, dy, M->a2, 2, B);
  data_grad(M, dy, 2, M->p2, M->d2, B);      // d(layer-2 pre-activation)
  weight_grad(M, M->d2, M->a1, 1, B);
  data_grad(M, M->d2, 1, M->p1, dh1, B);     // d(layer-1 pre-activation)
  weight_grad(M, dh1, X, 0, B);
  ckm(cudaGetLastError(), "mlp backward");
  std::vector<float> part(gl);
  ckm(cudaMemcpyAsync(part.data(), M->part, sizeof(float) * gl, cudaMemcpyDeviceToHost, M->s), "loss copy");
  check_err(M);
  double loss = 0;
  for (float p : part) loss += p;
  return static_cast<float>(loss / static_cast<double>(M->loss_kind == 1 ? B : ny));
}

}  // namespace

// ------------------------------------------------------------------ terminator inference
// Inputs of the rows (tier-N ADO j, mode k), d_in = 4 n2 + K:
//   [Re rho/s, Im rho/s (2 n2), onehot(k) (K), Re A/s, Im A/s (2 n2)]
// with s = max_e |rho_l[e]| and A the adiabatic estimate of rho_{n+1_k}
// (the tier-(N+1) equation with its own time derivative and the commutator
// with H dropped; V_u diagonal):
//   A[ab] = (n_k+1) (-i s_k (v_a - v_b) + a_k (v_a + v_b)) rho_ab / (ngamma_l + gamma_kk).
// CTA j stages rho_l (l = first+j), reduces s, and writes the K rows.
template <typename TB>
__global__ void k_term_pack(const TermInput in, const TermModel tm, int first, int n_tier, float* __restrict__ X,
                            float* __restrict__ scale) {
  __shared__ float red[128];
  const int j = blockIdx.x;
  if (j >= n_tier) return;
  const int n = tm.n, n2 = n * n, K = tm.K;
  const int cur = in.ctl ? in.ctl->cur : 0;
  const void* ysel = in.y_sel == 1 ? in.yb[cur] : (in.y_sel == 2 ? in.yb[1 - cur] : in.y_fixed);
  const int l = first + j;
  const TB* yl = static_cast<const TB*>(ysel) + static_cast<size_t>(l) * n2;
  float mx = 0.f;
  for (int e = threadIdx.x; e < n2; e += blockDim.x) {
    const float re = static_cast<float>(yl[e].x), im = static_cast<float>(yl[e].y);
    mx = fmaxf(mx, re * re + im * im);
  }
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  const float s = sqrtf(red[0]) + 1e-30f;
  const float inv = 1.0f / s;
  if (threadIdx.x == 0) scale[j] = s;
  const int din = 4 * n2 + K;
  const double2 gl = tm.ngd[l];
  for (int k = 0; k < K; ++k) {
    float* row = X + (static_cast<size_t>(j) * K + k) * din;
    int u = 0;
    while (u + 1 < tm.U && tm.bath_ptr[u + 1] <= k) ++u;
    const double2 sk = tm.s[k], ak = tm.a[k], gk = tm.gdiag[k];
    const double nk1 = static_cast<double>(tm.nidx[static_cast<size_t>(l) * K + k]) + 1.0;
    // 1 / (ngamma_l + gamma_kk)
    const double dr = gl.x + gk.x, di = gl.y + gk.y, dd = dr * dr + di * di;
    const double ir = dd > 0.0 ? dr / dd : 0.0, ii = dd > 0.0 ? -di / dd : 0.0;
    for (int f = threadIdx.x; f < din; f += blockDim.x) {
      float v;
      if (f < 2 * n2) {
        const int e = f < n2 ? f : f - n2;
        v = static_cast<float>(f < n2 ? yl[e].x : yl[e].y) * inv;
      } else if (f < 2 * n2 + K) {
        v = (f - 2 * n2 == k) ? 1.f : 0.f;
      } else {
        const int g2 = f - 2 * n2 - K;
        const int e = g2 < n2 ? g2 : g2 - n2;
        const int a = e / n, b = e - a * n;
        const double2 va = tm.V[static_cast<size_t>(u) * n2 + a * n + a], vb = tm.V[static_cast<size_t>(u) * n2 + b * n + b];
        // c = -i s_k (va - vb) + a_k (va + vb)
        const double mr = va.x - vb.x, mi = va.y - vb.y, pr = va.x + vb.x, pi = va.y + vb.y;
        const double t1r = sk.x * mr - sk.y * mi, t1i = sk.x * mi + sk.y * mr;  // s_k (va - vb)
        const double cr = t1i + (ak.x * pr - ak.y * pi), ci = -t1r + (ak.x * pi + ak.y * pr);
        const double yr = static_cast<double>(yl[e].x), yi = static_cast<double>(yl[e].y);
        const double zr = cr * yr - ci * yi, zi = cr * yi + ci * yr;     // c * rho_ab
        const double wr = zr * ir - zi * ii, wi = zr * ii + zi * ir;     // / (ngamma + gamma_k)
        v = static_cast<float>((g2 < n2 ? wr : wi) * nk1) * inv;
      }
      row[f] = v;
    }
  }
}

// Gain head: row (j, k) gives C_e = Y[e] - i sg_e softplus(Y[n2+e]) with
// sg_e = sign(Re(v_a - v_b)) for the bath of mode k, and the prediction
//   P[(j*K+k)*n2 + e] = C_e rho_l[e] / sigma_k   (rho_l[e] = s_j X[row][e] + i s_j X[row][n2+e]).
// Its +1 term in the right-hand side, i (v_a - v_b) sigma_k P_e, is then
// i (v_a - v_b) C_e rho_l[e]: a rate whose real part is -|v_a - v_b| softplus <= 0,
// so the closure only damps (or shifts the frequency of) the tier-N ADOs.
__global__ void k_term_scatter(const float* __restrict__ Y, const float* __restrict__ X,
                               const float* __restrict__ scale, const TermModel tm, int n_tier, int din,
                               float2* __restrict__ P) {
  const int n = tm.n, n2 = n * n, K = tm.K;
  const long long total = static_cast<long long>(n_tier) * K * n2;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long r = i / n2;
    const int e = static_cast<int>(i - r * n2);
    const int k = static_cast<int>(r % K);
    int u = 0;
    while (u + 1 < tm.U && tm.bath_ptr[u + 1] <= k) ++u;
    const int a = e / n, b = e - a * n;
    const double dv = tm.V[static_cast<size_t>(u) * n2 + a * n + a].x - tm.V[static_cast<size_t>(u) * n2 + b * n + b].x;
    if (dv == 0.0) {
      P[i] = make_float2(0.f, 0.f);
      continue;
    }
    const float sg = dv > 0.0 ? 1.f : -1.f;
    const float s = scale[r / K];
    const float* yr = Y + r * (2 * n2);
    const float* xr = X + r * din;
    const float cr = yr[e], ci = -sg * softplus_f(yr[n2 + e]);
    const float rr = s * xr[e], ri = s * xr[n2 + e];
    // (C rho) / sigma_k
    const float pr = cr * rr - ci * ri, pi = cr * ri + ci * rr;
    const double2 sk = tm.sigma[k];
    const double dd = sk.x * sk.x + sk.y * sk.y;
    const float ir = static_cast<float>(sk.x / dd), ii = static_cast<float>(-sk.y / dd);
    P[i] = make_float2(pr * ir - pi * ii, pr * ii + pi * ir);
  }
}

namespace heomgb {

cudaError_t term_enqueue(heomgb_mlp* M, const TermBuffers& tb, const TermModel& tm, const TermInput& in,
                         bool y_float, cudaStream_t s) {
  if (tb.n_tier <= 0) return cudaSuccess;
  // one fused launch (features, three tensor-core layers, gain head) where the
  // sizes allow it; HEOMGB_TERM_FUSED=0 keeps the five-launch form below
  const char* fused_env = std::getenv("HEOMGB_TERM_FUSED");
  if (term_fused_ok(M->din, M->h, M->dout, tb.K) && !(fused_env && std::string(fused_env) == "0")) {
    TermMlpArgs a{};
    a.in = in;
    a.tm = tm;
    a.first = tb.first;
    a.n_tier = tb.n_tier;
    a.apt = 128 / tb.K;
    a.din = M->din;
    a.h = M->h;
    a.dout = M->dout;
    a.W1 = M->wb + M->off[0];
    a.W2 = M->wb + M->off[2];
    a.W3 = M->wb + M->off[4];
    a.b1 = M->w + M->off[1];
    a.b2 = M->w + M->off[3];
    a.b3 = M->w + M->off[5];
    a.P = tb.P;
    a.err = M->err;
    return launch_term_fused(a, y_float, s);
  }
  const int R = tb.n_tier * tb.K;
  if (y_float)
    k_term_pack<float2><<<tb.n_tier, 128, 0, s>>>(in, tm, tb.first, tb.n_tier, tb.X, tb.scale);
  else
    k_term_pack<double2><<<tb.n_tier, 128, 0, s>>>(in, tm, tb.first, tb.n_tier, tb.X, tb.scale);
  const int din = M->din, h = M->h, dout = M->dout;
  gemm(M, op_f32(tb.X, din, 1), op_bf16(M->wb + M->off[0], din, 1), tb.A1, h, M->w + M->off[1], nullptr, R, h, din,
       GEMM_GELU, s);
  gemm(M, op_f32(tb.A1, h, 1), op_bf16(M->wb + M->off[2], h, 1), tb.A2, h, M->w + M->off[3], nullptr, R, h, h,
       GEMM_GELU, s);
  gemm(M, op_f32(tb.A2, h, 1), op_bf16(M->wb + M->off[4], h, 1), tb.Y, dout, M->w + M->off[5], nullptr, R, dout, h,
       GEMM_STORE, s);
  const long long tot = static_cast<long long>(R) * tb.n2;
  k_term_scatter<<<grid_for(tot), 256, 0, s>>>(tb.Y, tb.X, tb.scale, tm, tb.n_tier, din, tb.P);
  g_launches += 2;  // the pack and scatter kernels; the GEMMs count their own
  return cudaGetLastError();
}

bool mlp_take_error(heomgb_mlp* M, cudaStream_t s) {
  int e = 0;
  ckm(cudaMemcpyAsync(&e, M->err, sizeof(int), cudaMemcpyDeviceToHost, s), "mlp status");
  ckm(cudaStreamSynchronize(s), "mlp sync");
  if (e) ckm(cudaMemsetAsync(M->err, 0, sizeof(int), s), "mlp status reset");
  return e != 0;
}

void mlp_dims(const heomgb_mlp* M, int* din, int* h, int* dout) {
  *din = M->din;
  *h = M->h;
  *dout = M->dout;
}

}  // namespace heomgb

extern "C" {

heomgb_status heomgb_mlp_create(int d_in, int d_hidden, int d_out, unsigned long long seed, heomgb_mlp** out) {
  return mguard([&] {
    if (!out || d_in < 1 || d_hidden < 1 || d_out < 1) throw std::invalid_argument("bad MLP sizes");
    auto M = std::make_unique<heomgb_mlp>();
    M->din = d_in;
    M->h = d_hidden;
    M->dout = d_out;
    const long long sz[6] = {static_cast<long long>(d_hidden) * d_in, d_hidden,
                             static_cast<long long>(d_hidden) * d_hidden, d_hidden,
                             static_cast<long long>(d_out) * d_hidden, d_out};
    long long o = 0;
    for (int i = 0; i < 6; ++i) {
      M->off[i] = o;
      o += sz[i];
    }
    M->n_params = o;
    // He-uniform initialisation from a 64-bit LCG (deterministic per seed); zero biases.
    std::vector<float> w(o, 0.f);
    unsigned long long st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
      st = st * 6364136223846793005ULL + 1442695040888963407ULL;
      return static_cast<float>((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    const int fan_in[3] = {d_in, d_hidden, d_hidden};
    for (int l = 0; l < 3; ++l) {
      const float a = std::sqrt(6.0f / static_cast<float>(fan_in[l])) * (l == 2 ? 0.5f : 1.0f);
      for (long long i = 0; i < sz[2 * l]; ++i) w[M->off[2 * l] + i] = a * uni();
    }
    ckm(cudaStreamCreateWithFlags(&M->s, cudaStreamNonBlocking), "stream");
    const size_t fb = sizeof(float) * o;
    ckm(cudaMalloc(&M->w, fb), "mlp alloc");
    ckm(cudaMalloc(&M->g, fb), "mlp alloc");
    ckm(cudaMalloc(&M->m, fb), "mlp alloc");
    ckm(cudaMalloc(&M->v, fb), "mlp alloc");
    ckm(cudaMalloc(&M->wb, sizeof(__nv_bfloat16) * o), "mlp alloc");
    ckm(cudaMalloc(&M->err, sizeof(int)), "mlp alloc");
    ckm(cudaMemsetAsync(M->err, 0, sizeof(int), M->s), "memset");
    ckm(cudaMemcpyAsync(M->w, w.data(), fb, cudaMemcpyHostToDevice, M->s), "mlp init");
    ckm(cudaMemsetAsync(M->g, 0, fb, M->s), "memset");
    ckm(cudaMemsetAsync(M->m, 0, fb, M->s), "memset");
    ckm(cudaMemsetAsync(M->v, 0, fb, M->s), "memset");
    k_to_bf16<<<grid_for(o), 256, 0, M->s>>>(M->w, M->wb, o);
    ++g_launches;
    ckm(cudaStreamSynchronize(M->s), "mlp init sync");
    *out = M.release();
  });
}

heomgb_status heomgb_mlp_destroy(heomgb_mlp* M) {
  if (M) {
    cudaStreamSynchronize(M->s);
    delete M;
  }
  return HEOMGB_OK;
}

heomgb_status heomgb_mlp_sizes(const heomgb_mlp* M, int* d_in, int* d_hidden, int* d_out, long long* n_params) {
  return mguard([&] {
    if (!M) throw std::invalid_argument("null mlp");
    if (d_in) *d_in = M->din;
    if (d_hidden) *d_hidden = M->h;
    if (d_out) *d_out = M->dout;
    if (n_params) *n_params = M->n_params;
  });
}

heomgb_status heomgb_mlp_get_params(heomgb_mlp* M, float* params) {
  return mguard([&] {
    if (!M || !params) throw std::invalid_argument("null argument");
    ckm(cudaMemcpyAsync(params, M->w, sizeof(float) * M->n_params, cudaMemcpyDeviceToHost, M->s), "copy");
    ckm(cudaStreamSynchronize(M->s), "sync");
  });
}

heomgb_status heomgb_mlp_set_params(heomgb_mlp* M, const float* params) {
  return mguard([&] {
    if (!M || !params) throw std::invalid_argument("null argument");
    ckm(cudaMemcpyAsync(M->w, params, sizeof(float) * M->n_params, cudaMemcpyHostToDevice, M->s), "copy");
    k_to_bf16<<<grid_for(M->n_params), 256, 0, M->s>>>(M->w, M->wb, M->n_params);
    ++g_launches;
    ckm(cudaStreamSynchronize(M->s), "sync");
  });
}

heomgb_status heomgb_mlp_set_loss(heomgb_mlp* M, int kind, int n2) {
  return mguard([&] {
    if (!M) throw std::invalid_argument("null mlp");
    if (kind != 0 && kind != 1) throw std::invalid_argument("unknown loss kind");
    if (kind == 1 && (n2 < 1 || M->dout != 2 * n2)) throw std::invalid_argument("closure loss needs d_out = 2 n2");
    M->loss_kind = kind;
    M->loss_n2 = kind == 1 ? n2 : 0;
  });
}

heomgb_status heomgb_mlp_forward(heomgb_mlp* M, const float* x_dev, float* y_dev, int batch) {
  return mguard([&] {
    if (!M || !x_dev || !y_dev || batch < 1) throw std::invalid_argument("bad argument");
    forward(M, x_dev, y_dev, batch);
    check_err(M);
  });
}

heomgb_status heomgb_mlp_gradients(heomgb_mlp* M, const float* x_dev, const float* t_dev, int batch,
                                   float* grad_host, float* loss) {
  return mguard([&] {
    if (!M || !x_dev || !t_dev || batch < 1) throw std::invalid_argument("bad argument");
    const float l = backward(M, x_dev, t_dev, batch);
    if (loss) *loss = l;
    if (grad_host) {
      ckm(cudaMemcpyAsync(grad_host, M->g, sizeof(float) * M->n_params, cudaMemcpyDeviceToHost, M->s), "copy");
      ckm(cudaStreamSynchronize(M->s), "sync");
    }
  });
}

heomgb_status heomgb_mlp_train_step(heomgb_mlp* M, const float* x_dev, const float* t_dev, int batch, float lr,
                                    float* loss) {
  return mguard([&] {
    if (!M || !x_dev || !t_dev || batch < 1) throw std::invalid_argument("bad argument");
    const float l = backward(M, x_dev, t_dev, batch);
    M->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, static_cast<float>(M->step));
    const float c2 = 1.f - std::pow(b2, static_cast<float>(M->step));
    k_adam<<<grid_for(M->n_params), 256, 0, M->s>>>(M->w, M->g, M->m, M->v, M->wb, M->n_params, lr, b1, b2, 1e-8f,
                                                    c1, c2);
    ++g_launches;
    ckm(cudaGetLastError(), "adam");
    ckm(cudaStreamSynchronize(M->s), "sync");
    if (loss) *loss = l;
  });
}

}  // extern "C"
