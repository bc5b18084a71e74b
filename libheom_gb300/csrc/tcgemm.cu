// BF16 GEMM on the 5th-generation tensor cores for the terminator's MLP:
// C[m][n] = sum_k A(m, k) B(n, k) with FP32 accumulation in tensor memory,
// followed by an epilogue (bias, GELU with its pre-activation kept, or the
// GELU derivative of a stored pre-activation).
//
// Operands are read from any strided layout (A(m, k) = a[m * a.sm + k * a.sk],
// FP32 or BF16), rounded to BF16 and staged by the CTA's threads in shared
// memory in the K-major layout without swizzle (8-row x 16-byte core
// matrices; K-adjacent core matrices 128 bytes apart, 8-row groups
// (BK / 8) * 128 bytes apart), so transposed operands (the backward pass)
// need no separate pass.  A CTA computes a 128 x BN tile (BN <= 256, a
// multiple of 16): K runs in chunks of 64 through two shared-memory stages;
// thread 0 issues four tcgen05.mma (kind::f16, BF16 inputs, K = 16 each) per
// chunk and commits them to the stage's mbarrier, and the CTA stages the next
// chunk meanwhile.  The accumulator (128 lanes x BN FP32 columns) is read
// back with tcgen05.ld by all eight warps (warp w: lanes 32 (w % 4) ..,
// columns of half w / 4).  Every mbarrier wait is bounded; one that runs out
// sets *err, drains the MMAs in flight (bounded again), frees the tensor
// memory and leaves.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "heomgb_impl.cuh"

namespace heomgb {

namespace {

constexpr int kBM = 128, kBK = 64;
constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t s_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ uint64_t g_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFF) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (static_cast<uint64_t>(1) << 46);
}

__device__ __forceinline__ void g_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void g_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(s_addr(mbar)));
}

// bounded wait for phase `parity` of an mbarrier; 1 when it completed
__device__ __forceinline__ uint32_t g_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t done = 0;
  for (int it = 0; it < (1 << 24) && !done; ++it) {
    asm volatile(
        "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.b32 %0, 1, 0, q;\n}\n"
        : "=r"(done)
        : "r"(s_addr(mbar)), "r"(parity));
  }
  return done;
}

__device__ __forceinline__ void g_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

__device__ __forceinline__ float load_as_float(const GemmOperand& o, long long off) {
  return o.bf16 ? __bfloat162float(static_cast<const __nv_bfloat16*>(o.p)[off]) : static_cast<const float*>(o.p)[off];
}

// Stages rows [r0, r0 + rows) x k [k0, k0 + kBK) of operand o (rows < lim_r,
// k < lim_k; zeros elsewhere) as BF16 into the core-matrix layout at dst.
// Unit u (8 consecutive k of one row, 16 bytes) is written by one thread; the
// eight rows of a core matrix are consecutive threads, so a warp's stores
// cover whole core matrices (no bank conflicts) and its loads of an operand
// whose rows are contiguous read whole 32-byte sectors.
__device__ __forceinline__ void stage_operand(const GemmOperand& o, int r0, int rows, int lim_r, int k0, int lim_k,
                                              unsigned char* dst) {
  const int units = rows * (kBK / 8);
  for (int u = threadIdx.x; u < units; u += blockDim.x) {
    const int r8 = u & 7, q = (u >> 3) & 7, g = u >> 6;
    const int r = g * 8 + r8, gr = r0 + r, gk = k0 + q * 8;
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float x0 = 0.f, x1 = 0.f;
      if (gr < lim_r) {
        const long long base = static_cast<long long>(gr) * o.sm;
        if (gk + 2 * j < lim_k) x0 = load_as_float(o, base + static_cast<long long>(gk + 2 * j) * o.sk);
        if (gk + 2 * j + 1 < lim_k) x1 = load_as_float(o, base + static_cast<long long>(gk + 2 * j + 1) * o.sk);
      }
      const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);  // x0 in the low half
      w[j] = *reinterpret_cast<const uint32_t*>(&h);
    }
    *reinterpret_cast<uint4*>(dst + g * (kBK / 8) * 128 + q * 128 + r8 * 16) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_f(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__global__ void __launch_bounds__(kThreads, 1) k_gemm_bf16(const GemmArgs g) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int BN = g.bn;
  const size_t a_bytes = static_cast<size_t>(kBM) * kBK * 2, b_bytes = static_cast<size_t>(BN) * kBK * 2;
  // stage b: A at smem_raw + b * (a_bytes + b_bytes), B after it (no arrays
  // indexed at run time: they would live in local memory)
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + 2 * (a_bytes + b_bytes));
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tslot)),
                 "r"(static_cast<uint32_t>(g.tmem_cols)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(mbar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(mbar + 1)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  // instruction descriptor: D FP32, A and B BF16, both K-major, N >> 3, M >> 4
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(BN >> 3) << 17) |
                         (static_cast<uint32_t>(kBM >> 4) << 24);
  const uint32_t sbo = (kBK / 8) * 128;
  const int nk = (g.K + kBK - 1) / kBK;
  uint32_t parity = 0u, issued = 0u;  // bit b: the stage's mbarrier phase, MMAs in flight
  int fail = 0;
  for (int c = 0; c < nk; ++c) {
    const int b = c & 1;
    unsigned char* sa = smem_raw + b * (a_bytes + b_bytes);
    unsigned char* sb = sa + a_bytes;
    if ((issued >> b) & 1u) {  // the MMAs that read this stage two chunks ago
      uint32_t done = 0;
      if (threadIdx.x == 0) done = g_wait(mbar + b, (parity >> b) & 1u);
      if (!__syncthreads_or(done)) {
        fail = 1;
        break;
      }
      parity ^= 1u << b;
      issued &= ~(1u << b);
    }
    stage_operand(g.a, m0, kBM, g.M, c * kBK, g.K, sa);
    stage_operand(g.b, n0, BN, g.N, c * kBK, g.K, sb);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    if (threadIdx.x == 0) {
      const uint32_t a0 = s_addr(sa), b0 = s_addr(sb);
#pragma unroll
      for (int s = 0; s < kBK / 16; ++s)
        g_mma(tmem, g_desc(a0 + s * 256, 128, sbo), g_desc(b0 + s * 256, 128, sbo), idesc, (c > 0 || s > 0) ? 1 : 0);
      g_commit(mbar + b);
    }
    issued |= 1u << b;
  }
  // the last chunks' MMAs (all earlier ones complete before them)
  if (!fail) {
    for (int b = 0; b < 2; ++b) {
      if (!((issued >> b) & 1u)) continue;
      uint32_t done = 0;
      if (threadIdx.x == 0) done = g_wait(mbar + b, (parity >> b) & 1u);
      if (!__syncthreads_or(done)) {
        fail = 1;
        break;
      }
      parity ^= 1u << b;
      issued &= ~(1u << b);
    }
  }
  if (fail) {  // drain what is still in flight (bounded) before freeing the tensor memory
    if (threadIdx.x == 0) {
      for (int b = 0; b < 2; ++b)
        if ((issued >> b) & 1u) g_wait(mbar + b, (parity >> b) & 1u);
      atomicExch(g.err, 1);
    }
    __syncthreads();
  } else {
    fence_after();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sp = warp & 3, half = warp >> 2;
    const int m = m0 + sp * 32 + lane;
    const int cols = BN / 2, c0 = half * cols;
    for (int q = 0; q < cols; q += 8) {
      float v[8];
      g_ld8(tmem + (static_cast<uint32_t>(sp * 32) << 16) + static_cast<uint32_t>(c0 + q), v);
      if (m >= g.M) continue;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int n = n0 + c0 + q + j;
        if (n >= g.N) continue;
        const long long o = static_cast<long long>(m) * g.ldc + n;
        float z = v[j];
        if (g.bias) z += g.bias[n];
        if (g.epi == GEMM_GELU) {
          if (g.pre) g.pre[o] = z;
          z = gelu_f(z);
        } else if (g.epi == GEMM_GELU_GRAD) {
          z *= gelu_grad_f(g.pre[o]);
        }
        g.c[o] = z;
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(static_cast<uint32_t>(g.tmem_cols)));
}

// ------------------------------------------------------------------ fused terminator inference
// One launch per stage evaluates the closure for every row (tier-N ADO j,
// mode k): CTA t takes the rows of ADOs [t * apt, (t + 1) * apt) (apt = 128 / K
// ADOs, at most 128 rows), builds their input features (the unfused pack's
// formula) directly into shared memory as BF16 (the K-major core-matrix
// layout), runs the three layers on the tensor cores with the activations in
// shared memory and the accumulator in tensor memory (bias and GELU in the
// epilogue that writes the next layer's operand), and applies the gain head:
// P[(j K + k) n2 + e] = C_e rho_l[e] / sigma_k, C_e = y_e - i sg_e softplus(z_e).

// One layer: D (tensor memory, 128 x n) = A (shared memory, 128 rows, K = kdim,
// row-group stride sbo_a) x W^T (W: n rows of kdim BF16, row stride ldw), K in
// chunks of 64 through the two B stages.  Returns false if a wait ran out (the
// MMAs in flight are then drained, bounded).
__device__ bool mma_layer(uint32_t a_base, uint32_t sbo_a, const __nv_bfloat16* W, int n, int kdim, int ldw, int npad,
                          unsigned char* wb, uint64_t* mbar, uint32_t& parity, uint32_t tmem) {
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(npad >> 3) << 17) |
                         (static_cast<uint32_t>(kBM >> 4) << 24);
  const int nk = (kdim + kBK - 1) / kBK;
  const size_t wbytes = static_cast<size_t>(256) * kBK * 2;
  uint32_t issued = 0u;
  bool ok = true;
  GemmOperand wo{W, 1, ldw, 1};
  for (int c = 0; c < nk && ok; ++c) {
    const int b = c & 1;
    unsigned char* sb = wb + b * wbytes;
    if ((issued >> b) & 1u) {
      uint32_t done = 0;
      if (threadIdx.x == 0) done = g_wait(mbar + b, (parity >> b) & 1u);
      if (!__syncthreads_or(done)) {
        ok = false;
        break;
      }
      parity ^= 1u << b;
      issued &= ~(1u << b);
    }
    stage_operand(wo, 0, npad, n, c * kBK, kdim, sb);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    if (threadIdx.x == 0) {
      const uint32_t b0 = s_addr(sb);
#pragma unroll
      for (int s = 0; s < kBK / 16; ++s)
        g_mma(tmem, g_desc(a_base + c * (kBK / 8) * 128 + s * 256, 128, sbo_a),
              g_desc(b0 + s * 256, 128, (kBK / 8) * 128), idesc, (c > 0 || s > 0) ? 1 : 0);
      g_commit(mbar + b);
    }
    issued |= 1u << b;
  }
  for (int b = 0; b < 2; ++b) {
    if (!((issued >> b) & 1u)) continue;
    uint32_t done = 0;
    if (threadIdx.x == 0) done = g_wait(mbar + b, (parity >> b) & 1u);
    done = __syncthreads_or(done);
    parity ^= 1u << b;
    ok = ok && done;
  }
  fence_after();
  return ok;
}

// Epilogue of a hidden layer: row r = 32 (w % 4) + lane, columns of half w / 4;
// bias, GELU, BF16, written as the next layer's A operand (K = h, row-group
// stride (h / 8) * 128).
__device__ void hidden_epilogue(uint32_t tmem, const float* bias, int h, unsigned char* act) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sp = warp & 3, half = warp >> 2;
  const int r = sp * 32 + lane, cols = h / 2, c0 = half * cols;
  const int sbo = (h / 8) * 128;
  for (int q = 0; q < cols; q += 8) {
    float v[8];
    g_ld8(tmem + (static_cast<uint32_t>(sp * 32) << 16) + static_cast<uint32_t>(c0 + q), v);
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const __nv_bfloat162 hv = __floats2bfloat162_rn(gelu_f(v[2 * j] + bias[c0 + q + 2 * j]),
                                                      gelu_f(v[2 * j + 1] + bias[c0 + q + 2 * j + 1]));
      w[j] = *reinterpret_cast<const uint32_t*>(&hv);
    }
    const int kq = (c0 + q) >> 3;
    *reinterpret_cast<uint4*>(act + (r >> 3) * sbo + kq * 128 + (r & 7) * 16) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  fence_before();
  __syncthreads();
  fence_after();
}

template <typename TB>
__global__ void __launch_bounds__(kThreads, 1) k_term_mlp(const TermMlpArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TermModel& tm = A.tm;
  const int n = tm.n, n2 = n * n, K = tm.K, din = A.din, h = A.h, dout = A.dout;
  const int kpad1 = (din + kBK - 1) / kBK * kBK;
  unsigned char* act = smem_raw;                         // 128 x 256 BF16
  unsigned char* wb = smem_raw + 128 * 256 * 2;          // two 256 x 64 BF16 stages (later: the outputs)
  float* ys = reinterpret_cast<float*>(wb);              // 128 x dout FP32 (after the last layer)
  float* s_ado = reinterpret_cast<float*>(wb + 2 * 256 * kBK * 2);
  float2* rowf = reinterpret_cast<float2*>(s_ado + 128);  // per row: (n_k + 1) / (ngamma_l + gamma_kk)
  float2* isig = rowf + 128;                              // per mode: 1 / sigma_k (K <= 128)
  uint64_t* mbar = reinterpret_cast<uint64_t*>(isig + 128);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
  const int j0 = blockIdx.x * A.apt, na = min(A.apt, A.n_tier - j0), rows = na * K;
  const int cur = A.in.ctl ? A.in.ctl->cur : 0;
  const void* ysel = A.in.y_sel == 1 ? A.in.yb[cur] : (A.in.y_sel == 2 ? A.in.yb[1 - cur] : A.in.y_fixed);
  const TB* y = static_cast<const TB*>(ysel);
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tslot)),
                 "r"(256u));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(mbar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(mbar + 1)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  // the scale s of every ADO of the tile: sqrt(max_e |rho_l[e]|^2) (a warp per ADO)
  for (int j = threadIdx.x >> 5; j < na; j += kThreads / 32) {
    const TB* yl = y + static_cast<size_t>(A.first + j0 + j) * n2;
    float mx = 0.f;
    for (int e = threadIdx.x & 31; e < n2; e += 32) {
      const float re = static_cast<float>(yl[e].x), im = static_cast<float>(yl[e].y);
      mx = fmaxf(mx, re * re + im * im);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) s_ado[j] = sqrtf(mx) + 1e-30f;
  }
  for (int k = threadIdx.x; k < K; k += kThreads) {
    const double2 sk = tm.sigma[k];
    const double sd = sk.x * sk.x + sk.y * sk.y;
    isig[k] = make_float2(static_cast<float>(sk.x / sd), static_cast<float>(-sk.y / sd));
  }
  // the row factors, in FP64 once per row (the per-feature work below is FP32)
  for (int r = threadIdx.x; r < rows; r += kThreads) {
    const int j = r / K, k = r - j * K, l = A.first + j0 + j;
    const double2 gk = tm.gdiag[k], gl = tm.ngd[l];
    const double nk1 = static_cast<double>(tm.nidx[static_cast<size_t>(l) * K + k]) + 1.0;
    const double dr = gl.x + gk.x, di = gl.y + gk.y, dd = dr * dr + di * di;
    rowf[r] = dd > 0.0 ? make_float2(static_cast<float>(nk1 * dr / dd), static_cast<float>(-nk1 * di / dd))
                       : make_float2(0.f, 0.f);
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  // input features, 8 per thread and unit (16 bytes of the core-matrix layout)
  {
    const int nq = kpad1 / 8, sbo = nq * 128, units = 128 * nq;
    for (int u = threadIdx.x; u < units; u += kThreads) {
      const int r8 = u & 7, q = (u >> 3) % nq, g = (u >> 3) / nq, r = g * 8 + r8;
      float f8[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) f8[t] = 0.f;
      if (r < rows) {
        const int j = r / K, k = r - j * K, l = A.first + j0 + j;
        const TB* yl = y + static_cast<size_t>(l) * n2;
        const float inv = 1.0f / s_ado[j];
        const float2 fr = rowf[r];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int f = q * 8 + t;
          float v = 0.f;
          if (f < 2 * n2) {
            const int e = f < n2 ? f : f - n2;
            v = static_cast<float>(f < n2 ? yl[e].x : yl[e].y) * inv;
          } else if (f < 2 * n2 + K) {
            v = (f - 2 * n2 == k) ? 1.f : 0.f;
          } else if (f < din) {  // the adiabatic estimate (n_k + 1) c_ke rho_e / (ngamma_l + gamma_kk), in FP32
            const int g2 = f - 2 * n2 - K;
            const int e = g2 < n2 ? g2 : g2 - n2;
            const float2 c = __ldg(tm.cke + static_cast<size_t>(k) * n2 + e);
            const float2 cf = make_float2(c.x * fr.x - c.y * fr.y, c.x * fr.y + c.y * fr.x);
            const float yr = static_cast<float>(yl[e].x), yi = static_cast<float>(yl[e].y);
            v = (g2 < n2 ? cf.x * yr - cf.y * yi : cf.x * yi + cf.y * yr) * inv;
          }
          f8[t] = v;
        }
      }
      uint32_t w[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const __nv_bfloat162 hv = __floats2bfloat162_rn(f8[2 * t], f8[2 * t + 1]);
        w[t] = *reinterpret_cast<const uint32_t*>(&hv);
      }
      *reinterpret_cast<uint4*>(act + g * sbo + q * 128 + r8 * 16) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  fence_before();
  __syncthreads();
  fence_after();
  uint32_t parity = 0u;
  const int npad3 = (dout + 15) / 16 * 16;
  bool ok = mma_layer(s_addr(act), (kpad1 / 8) * 128, A.W1, h, din, din, h, wb, mbar, parity, tmem);
  if (ok) hidden_epilogue(tmem, A.b1, h, act);
  ok = ok && mma_layer(s_addr(act), (h / 8) * 128, A.W2, h, h, h, h, wb, mbar, parity, tmem);
  if (ok) hidden_epilogue(tmem, A.b2, h, act);
  ok = ok && mma_layer(s_addr(act), (h / 8) * 128, A.W3, dout, h, h, npad3, wb, mbar, parity, tmem);
  if (ok) {  // the outputs into shared memory (the B stages are free now)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sp = warp & 3, half = warp >> 2;
    const int r = sp * 32 + lane, cols = npad3 / 2;
    for (int q = half * cols; q < (half + 1) * cols; q += 8) {
      float v[8];
      g_ld8(tmem + (static_cast<uint32_t>(sp * 32) << 16) + static_cast<uint32_t>(q), v);
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (q + t < dout) ys[r * dout + q + t] = v[t] + A.b3[q + t];
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(256u));
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(A.err, 1);
    return;
  }
  // gain head: the prediction of rho_{n+1_k} for every (row, element)
  for (int i = threadIdx.x; i < rows * n2; i += kThreads) {
    const int r = i / n2, e = i - r * n2;
    const int j = r / K, k = r - j * K, l = A.first + j0 + j;
    const float sg = __ldg(tm.sgn + static_cast<size_t>(k) * n2 + e);  // sign(Re(v_a - v_b))
    float2 out = make_float2(0.f, 0.f);
    if (sg != 0.f) {
      const float* yr = ys + r * dout;
      const float cr = yr[e], zz = yr[n2 + e];
      const float ci = -sg * (fmaxf(zz, 0.f) + log1pf(expf(-fabsf(zz))));
      const TB rho = y[static_cast<size_t>(l) * n2 + e];
      const float rr = static_cast<float>(rho.x), ri = static_cast<float>(rho.y);
      const float pr = cr * rr - ci * ri, pi = cr * ri + ci * rr;  // C rho
      const float2 is = isig[k];  // 1 / sigma_k
      out = make_float2(pr * is.x - pi * is.y, pr * is.y + pi * is.x);
    }
    A.P[(static_cast<size_t>(j0 + j) * K + k) * n2 + e] = out;
  }
}

}  // namespace

bool term_fused_ok(int din, int h, int dout, int K) {
  return din <= 256 && h % kBK == 0 && h >= 64 && h <= 256 && dout <= 128 && K >= 1 && K <= 128;
}

size_t term_fused_smem() {
  return 128 * 256 * 2 + 2 * 256 * kBK * 2 + 128 * sizeof(float) + 2 * 128 * sizeof(float2) + 32;
}

cudaError_t launch_term_fused(const TermMlpArgs& a, bool y_float, cudaStream_t s) {
  if (a.n_tier <= 0) return cudaSuccess;
  const size_t smem = term_fused_smem();
  const int grid = (a.n_tier + a.apt - 1) / a.apt;
  const void* kern = y_float ? reinterpret_cast<const void*>(k_term_mlp<float2>)
                             : reinterpret_cast<const void*>(k_term_mlp<double2>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  if (y_float)
    k_term_mlp<float2><<<grid, kThreads, smem, s>>>(a);
  else
    k_term_mlp<double2><<<grid, kThreads, smem, s>>>(a);
  ++g_launches;
  return cudaGetLastError();
}

size_t gemm_smem(int bn) {
  return 2 * (static_cast<size_t>(kBM) * kBK * 2 + static_cast<size_t>(bn) * kBK * 2) + 32;
}

cudaError_t launch_gemm_bf16(GemmArgs g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  // N tile: the whole of N up to 256 columns (a multiple of 16), else 256-column tiles
  const int n16 = (g.N + 15) / 16 * 16;
  g.bn = n16 <= 256 ? n16 : 256;
  int cols = 32;
  while (cols < g.bn) cols *= 2;
  g.tmem_cols = cols;
  const size_t smem = gemm_smem(g.bn);
  cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  const dim3 grid((g.M + kBM - 1) / kBM, (g.N + g.bn - 1) / g.bn);
  k_gemm_bf16<<<grid, kThreads, smem, s>>>(g);
  ++g_launches;
  return cudaGetLastError();
}

}  // namespace heomgb
